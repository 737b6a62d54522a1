"""Pin NIST KAT responses from the reference's own generator.

oracle/build_ref.sh compiles the reference's PQCgenKAT_sign.cu (100 counts,
mlen = 33*(i+1), DRBG reseeded per count, crypto_sign_keypair ->
crypto_sign -> crypto_sign_open) per parameter set; this script runs it in
oracle/_ref/<set>/ and records, per count, SHA-256 digests of pk, sk and sm
plus smlen, and the digest of the whole .rsp file, in tests/golden/kat_<set>.json
(the .rsp files themselves are megabytes).

    python tests/golden/make_kat.py [set ...]
"""
import hashlib
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.dirname(os.path.abspath(__file__))
SETS = ["sha256-128f", "sha256-192f", "sha256-256f", "shake256-128f", "shake256-192f", "shake256-256f",
        "sha256-128s", "shake256-128s", "sha256-192s", "sha256-256s", "shake256-192s", "shake256-256s"]


def parse_rsp(text):
    entries, cur = [], None
    for line in text.splitlines():
        if line.startswith("count = "):
            cur = {"count": int(line.split("=")[1])}
            entries.append(cur)
        elif cur is not None and " = " in line:
            k, v = line.split(" = ", 1)
            cur[k.strip()] = v.strip()
    return entries


def digest_entries(entries):
    out = []
    for e in entries:
        out.append({"count": e["count"], "mlen": int(e["mlen"]), "smlen": int(e["smlen"]),
                    "pk_sha256": hashlib.sha256(bytes.fromhex(e["pk"])).hexdigest(),
                    "sk_sha256": hashlib.sha256(bytes.fromhex(e["sk"])).hexdigest(),
                    "sm_sha256": hashlib.sha256(bytes.fromhex(e["sm"])).hexdigest(),
                    "seed": e["seed"]})
    return out


def gen(setname):
    d = os.path.join(ROOT, "oracle", "_ref", setname)
    exe = os.path.join(d, "PQCgenKAT_sign")
    if not os.path.exists(exe):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), setname], check=True)
    subprocess.run([exe], cwd=d, check=True, stdout=subprocess.DEVNULL)
    rsp = [f for f in os.listdir(d) if f.endswith(".rsp")][0]
    text = open(os.path.join(d, rsp)).read()
    rec = {"set": setname + "-simple", "rsp_name": rsp, "rsp_sha256": hashlib.sha256(text.encode()).hexdigest(),
           "entries": digest_entries(parse_rsp(text))}
    with open(os.path.join(OUT, "kat_%s.json" % setname), "w") as f:
        json.dump(rec, f, indent=0)
    print(setname, len(rec["entries"]), rec["rsp_sha256"][:16])


if __name__ == "__main__":
    for s in (sys.argv[1:] or SETS):
        gen(s)
