"""Generate tests/golden/*.json from the reference's own CPU implementation.

The reference (CUDA C++ sources) is compiled per parameter set by
oracle/build_ref.sh into oracle/_ref/<set>/ref_golden, a line-oriented driver
over the reference api.h / rng.h entry points.  This script feeds it seeded
inputs and records what the reference produced:

* the NIST DRBG stream for entropy 0..47 (randombytes_init/randombytes);
* crypto_sign_seed_keypair on a DRBG-drawn seed, and crypto_sign_keypair
  (whose seed the shipped DEBUG_MODE forces to 0..3n-1);
* crypto_sign_signature on DRBG-drawn messages whose lengths straddle every
  SHA-256 / SHAKE-256 padding boundary of PRF_msg and H_msg, stored as
  SHA-256 digests (plus the full signature bytes for two 128f sets);
* crypto_sign_verify verdicts for the good signatures, for one-byte
  corruptions at seeded positions and for one flipped message bit;
* crypto_sign / crypto_sign_open, including a short sm.

Run from the repository root (needs the reference tree and nvcc):
    python tests/golden/make_golden.py [set ...]

With --release it writes tests/golden/<set>_release.json instead, from the
reference built without DEBUG_MODE (oracle/build_ref.sh --release): the
keypair seed and every optrand then come from the DRBG, so the record pins
the DRBG consumption of crypto_sign_keypair (3n bytes), crypto_sign_signature
and crypto_sign (n bytes each) in call order:
    python tests/golden/make_golden.py --release [set ...]
"""
import hashlib
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.dirname(os.path.abspath(__file__))

SETS = ["sha256-128f", "sha256-128s", "sha256-192f", "sha256-192s", "sha256-256f", "sha256-256s",
        "shake256-128f", "shake256-128s", "shake256-192f", "shake256-192s", "shake256-256f", "shake256-256s"]
FULL_SIG_SETS = {"sha256-128f", "shake256-128f"}


def lengths_for(setname, n):
    if setname.endswith("s"):
        return [0, 33, 200]
    # PRF_msg absorbs optrand(n)||m after one key block; H_msg absorbs
    # R(n)||PK(2n)||m.  Straddle the 55/56 (SHA-256) and 135/136 (SHAKE)
    # padding edges of both, plus empty and multi-block messages.
    if setname.startswith("sha256"):
        edges = [55 - n, 56 - n, 63 - n, 64 - n, 119 - n, 120 - n, 55 - 3 * n + 64, 56 - 3 * n + 64,
                 64 - 3 * n, 65 - 3 * n]
    else:
        edges = [135 - 2 * n, 136 - 2 * n, 135 - 3 * n, 136 - 3 * n, 271 - 3 * n, 272 - 3 * n]
    base = [0, 1, 32, 33, 64, 1000, 4096]
    return sorted(set(x for x in base + edges if x >= 0))


RELEASE_SETS = ["sha256-128f", "shake256-256f", "sha256-192f"]


def release_messages():
    """Three fixed messages (0, 33 and 1000 bytes) that do not touch the DRBG."""
    return [b"", hashlib.shake_256(b"release m1").digest(33), hashlib.shake_256(b"release m2").digest(1000)]


RELEASE_ENTROPY = bytes((7 * i + 3) & 0xFF for i in range(48))


class Ref:
    def __init__(self, setname, release=False):
        sub = setname + ("-release" if release else "")
        exe = os.path.join(ROOT, "oracle", "_ref", sub, "ref_golden")
        if not os.path.exists(exe):
            cmd = [os.path.join(ROOT, "oracle", "build_ref.sh")] + (["--release"] if release else []) + [setname]
            subprocess.run(cmd, check=True)
        self.p = subprocess.Popen([exe], stdin=subprocess.PIPE, stdout=subprocess.PIPE, text=True)

    def __call__(self, line):
        self.p.stdin.write(line + "\n")
        self.p.stdin.flush()
        return self.p.stdout.readline().strip()

    def close(self):
        self.p.stdin.close()
        self.p.wait()


def hx(b):
    return b.hex() if b else "-"


def gen(setname):
    ref = Ref(setname)
    n, pkb, skb, sigb, seedb = map(int, ref("info").split())
    ent = bytes(range(48))
    ref("drbg_init " + ent.hex())
    rec = {"set": setname + "-simple", "n": n, "pk_bytes": pkb, "sk_bytes": skb, "sig_bytes": sigb,
           "seed_bytes": seedb, "entropy": ent.hex()}
    rec["drbg_first48"] = ref("drbg 48")
    seed = bytes.fromhex(ref("drbg %d" % seedb))
    pk, sk = ref("seedkp " + seed.hex()).split()
    rec["seed"], rec["pk"], rec["sk"] = seed.hex(), pk, sk
    kpk, ksk = ref("kp").split()
    rec["debug_keypair"] = {"pk": kpk, "sk": ksk}
    msgs = []
    for L in lengths_for(setname, n):
        m = bytes.fromhex(ref("drbg %d" % L)) if L else b""
        msgs.append(m)
    cases = []
    for i, m in enumerate(msgs):
        sig = bytes.fromhex(ref("sign %s %s" % (sk, hx(m))))
        assert len(sig) == sigb
        case = {"mlen": len(m), "msg": m.hex(), "sig_sha256": hashlib.sha256(sig).hexdigest(),
                "sig_head": sig[:64].hex(), "verify": int(ref("verify %s %s %s" % (pk, sig.hex(), hx(m))))}
        if setname in FULL_SIG_SETS and i < 2:
            fn = "%s_sig%d.bin" % (setname, i)
            with open(os.path.join(OUT, fn), "wb") as f:
                f.write(sig)
            case["sig_file"] = fn
        # one-byte corruptions at seeded positions spread over R, FORS and the hypertree
        flips = []
        for j, pos in enumerate([0, n + 5, sigb // 3, sigb // 2 + 7, sigb - 1]):
            bad = bytearray(sig)
            bad[pos] ^= (0x01 << (j % 8))
            flips.append({"pos": pos, "xor": 0x01 << (j % 8),
                          "verify": int(ref("verify %s %s %s" % (pk, bad.hex(), hx(m))))})
        case["corrupt"] = flips
        if m:
            bm = bytearray(m)
            bm[len(m) // 2] ^= 0x10
            case["msgflip_verify"] = int(ref("verify %s %s %s" % (pk, sig.hex(), bytes(bm).hex())))
        case["shortsig_verify"] = int(ref("verify %s %s %s" % (pk, sig[:-1].hex(), hx(m))))
        cases.append(case)
    rec["cases"] = cases
    # crypto_sign / crypto_sign_open round trip and a short sm
    m = msgs[1] if len(msgs) > 1 else b"\x01"
    sm = bytes.fromhex(ref("smsign %s %s" % (sk, hx(m))))
    rc, mlen, mo = ref("open %s %s" % (pk, sm.hex())).split()
    rec["sm"] = {"msg": m.hex(), "sm_sha256": hashlib.sha256(sm).hexdigest(), "open_rc": int(rc),
                 "open_mlen": int(mlen), "open_msg": mo if mo != "-" else ""}
    rc, mlen, _ = ref("open %s %s" % (pk, sm[:sigb - 1].hex())).split()
    rec["sm_short"] = {"open_rc": int(rc), "open_mlen": int(mlen)}
    ref.close()
    with open(os.path.join(OUT, setname + ".json"), "w") as f:
        json.dump(rec, f, indent=1)
    print(setname, len(cases), "cases")


def gen_release(setname):
    """The reference's release call sequence: keypair, sign, crypto_sign,
    open, verify, a second keypair and sign, then 16 more DRBG bytes."""
    ref = Ref(setname, release=True)
    n, pkb, skb, sigb, seedb = map(int, ref("info").split())
    m0, m1, m2 = release_messages()
    ref("drbg_init " + RELEASE_ENTROPY.hex())
    rec = {"set": setname + "-simple", "n": n, "sig_bytes": sigb, "entropy": RELEASE_ENTROPY.hex(),
           "msgs": [m0.hex(), m1.hex(), m2.hex()]}
    pk1, sk1 = ref("kp").split()
    sig0 = bytes.fromhex(ref("sign %s %s" % (sk1, hx(m0))))
    sm1 = bytes.fromhex(ref("smsign %s %s" % (sk1, hx(m1))))
    rc, mlen, mo = ref("open %s %s" % (pk1, sm1.hex())).split()
    v0 = int(ref("verify %s %s %s" % (pk1, sig0.hex(), hx(m0))))
    pk2, sk2 = ref("kp").split()
    sig2 = bytes.fromhex(ref("sign %s %s" % (sk2, hx(m2))))
    tail = ref("drbg 16")
    rec.update({
        "kp1": {"pk": pk1, "sk": sk1},
        "sig0": {"sha256": hashlib.sha256(sig0).hexdigest(), "head": sig0[:64].hex(), "verify": v0},
        "sm1": {"sha256": hashlib.sha256(sm1).hexdigest(), "open_rc": int(rc), "open_mlen": int(mlen),
                "open_msg": mo if mo != "-" else ""},
        "kp2": {"pk": pk2, "sk": sk2},
        "sig2": {"sha256": hashlib.sha256(sig2).hexdigest(), "head": sig2[:64].hex()},
        "drbg_tail16": tail,
    })
    ref.close()
    with open(os.path.join(OUT, setname + "_release.json"), "w") as f:
        json.dump(rec, f, indent=1)
    print(setname, "release")


if __name__ == "__main__":
    args = sys.argv[1:]
    if args and args[0] == "--release":
        for s in (args[1:] or RELEASE_SETS):
            gen_release(s)
    else:
        for s in (args or SETS):
            gen(s)
