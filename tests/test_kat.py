"""NIST KAT responses (the reference's PQCgenKAT_sign.cu format) against
per-count digests recorded from the reference's own generator
(tests/golden/kat_<set>.json, written by tests/golden/make_kat.py).

CPU: the oracle's API mirror produces the first counts.  GPU: the engine's
drop-in produces the whole .rsp, which must hash to the reference's file."""
import ctypes
import hashlib
import os

import pytest

from conftest import GOLDEN

KAT_SETS = [s for s in ("sha256-128f", "sha256-192f", "sha256-256f", "shake256-128f", "shake256-192f",
                        "shake256-256f", "sha256-128s", "shake256-128s", "sha256-192s", "sha256-256s",
                        "shake256-192s", "shake256-256s")
            if os.path.exists(os.path.join(GOLDEN, "kat_%s.json" % s))]


def _golden(setname):
    import json
    with open(os.path.join(GOLDEN, "kat_%s.json" % setname)) as f:
        return json.load(f)


def _digests(entry_pk, entry_sk, sm):
    return (hashlib.sha256(entry_pk).hexdigest(), hashlib.sha256(entry_sk).hexdigest(),
            hashlib.sha256(sm).hexdigest())


@pytest.mark.parametrize("setname", [s for s in KAT_SETS if s in ("sha256-128f", "shake256-128f")])
def test_oracle_kat_first_counts(setname):
    import spx_oracle
    g = _golden(setname)
    o = spx_oracle.Oracle(setname + "-simple")
    L = spx_oracle.lib()
    L.spxo_set_deterministic(1)
    L.spxo_randombytes_init(bytes(range(48)))
    reqs = []
    for i in range(4):
        seed = ctypes.create_string_buffer(48)
        L.spxo_randombytes(seed, 48)
        mlen = 33 * (i + 1)
        msg = ctypes.create_string_buffer(mlen)
        L.spxo_randombytes(msg, mlen)
        reqs.append((seed.raw, msg.raw))
    for i, (seed, msg) in enumerate(reqs):
        e = g["entries"][i]
        assert seed.hex().upper() == e["seed"]
        L.spxo_randombytes_init(seed)
        pk = ctypes.create_string_buffer(o.p.pk_bytes)
        sk = ctypes.create_string_buffer(o.p.sk_bytes)
        L.spxo_crypto_sign_keypair(ctypes.byref(o.p), pk, sk)
        sm = ctypes.create_string_buffer(o.p.sig_bytes + len(msg))
        smlen = ctypes.c_ulonglong()
        L.spxo_crypto_sign(ctypes.byref(o.p), sm, ctypes.byref(smlen), msg, len(msg), sk.raw)
        assert smlen.value == e["smlen"]
        assert _digests(pk.raw, sk.raw, sm.raw[:smlen.value]) == (e["pk_sha256"], e["sk_sha256"], e["sm_sha256"])


@pytest.mark.gpu
@pytest.mark.parametrize("setname", KAT_SETS)
def test_gpu_kat_file_matches_reference(setname):
    from cuspx_gb300 import kat
    g = _golden(setname)
    req, rsp, skb = kat.generate(setname + "-simple", count=len(g["entries"]))
    assert "PQCsignKAT_%d.rsp" % skb == g["rsp_name"]
    entries = []
    cur = None
    for line in rsp.splitlines():
        if line.startswith("count = "):
            cur = {"count": int(line.split("=")[1])}
            entries.append(cur)
        elif cur is not None and " = " in line:
            k, v = line.split(" = ", 1)
            cur[k] = v
    for e, want in zip(entries, g["entries"]):
        assert e["seed"] == want["seed"] and int(e["smlen"]) == want["smlen"]
        assert _digests(bytes.fromhex(e["pk"]), bytes.fromhex(e["sk"]), bytes.fromhex(e["sm"])) == \
            (want["pk_sha256"], want["sk_sha256"], want["sm_sha256"]), "count %d" % e["count"]
    assert hashlib.sha256(rsp.encode()).hexdigest() == g["rsp_sha256"]
