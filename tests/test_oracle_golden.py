"""The oracle (C restatement, oracle/spx_oracle.c) against the reference's own
outputs recorded in tests/golden -- CPU only.  This is what pins the oracle
before the GPU tests trust it."""
import hashlib
import os

import pytest

from conftest import GOLDEN, load_golden

SETS = ["sha256-128f", "sha256-128s", "sha256-192f", "sha256-192s", "sha256-256f", "sha256-256s",
        "shake256-128f", "shake256-128s", "shake256-192f", "shake256-192s", "shake256-256f", "shake256-256s"]


@pytest.fixture(scope="module")
def so():
    import spx_oracle
    return spx_oracle


@pytest.mark.parametrize("setname", SETS)
def test_sizes_and_keypairs(so, setname):
    g = load_golden(setname)
    o = so.Oracle(setname)
    assert (o.p.n, o.p.pk_bytes, o.p.sk_bytes, o.p.sig_bytes, o.p.seed_bytes) == \
        (g["n"], g["pk_bytes"], g["sk_bytes"], g["sig_bytes"], g["seed_bytes"])
    pk, sk = o.seed_keypair(bytes.fromhex(g["seed"]))
    assert pk.hex() == g["pk"] and sk.hex() == g["sk"]
    pk, sk = o.seed_keypair(bytes(range(g["seed_bytes"])))
    assert pk.hex() == g["debug_keypair"]["pk"] and sk.hex() == g["debug_keypair"]["sk"]


@pytest.mark.parametrize("setname", SETS)
def test_signatures_and_verdicts(so, setname):
    g = load_golden(setname)
    o = so.Oracle(setname)
    sk, pk = bytes.fromhex(g["sk"]), bytes.fromhex(g["pk"])
    cases = g["cases"] if setname.endswith("f") else g["cases"][:2]
    for c in cases:
        m = bytes.fromhex(c["msg"])
        sig = o.sign(m, sk)
        assert hashlib.sha256(sig).hexdigest() == c["sig_sha256"], "mlen=%d" % c["mlen"]
        if "sig_file" in c:
            with open(os.path.join(GOLDEN, c["sig_file"]), "rb") as f:
                assert sig == f.read()
        assert o.verify(sig, m, pk) == c["verify"]
        for fl in c["corrupt"]:
            bad = bytearray(sig)
            bad[fl["pos"]] ^= fl["xor"]
            assert o.verify(bytes(bad), m, pk) == fl["verify"]
        if "msgflip_verify" in c:
            bm = bytearray(m)
            bm[len(m) // 2] ^= 0x10
            assert o.verify(sig, bytes(bm), pk) == c["msgflip_verify"]
        assert o.verify(sig[:-1], m, pk) == c["shortsig_verify"]


def test_drbg_matches_reference_stream(so):
    for setname in ("sha256-128f", "shake256-256f"):
        g = load_golden(setname)
        d = so.Drbg(bytes.fromhex(g["entropy"]))
        assert d.bytes(48).hex() == g["drbg_first48"]
        assert d.bytes(g["seed_bytes"]).hex() == g["seed"]


def test_aes256_fips197_vector(so):
    # FIPS 197 Appendix C.3 (AES-256)
    key = bytes(range(32))
    pt = bytes.fromhex("00112233445566778899aabbccddeeff")
    assert so.aes256_ecb(key, pt).hex() == "8ea2b7ca516745bfeafc49904b496089"


def test_hash_primitives_against_hashlib(so):
    import hashlib as hl
    import random
    rng = random.Random(5)
    for L in (0, 1, 55, 56, 63, 64, 65, 119, 120, 135, 136, 137, 1000):
        m = bytes(rng.randrange(256) for _ in range(L))
        assert so.sha256(m) == hl.sha256(m).digest()
        assert so.shake256(m, 200) == hl.shake_256(m).digest(200)


@pytest.mark.parametrize("setname", ["sha256-128f", "shake256-192f"])
def test_crypto_sign_open_semantics(so, setname):
    """crypto_sign / crypto_sign_open through the DRBG mirror (sign.cu:3302, :6058)."""
    import ctypes
    g = load_golden(setname)
    o = so.Oracle(setname)
    L = so.lib()
    L.spxo_randombytes_init(bytes.fromhex(g["entropy"]))
    L.spxo_set_deterministic(1)
    sk, pk = bytes.fromhex(g["sk"]), bytes.fromhex(g["pk"])
    m = bytes.fromhex(g["sm"]["msg"])
    sm = ctypes.create_string_buffer(o.p.sig_bytes + len(m))
    smlen = ctypes.c_ulonglong()
    L.spxo_crypto_sign(ctypes.byref(o.p), sm, ctypes.byref(smlen), m, len(m), sk)
    assert hashlib.sha256(sm.raw[:smlen.value]).hexdigest() == g["sm"]["sm_sha256"]
    out = ctypes.create_string_buffer(smlen.value)
    mlen = ctypes.c_ulonglong()
    rc = L.spxo_crypto_sign_open(ctypes.byref(o.p), out, ctypes.byref(mlen), sm.raw[:smlen.value], smlen.value, pk)
    assert (rc, mlen.value) == (g["sm"]["open_rc"], g["sm"]["open_mlen"])
    assert out.raw[:mlen.value].hex() == g["sm"]["open_msg"]
    short = sm.raw[:o.p.sig_bytes - 1]
    rc = L.spxo_crypto_sign_open(ctypes.byref(o.p), out, ctypes.byref(mlen), short, len(short), pk)
    assert (rc, mlen.value) == (g["sm_short"]["open_rc"], g["sm_short"]["open_mlen"])


def test_robust_differs_from_simple(so):
    """Robust sets (not in the reference; parity unpinned) must at least be a
    different function of the same inputs and round-trip."""
    s, r = so.Oracle("sha256-128f-simple"), so.Oracle("sha256-128f-robust")
    seed = bytes(range(48))
    pks, sks = s.seed_keypair(seed)
    pkr, skr = r.seed_keypair(seed)
    assert pks[:16] == pkr[:16] and pks[16:] != pkr[16:]
    sig = r.sign(b"robust", skr)
    assert r.verify(sig, b"robust", pkr) == 0
    assert s.verify(sig, b"robust", pks) == -1


@pytest.mark.parametrize("setname", ["sha256-128f", "shake256-256f", "sha256-192f"])
def test_release_mode_call_sequence(so, setname):
    """With DEBUG_MODE off (the reference built by oracle/build_ref.sh
    --release) the keypair seed and each optrand come from the DRBG
    (sign.cu:344-349, :1950-1954).  The oracle, switched to that mode,
    reproduces the reference's keypairs, signatures, crypto_sign / open and
    the DRBG bytes left after the whole call sequence."""
    import ctypes
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, setname + "_release.json")) as f:
        g = json.load(f)
    o = so.Oracle(setname)
    L = so.lib()
    p = ctypes.byref(o.p)
    m0, m1, m2 = (bytes.fromhex(x) for x in g["msgs"])
    L.spxo_set_deterministic(0)
    try:
        L.spxo_randombytes_init(bytes.fromhex(g["entropy"]))
        pk1 = ctypes.create_string_buffer(o.p.pk_bytes)
        sk1 = ctypes.create_string_buffer(o.p.sk_bytes)
        L.spxo_crypto_sign_keypair(p, pk1, sk1)
        assert (pk1.raw.hex(), sk1.raw.hex()) == (g["kp1"]["pk"], g["kp1"]["sk"])
        sig = ctypes.create_string_buffer(o.p.sig_bytes)
        siglen = ctypes.c_size_t()
        L.spxo_crypto_sign_signature(p, sig, ctypes.byref(siglen), m0, len(m0), sk1.raw)
        assert hashlib.sha256(sig.raw).hexdigest() == g["sig0"]["sha256"]
        assert o.verify(sig.raw, m0, pk1.raw) == g["sig0"]["verify"] == 0
        sm = ctypes.create_string_buffer(o.p.sig_bytes + len(m1))
        smlen = ctypes.c_ulonglong()
        L.spxo_crypto_sign(p, sm, ctypes.byref(smlen), m1, len(m1), sk1.raw)
        assert hashlib.sha256(sm.raw[:smlen.value]).hexdigest() == g["sm1"]["sha256"]
        out = ctypes.create_string_buffer(smlen.value)
        mlen = ctypes.c_ulonglong()
        rc = L.spxo_crypto_sign_open(p, out, ctypes.byref(mlen), sm.raw[:smlen.value], smlen.value, pk1.raw)
        assert (rc, mlen.value) == (g["sm1"]["open_rc"], g["sm1"]["open_mlen"])
        assert out.raw[:mlen.value].hex() == g["sm1"]["open_msg"]
        pk2 = ctypes.create_string_buffer(o.p.pk_bytes)
        sk2 = ctypes.create_string_buffer(o.p.sk_bytes)
        L.spxo_crypto_sign_keypair(p, pk2, sk2)
        assert (pk2.raw.hex(), sk2.raw.hex()) == (g["kp2"]["pk"], g["kp2"]["sk"])
        L.spxo_crypto_sign_signature(p, sig, ctypes.byref(siglen), m2, len(m2), sk2.raw)
        assert hashlib.sha256(sig.raw).hexdigest() == g["sig2"]["sha256"]
        tail = ctypes.create_string_buffer(16)
        L.spxo_randombytes(tail, 16)
        assert tail.raw.hex() == g["drbg_tail16"]
    finally:
        L.spxo_set_deterministic(1)
