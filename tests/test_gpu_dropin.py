"""The NIST api.h drop-in (libspx_<set>.so) on the GPU, against the
reference's recorded behaviour (tests/golden) and the oracle: DRBG
consumption order, DEBUG_MODE keypairs, crypto_sign / crypto_sign_open
semantics (in-place, short sm, corruption) and the reference's batched
faces."""
import ctypes
import hashlib

import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

u8p = ctypes.c_char_p
ull = ctypes.c_ulonglong


def _lib(setname):
    import cuspx_gb300
    L = ctypes.CDLL(cuspx_gb300.dropin_path(setname + "-simple"))
    for f in ("crypto_sign_bytes", "crypto_sign_publickeybytes", "crypto_sign_secretkeybytes", "crypto_sign_seedbytes"):
        getattr(L, f).restype = ull
    L.crypto_sign_signature.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), u8p, ctypes.c_size_t, u8p]
    L.crypto_sign_verify.argtypes = [u8p, ctypes.c_size_t, u8p, ctypes.c_size_t, u8p]
    L.crypto_sign.argtypes = [ctypes.c_void_p, ctypes.POINTER(ull), ctypes.c_void_p, ull, u8p]
    L.crypto_sign_open.argtypes = [ctypes.c_void_p, ctypes.POINTER(ull), ctypes.c_void_p, ull, u8p]
    L.crypto_sign_keypair.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.crypto_sign_seed_keypair.argtypes = [ctypes.c_void_p, ctypes.c_void_p, u8p]
    L.randombytes_init.argtypes = [u8p, u8p, ctypes.c_int]
    L.randombytes.argtypes = [ctypes.c_void_p, ull]
    L.face_mhp_crypto_sign_scheme2.argtypes = [ctypes.c_void_p, ctypes.POINTER(ull), u8p, ull, u8p, ctypes.c_uint,
                                               ctypes.c_uint]
    L.face_mhp_crypto_sign_open.argtypes = [ctypes.c_void_p, ctypes.POINTER(ull), u8p, ull, u8p, ctypes.c_uint,
                                            ctypes.c_uint]
    L.face_mdp_crypto_sign_keypair.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint]
    return L


@pytest.mark.parametrize("setname", ["sha256-128f", "shake256-192f"])
def test_dropin_matches_reference_call_sequence(setname):
    """randombytes_init(0..47); randombytes(48); seed = randombytes(3n);
    seed keypair; DEBUG keypair (draws 3n); then sign the recorded messages
    (each call draws n bytes, which DEBUG_MODE replaces by 0xAD)."""
    g = load_golden(setname)
    L = _lib(setname)
    assert L.crypto_sign_bytes() == g["sig_bytes"]
    L.randombytes_init(bytes.fromhex(g["entropy"]), None, 256)
    first = ctypes.create_string_buffer(48)
    L.randombytes(first, 48)
    assert first.raw.hex() == g["drbg_first48"]
    seed = ctypes.create_string_buffer(g["seed_bytes"])
    L.randombytes(seed, g["seed_bytes"])
    assert seed.raw.hex() == g["seed"]
    pk = ctypes.create_string_buffer(g["pk_bytes"])
    sk = ctypes.create_string_buffer(g["sk_bytes"])
    assert L.crypto_sign_seed_keypair(pk, sk, seed.raw) == 0
    assert pk.raw.hex() == g["pk"] and sk.raw.hex() == g["sk"]
    assert L.crypto_sign_keypair(pk, sk) == 0
    assert pk.raw.hex() == g["debug_keypair"]["pk"] and sk.raw.hex() == g["debug_keypair"]["sk"]
    sk_b, pk_b = bytes.fromhex(g["sk"]), bytes.fromhex(g["pk"])
    sig = ctypes.create_string_buffer(g["sig_bytes"])
    sl = ctypes.c_size_t()
    for c in g["cases"][:6]:
        m = bytes.fromhex(c["msg"])
        assert L.crypto_sign_signature(sig, ctypes.byref(sl), m, len(m), sk_b) == 0
        assert sl.value == g["sig_bytes"]
        assert hashlib.sha256(sig.raw).hexdigest() == c["sig_sha256"]
        assert L.crypto_sign_verify(sig.raw, sl.value, m, len(m), pk_b) == 0
        assert L.crypto_sign_verify(sig.raw, sl.value - 1, m, len(m), pk_b) == -1


def test_sign_open_semantics():
    g = load_golden("sha256-128f")
    L = _lib("sha256-128f")
    sk, pk = bytes.fromhex(g["sk"]), bytes.fromhex(g["pk"])
    m = bytes.fromhex(g["sm"]["msg"])
    sigb = g["sig_bytes"]
    sm = ctypes.create_string_buffer(sigb + len(m))
    smlen = ull()
    assert L.crypto_sign(sm, ctypes.byref(smlen), m, len(m), sk) == 0
    assert smlen.value == sigb + len(m)
    assert hashlib.sha256(sm.raw).hexdigest() == g["sm"]["sm_sha256"]
    out = ctypes.create_string_buffer(smlen.value)
    mlen = ull()
    assert L.crypto_sign_open(out, ctypes.byref(mlen), sm.raw, smlen.value, pk) == 0
    assert out.raw[:mlen.value] == m
    # in-place open (test/spx.cu:149)
    inplace = ctypes.create_string_buffer(sm.raw, len(sm.raw))
    assert L.crypto_sign_open(inplace, ctypes.byref(mlen), inplace, smlen.value, pk) == 0
    assert inplace.raw[:mlen.value] == m
    # a flipped bit rejects, zero-fills m over smlen and sets mlen = 0
    bad = bytearray(sm.raw)
    bad[sigb // 2] ^= 0x20
    out = ctypes.create_string_buffer(b"\xff" * len(bad), len(bad))
    mlen = ull(123)
    assert L.crypto_sign_open(out, ctypes.byref(mlen), bytes(bad), len(bad), pk) == -1
    assert mlen.value == 0 and out.raw == bytes(len(bad))
    # sm shorter than a signature
    out = ctypes.create_string_buffer(b"\xff" * 10, 10)
    assert L.crypto_sign_open(out, ctypes.byref(mlen), sm.raw[:10], 10, pk) == -1
    assert mlen.value == 0 and out.raw == bytes(10)


def test_reference_batched_faces():
    """face_mhp_crypto_sign_scheme2 / face_mhp_crypto_sign_open with the
    reference's layouts (test/hp_spx.cu): num rows of sig || m_i."""
    import spx_oracle
    L = _lib("sha256-128f")
    o = spx_oracle.Oracle("sha256-128f-simple")
    num, mlen, sigb = 8, 32, o.p.sig_bytes
    pk = ctypes.create_string_buffer(num * 32)
    sk = ctypes.create_string_buffer(num * 64)
    assert L.face_mdp_crypto_sign_keypair(pk, sk, num) == 0
    # DEBUG_MODE: every keypair comes from seed 0..47
    assert all(sk.raw[i * 64:(i + 1) * 64] == sk.raw[:64] for i in range(num))
    m = bytes(range(256))[:num * mlen]
    sm = ctypes.create_string_buffer(num * (sigb + mlen))
    smlen = ull()
    assert L.face_mhp_crypto_sign_scheme2(sm, ctypes.byref(smlen), m, mlen, sk.raw, num, 8) == 0
    assert smlen.value == sigb + mlen
    for i in range(num):
        row = sm.raw[i * smlen.value:(i + 1) * smlen.value]
        assert row[:sigb] == o.sign(m[i * mlen:(i + 1) * mlen], sk.raw[i * 64:(i + 1) * 64])
        assert row[sigb:] == m[i * mlen:(i + 1) * mlen]
    out = ctypes.create_string_buffer(num * mlen)
    ml = ull()
    assert L.face_mhp_crypto_sign_open(out, ctypes.byref(ml), sm.raw, smlen.value, pk.raw, num, 8) == 0
    assert ml.value == mlen and out.raw == m
    bad = bytearray(sm.raw)
    bad[3 * smlen.value + 100] ^= 1
    assert L.face_mhp_crypto_sign_open(out, ctypes.byref(ml), bytes(bad), smlen.value, pk.raw, num, 8) == -1
    assert out.raw[3 * mlen:4 * mlen] == bytes(mlen) and out.raw[:3 * mlen] == m[:3 * mlen]


@pytest.mark.parametrize("setname", ["sha256-128f", "shake256-256f", "sha256-192f"])
def test_dropin_release_mode_matches_reference(setname):
    """With deterministic mode off the drop-in behaves like the reference
    built without DEBUG_MODE (oracle/build_ref.sh --release): the keypair
    seed (3n bytes) and each optrand (n bytes) come from the DRBG in call
    order (sign.cu:344-349, :1950-1954).  Keypairs, signatures, crypto_sign /
    crypto_sign_open and the DRBG bytes left afterwards equal the reference's
    recorded run."""
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, setname + "_release.json")) as f:
        g = json.load(f)
    L = _lib(setname)
    L.cuspx_set_deterministic.argtypes = [ctypes.c_int]
    m0, m1, m2 = (bytes.fromhex(x) for x in g["msgs"])
    pkb, skb, sigb = L.crypto_sign_publickeybytes(), L.crypto_sign_secretkeybytes(), L.crypto_sign_bytes()
    L.cuspx_set_deterministic(0)
    try:
        L.randombytes_init(bytes.fromhex(g["entropy"]), None, 256)
        pk1, sk1 = ctypes.create_string_buffer(pkb), ctypes.create_string_buffer(skb)
        assert L.crypto_sign_keypair(pk1, sk1) == 0
        assert (pk1.raw.hex(), sk1.raw.hex()) == (g["kp1"]["pk"], g["kp1"]["sk"])
        sig = ctypes.create_string_buffer(sigb)
        sl = ctypes.c_size_t()
        assert L.crypto_sign_signature(sig, ctypes.byref(sl), m0, len(m0), sk1.raw) == 0
        assert hashlib.sha256(sig.raw).hexdigest() == g["sig0"]["sha256"]
        sm = ctypes.create_string_buffer(sigb + len(m1))
        smlen = ull()
        assert L.crypto_sign(sm, ctypes.byref(smlen), m1, len(m1), sk1.raw) == 0
        assert hashlib.sha256(sm.raw[:smlen.value]).hexdigest() == g["sm1"]["sha256"]
        out = ctypes.create_string_buffer(smlen.value)
        mlen = ull()
        rc = L.crypto_sign_open(out, ctypes.byref(mlen), sm.raw, smlen.value, pk1.raw)
        assert (rc, mlen.value) == (g["sm1"]["open_rc"], g["sm1"]["open_mlen"])
        assert out.raw[:mlen.value].hex() == g["sm1"]["open_msg"]
        assert L.crypto_sign_verify(sig.raw, sigb, m0, len(m0), pk1.raw) == g["sig0"]["verify"]
        pk2, sk2 = ctypes.create_string_buffer(pkb), ctypes.create_string_buffer(skb)
        assert L.crypto_sign_keypair(pk2, sk2) == 0
        assert (pk2.raw.hex(), sk2.raw.hex()) == (g["kp2"]["pk"], g["kp2"]["sk"])
        assert L.crypto_sign_signature(sig, ctypes.byref(sl), m2, len(m2), sk2.raw) == 0
        assert hashlib.sha256(sig.raw).hexdigest() == g["sig2"]["sha256"]
        tail = ctypes.create_string_buffer(16)
        L.randombytes(tail, 16)
        assert tail.raw.hex() == g["drbg_tail16"]
    finally:
        L.cuspx_set_deterministic(1)


def test_dropin_concurrent_threads_share_launches():
    """Eight threads call crypto_sign_signature and crypto_sign_verify of one
    drop-in at once (the reference's CPU API is not thread-safe at all:
    sha256.cu:385 keeps a global hash state).  Concurrent calls are combined
    into shared launches; every signature equals the oracle's and every
    verdict is right, corrupted signatures included."""
    import threading
    import spx_oracle
    L = _lib("sha256-128f")
    o = spx_oracle.Oracle("sha256-128f-simple")
    sigb = L.crypto_sign_bytes()
    pk = ctypes.create_string_buffer(32)
    sk = ctypes.create_string_buffer(64)
    assert L.crypto_sign_seed_keypair(pk, sk, bytes(range(100, 148))) == 0
    pk_b, sk_b = pk.raw, sk.raw
    nthreads, per = 8, 6
    msgs = [[hashlib.sha256(b"%d/%d" % (t, i)).digest() * (1 + (t + i) % 5) for i in range(per)]
            for t in range(nthreads)]
    results = [[None] * per for _ in range(nthreads)]
    verdicts = [[None] * per for _ in range(nthreads)]
    errors = []
    start = threading.Barrier(nthreads)

    def worker(t):
        try:
            start.wait()
            sig = ctypes.create_string_buffer(sigb)
            sl = ctypes.c_size_t()
            for i, m in enumerate(msgs[t]):
                assert L.crypto_sign_signature(sig, ctypes.byref(sl), m, len(m), sk_b) == 0
                results[t][i] = sig.raw
                bad = bytearray(sig.raw)
                bad[(t * 977 + i * 131) % sigb] ^= 0x20
                verdicts[t][i] = (L.crypto_sign_verify(sig.raw, sigb, m, len(m), pk_b),
                                  L.crypto_sign_verify(bytes(bad), sigb, m, len(m), pk_b))
        except Exception as e:   # reported below
            errors.append(repr(e))

    ths = [threading.Thread(target=worker, args=(t,)) for t in range(nthreads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    assert not errors, errors
    for t in range(nthreads):
        for i, m in enumerate(msgs[t]):
            assert results[t][i] == o.sign(m, sk_b), (t, i)
            assert verdicts[t][i] == (0, -1), (t, i)
