"""NIST known-answer files in the reference's format, produced on the GPU.

Writes the request/response pair that the reference's PQCgenKAT_sign.cu
writes (PQCsignKAT_<sk bytes>.req / .rsp): the DRBG seeded with entropy
0..47 draws, for each of `count` entries, a 48-byte seed and a message of
33*(i+1) bytes; for each entry the DRBG is reseeded with its seed and
crypto_sign_keypair, crypto_sign and crypto_sign_open run -- here through
the GPU drop-in library of the parameter set.  Byte strings are upper-case
hex, an empty one is written as "00".

    python -m cuspx_gb300.kat sha256-128f-simple [count] [outdir]
"""
import ctypes
import os
import sys

from . import dropin_path


def _hex(b):
    return b.hex().upper() if b else "00"


class _Dropin:
    def __init__(self, set_name):
        L = ctypes.CDLL(dropin_path(set_name))
        for f in ("crypto_sign_bytes", "crypto_sign_publickeybytes", "crypto_sign_secretkeybytes"):
            getattr(L, f).restype = ctypes.c_ulonglong
        L.randombytes_init.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        L.randombytes.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong]
        L.crypto_sign_keypair.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.crypto_sign.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_char_p,
                                  ctypes.c_ulonglong, ctypes.c_char_p]
        L.crypto_sign_open.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_char_p,
                                       ctypes.c_ulonglong, ctypes.c_char_p]
        self.L = L
        self.sig = L.crypto_sign_bytes()
        self.pk = L.crypto_sign_publickeybytes()
        self.sk = L.crypto_sign_secretkeybytes()

    def randombytes(self, n):
        b = ctypes.create_string_buffer(max(n, 1))
        self.L.randombytes(b, n)
        return b.raw[:n]


def generate(set_name, count=100):
    """Returns (req_text, rsp_text, sk_bytes)."""
    d = _Dropin(set_name)
    L = d.L
    L.randombytes_init(bytes(range(48)), None, 256)
    entries = []
    req = []
    for i in range(count):
        seed = d.randombytes(48)
        mlen = 33 * (i + 1)
        msg = d.randombytes(mlen)
        entries.append((i, seed, mlen, msg))
        req += ["count = %d" % i, "seed = " + _hex(seed), "mlen = %d" % mlen, "msg = " + _hex(msg),
                "pk =", "sk =", "smlen =", "sm =", ""]
    rsp = ["# SPHINCS+", ""]
    for i, seed, mlen, msg in entries:
        L.randombytes_init(seed, None, 256)
        pk = ctypes.create_string_buffer(d.pk)
        sk = ctypes.create_string_buffer(d.sk)
        if L.crypto_sign_keypair(pk, sk) != 0:
            raise RuntimeError("crypto_sign_keypair failed at count %d" % i)
        sm = ctypes.create_string_buffer(d.sig + mlen)
        smlen = ctypes.c_ulonglong()
        if L.crypto_sign(sm, ctypes.byref(smlen), msg, mlen, sk.raw) != 0:
            raise RuntimeError("crypto_sign failed at count %d" % i)
        m1 = ctypes.create_string_buffer(d.sig + mlen)
        mlen1 = ctypes.c_ulonglong()
        if L.crypto_sign_open(m1, ctypes.byref(mlen1), sm.raw[:smlen.value], smlen.value, pk.raw) != 0:
            raise RuntimeError("crypto_sign_open failed at count %d" % i)
        if mlen1.value != mlen or m1.raw[:mlen] != msg:
            raise RuntimeError("crypto_sign_open returned a different message at count %d" % i)
        rsp += ["count = %d" % i, "seed = " + _hex(seed), "mlen = %d" % mlen, "msg = " + _hex(msg),
                "pk = " + _hex(pk.raw), "sk = " + _hex(sk.raw), "smlen = %d" % smlen.value,
                "sm = " + _hex(sm.raw[:smlen.value]), ""]
    return "\n".join(req) + "\n", "\n".join(rsp) + "\n", d.sk


def write(set_name, outdir, count=100):
    req, rsp, skb = generate(set_name, count)
    os.makedirs(outdir, exist_ok=True)
    base = os.path.join(outdir, "PQCsignKAT_%d" % skb)
    with open(base + ".req", "w") as f:
        f.write(req)
    with open(base + ".rsp", "w") as f:
        f.write(rsp)
    return base + ".rsp"


if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "sha256-128f-simple"
    cnt = int(sys.argv[2]) if len(sys.argv) > 2 else 100
    out = sys.argv[3] if len(sys.argv) > 3 else "."
    print(write(name, out, cnt))
