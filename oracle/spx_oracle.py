"""ctypes face of the C restatement in spx_oracle.c (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs
import this module; the product package never does.
"""
import ctypes
import os
import platform
import subprocess

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libspx_oracle.%s.so" % platform.machine())


class Params(ctypes.Structure):
    _fields_ = [(f, ctypes.c_int) for f in (
        "hash", "robust", "n", "h", "d", "a", "k", "w", "hp", "len1", "len2", "len",
        "fors_msg_bytes", "fors_bytes", "wots_bytes", "sig_bytes", "pk_bytes", "sk_bytes",
        "seed_bytes", "tree_bits", "tree_bytes", "leaf_bits", "leaf_bytes", "dgst_bytes")]


class DRBG(ctypes.Structure):
    _fields_ = [("key", ctypes.c_uint8 * 32), ("v", ctypes.c_uint8 * 16), ("reseed_counter", ctypes.c_int)]


def build():
    """Compile libspx_oracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "spx_oracle.c")):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER(Params)
        u8p = ctypes.c_char_p
        L.spxo_params_from_name.argtypes = [P, ctypes.c_char_p]
        L.spxo_seed_keypair.argtypes = [P, u8p, u8p, u8p]
        L.spxo_sign_signature.argtypes = [P, u8p, ctypes.POINTER(ctypes.c_size_t), u8p, ctypes.c_size_t, u8p, u8p]
        L.spxo_verify.argtypes = [P, u8p, ctypes.c_size_t, u8p, ctypes.c_size_t, u8p]
        L.spxo_sha256.argtypes = [u8p, u8p, ctypes.c_size_t]
        L.spxo_shake256.argtypes = [u8p, ctypes.c_size_t, u8p, ctypes.c_size_t]
        L.spxo_mgf1.argtypes = [u8p, ctypes.c_size_t, u8p, ctypes.c_size_t]
        L.spxo_aes256_ecb.argtypes = [u8p, u8p, u8p]
        L.spxo_drbg_init.argtypes = [ctypes.POINTER(DRBG), u8p, u8p]
        L.spxo_drbg_bytes.argtypes = [ctypes.POINTER(DRBG), u8p, ctypes.c_size_t]
        L.spxo_randombytes_init.argtypes = [u8p]
        L.spxo_randombytes.argtypes = [u8p, ctypes.c_size_t]
        L.spxo_set_deterministic.argtypes = [ctypes.c_int]
        L.spxo_crypto_sign_keypair.argtypes = [P, u8p, u8p]
        L.spxo_crypto_sign_signature.argtypes = [P, u8p, ctypes.POINTER(ctypes.c_size_t), u8p, ctypes.c_size_t, u8p]
        L.spxo_crypto_sign.argtypes = [P, u8p, ctypes.POINTER(ctypes.c_ulonglong), u8p, ctypes.c_ulonglong, u8p]
        L.spxo_crypto_sign_open.argtypes = [P, u8p, ctypes.POINTER(ctypes.c_ulonglong), u8p, ctypes.c_ulonglong, u8p]
        L.spxo_thash.argtypes = [P, u8p, u8p, ctypes.c_uint, u8p, u8p]
        L.spxo_hash_message.argtypes = [P, u8p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32),
                                        u8p, u8p, u8p, ctypes.c_size_t]
        L.spxo_gen_message_random.argtypes = [P, u8p, u8p, u8p, u8p, ctypes.c_size_t]
        L.spxo_throughput.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_size_t, ctypes.c_double,
                                      ctypes.c_long, ctypes.POINTER(ctypes.c_double)]
        L.spxo_throughput.restype = ctypes.c_long
        L.spxo_units.argtypes = [ctypes.POINTER(ctypes.c_ulonglong * 3)]
        L.spxo_units.restype = None
        L.spxo_units_reset.argtypes = []
        L.spxo_units_reset.restype = None
        _lib = L
    return _lib


def params(name):
    p = Params()
    if lib().spxo_params_from_name(ctypes.byref(p), name.encode()) != 0:
        raise ValueError("unknown parameter set %r" % name)
    return p


class Oracle:
    """One parameter set of the CPU restatement."""

    def __init__(self, name):
        self.name = name
        self.p = params(name)
        self.L = lib()

    @property
    def sig_bytes(self):
        return self.p.sig_bytes

    def seed_keypair(self, seed):
        assert len(seed) == self.p.seed_bytes
        pk = ctypes.create_string_buffer(self.p.pk_bytes)
        sk = ctypes.create_string_buffer(self.p.sk_bytes)
        self.L.spxo_seed_keypair(ctypes.byref(self.p), pk, sk, bytes(seed))
        return pk.raw, sk.raw

    def sign(self, m, sk, optrand=None):
        if optrand is None:
            optrand = b"\xad" * self.p.n
        sig = ctypes.create_string_buffer(self.p.sig_bytes)
        siglen = ctypes.c_size_t(0)
        self.L.spxo_sign_signature(ctypes.byref(self.p), sig, ctypes.byref(siglen), bytes(m), len(m),
                                   bytes(sk), bytes(optrand))
        return sig.raw[:siglen.value]

    def verify(self, sig, m, pk):
        return self.L.spxo_verify(ctypes.byref(self.p), bytes(sig), len(sig), bytes(m), len(m), bytes(pk))

    def thash(self, data, inblocks, pub_seed, addr):
        out = ctypes.create_string_buffer(self.p.n)
        self.L.spxo_thash(ctypes.byref(self.p), out, bytes(data), inblocks, bytes(pub_seed), bytes(addr))
        return out.raw

    def hash_message(self, R, pk, m):
        dg = ctypes.create_string_buffer(64)
        tree = ctypes.c_uint64(0)
        leaf = ctypes.c_uint32(0)
        self.L.spxo_hash_message(ctypes.byref(self.p), dg, ctypes.byref(tree), ctypes.byref(leaf), bytes(R),
                                 bytes(pk), bytes(m), len(m))
        return dg.raw[:self.p.fors_msg_bytes], tree.value, leaf.value

    def throughput(self, op, threads, mlen, seconds, max_ops=1 << 40):
        secs = ctypes.c_double(0)
        done = self.L.spxo_throughput(ctypes.byref(self.p), op, threads, mlen, seconds, max_ops,
                                      ctypes.byref(secs))
        return done, secs.value


def units_reset():
    lib().spxo_units_reset()


def units():
    """(SHA-256 compressions, Keccak-f permutations, units inside wots_sign)
    counted on this thread since units_reset()."""
    a = (ctypes.c_ulonglong * 3)()
    lib().spxo_units(ctypes.byref(a))
    return tuple(a)


def sha256(data):
    out = ctypes.create_string_buffer(32)
    lib().spxo_sha256(out, bytes(data), len(data))
    return out.raw


def shake256(data, outlen):
    out = ctypes.create_string_buffer(outlen)
    lib().spxo_shake256(out, outlen, bytes(data), len(data))
    return out.raw


def aes256_ecb(key, block):
    out = ctypes.create_string_buffer(16)
    lib().spxo_aes256_ecb(bytes(key), bytes(block), out)
    return out.raw


class Drbg:
    """NIST AES-256 CTR DRBG with explicit state (rng.cu:139-241)."""

    def __init__(self, entropy48, personalization=None):
        self.s = DRBG()
        lib().spxo_drbg_init(ctypes.byref(self.s), bytes(entropy48), personalization)

    def bytes(self, n):
        out = ctypes.create_string_buffer(max(n, 1))
        lib().spxo_drbg_bytes(ctypes.byref(self.s), out, n)
        return out.raw[:n]
