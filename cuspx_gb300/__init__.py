"""cuspx_gb300 -- GB300-native SPHINCS+ signing and verification engine.

Python face of the C ABI in include/cuspx.h (the product is the native
library lib/libcuspx.so; this module only binds it with ctypes).  There is
no CPU fallback: importing the engine without its built library raises.

    from cuspx_gb300 import Engine
    eng = Engine()                                   # device 0
    s = eng.set_id("sha256-128f-simple")
    pks, sks = eng.keypair_batch(s, seeds)           # seeds: list of 3n-byte strings
    sigs, status = eng.sign_batch(s, sks, msgs)      # one sk per message
    verdicts = eng.verify_batch(s, pks, msgs, sigs)  # 0 accept / -1 reject
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(_HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libcuspx.so")

OP_KEYGEN, OP_SIGN, OP_VERIFY = 0, 1, 2

EXPORTS = [
    "cuspx_num_sets", "cuspx_set_id", "cuspx_set_name", "cuspx_set_sizes", "cuspx_create", "cuspx_destroy",
    "cuspx_error", "cuspx_set_tuning", "cuspx_get_tuning", "cuspx_keypair_batch", "cuspx_sign_batch",
    "cuspx_verify_batch", "cuspx_batch_create", "cuspx_batch_destroy", "cuspx_batch_upload", "cuspx_batch_run",
    "cuspx_batch_download", "cuspx_batch_download_async", "cuspx_batch_sync", "cuspx_batch_last_ms", "cuspx_batch_stream",
    "cuspx_batch_device_ptrs", "cuspx_batch_profile", "cuspx_batch_kernel_ms",
    "cuspx_randombytes_init", "cuspx_randombytes", "cuspx_aes256_ecb", "cuspx_set_deterministic",
    "cuspx_deterministic", "cuspx_int_peak", "cuspx_int_peak_mix", "cuspx_cmp_rate",
    "cuspx_set_tuning_for", "cuspx_get_tuning_for", "cuspx_clear_tuning_for", "cuspx_load_tuning",
    "cuspx_device_name",
]


class CuspxError(RuntimeError):
    pass


class Tuning(ctypes.Structure):
    """cuspx_tuning: the launch mapping of one parameter set."""
    _fields_ = [(f, ctypes.c_int) for f in ("leaf_block", "fors_block", "verify_block", "tree_warps",
                                            "chains_per_warp", "verify_mode", "fors_lanes_log2", "tree_mode",
                                            "chain_mode_max", "verify_slots", "verify_item_max",
                                            "verify_claim_min", "verify_groups", "verify_sorted_min",
                                            "verify_spec_max")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def lib():
    """Load lib/libcuspx.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("cuspx_gb300: %s is missing; build it with `python -m cuspx_gb300.build`" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    c = ctypes
    vp, sz, u8p, i32p, u64p, u32p = c.c_void_p, c.c_size_t, c.c_char_p, c.c_void_p, c.c_void_p, c.c_void_p
    L.cuspx_set_id.argtypes = [c.c_char_p]
    L.cuspx_set_name.argtypes = [c.c_int]
    L.cuspx_set_name.restype = c.c_char_p
    L.cuspx_set_sizes.argtypes = [c.c_int] + [c.POINTER(c.c_size_t)] * 4 + [c.POINTER(c.c_int)]
    L.cuspx_create.argtypes = [c.c_int, c.POINTER(vp)]
    L.cuspx_destroy.argtypes = [vp]
    L.cuspx_destroy.restype = None
    L.cuspx_error.argtypes = [vp]
    L.cuspx_error.restype = c.c_char_p
    L.cuspx_set_tuning.argtypes = [vp, c.c_int, c.POINTER(Tuning)]
    L.cuspx_get_tuning.argtypes = [vp, c.c_int, c.POINTER(Tuning)]
    L.cuspx_keypair_batch.argtypes = [vp, c.c_int, sz, vp, vp, vp]
    L.cuspx_sign_batch.argtypes = [vp, c.c_int, sz, vp, vp, vp, vp, vp, vp, vp]
    L.cuspx_verify_batch.argtypes = [vp, c.c_int, sz, vp, vp, vp, vp, vp, vp, vp]
    L.cuspx_batch_create.argtypes = [vp, c.c_int, c.c_int, sz, sz, sz, c.POINTER(vp)]
    L.cuspx_batch_destroy.argtypes = [vp]
    L.cuspx_batch_destroy.restype = None
    L.cuspx_batch_upload.argtypes = [vp, sz, vp, sz, vp, vp, sz, vp, vp, vp, vp]
    L.cuspx_batch_run.argtypes = [vp]
    L.cuspx_batch_download.argtypes = [vp, vp, vp, vp]
    L.cuspx_batch_download_async.argtypes = [vp, vp, vp, vp]
    L.cuspx_batch_sync.argtypes = [vp]
    L.cuspx_batch_last_ms.argtypes = [vp, c.POINTER(c.c_float)]
    L.cuspx_batch_stream.argtypes = [vp]
    L.cuspx_batch_stream.restype = vp
    L.cuspx_batch_device_ptrs.argtypes = [vp] + [c.POINTER(vp)] * 7
    L.cuspx_batch_profile.argtypes = [vp, c.c_int]
    L.cuspx_batch_kernel_ms.argtypes = [vp, c.c_int, c.POINTER(c.c_char_p), c.POINTER(c.c_double),
                                        c.POINTER(c.c_long)]
    L.cuspx_randombytes_init.argtypes = [vp, vp, c.c_int]
    L.cuspx_randombytes_init.restype = None
    L.cuspx_randombytes.argtypes = [vp, c.c_ulonglong]
    L.cuspx_aes256_ecb.argtypes = [vp, vp, vp]
    L.cuspx_aes256_ecb.restype = None
    L.cuspx_set_deterministic.argtypes = [c.c_int]
    L.cuspx_set_deterministic.restype = None
    L.cuspx_int_peak.argtypes = [c.c_int, c.c_int, c.POINTER(c.c_double), c.POINTER(c.c_float)]
    L.cuspx_int_peak_mix.argtypes = [c.c_int, c.c_int, c.c_int, c.POINTER(c.c_double), c.POINTER(c.c_float)]
    L.cuspx_cmp_rate.argtypes = [c.c_int, c.c_int, c.c_int, c.POINTER(c.c_double), c.POINTER(c.c_double)]
    L.cuspx_set_tuning_for.argtypes = [vp, c.c_int, c.c_int, sz, sz, c.POINTER(Tuning)]
    L.cuspx_get_tuning_for.argtypes = [vp, c.c_int, c.c_int, sz, c.POINTER(Tuning)]
    L.cuspx_clear_tuning_for.argtypes = [vp, c.c_int, c.c_int]
    L.cuspx_load_tuning.argtypes = [vp, c.c_char_p]
    L.cuspx_device_name.argtypes = [c.c_int, c.c_char_p, sz]
    _lib = L
    return L


def _buf(b):
    """ctypes pointer to the bytes of b (bytes / bytearray / numpy array)."""
    if b is None:
        return None
    if isinstance(b, bytes):
        return ctypes.cast(ctypes.c_char_p(b), ctypes.c_void_p)
    try:
        import numpy as np
        if isinstance(b, np.ndarray):
            assert b.flags["C_CONTIGUOUS"]
            return ctypes.c_void_p(b.ctypes.data)
    except ImportError:
        pass
    if isinstance(b, (bytearray, memoryview)):
        return ctypes.cast((ctypes.c_char * len(b)).from_buffer(b), ctypes.c_void_p)
    if isinstance(b, ctypes.Array):
        return ctypes.cast(b, ctypes.c_void_p)
    raise TypeError("unsupported buffer %r" % type(b))


def num_sets():
    return lib().cuspx_num_sets()


def set_id(name):
    r = lib().cuspx_set_id(name.encode())
    if r < 0:
        raise ValueError("unknown parameter set %r" % name)
    return r


def set_name(sid):
    return lib().cuspx_set_name(sid).decode()


def set_sizes(sid):
    """dict(pk, sk, sig, seed, n) in bytes"""
    v = [ctypes.c_size_t() for _ in range(4)]
    n = ctypes.c_int()
    if lib().cuspx_set_sizes(sid, *[ctypes.byref(x) for x in v], ctypes.byref(n)) != 0:
        raise ValueError("bad set id %r" % sid)
    return dict(pk=v[0].value, sk=v[1].value, sig=v[2].value, seed=v[3].value, n=n.value)


def pack_messages(msgs):
    """Messages -> (slab bytes, offsets, lengths) with 16-byte aligned offsets."""
    import numpy as np
    lens = np.array([len(m) for m in msgs], dtype=np.uint64)
    offs = np.zeros(len(msgs), dtype=np.uint64)
    total = 0
    for i, m in enumerate(msgs):
        offs[i] = total
        total += (len(m) + 15) & ~15
    slab = bytearray(total + 16)
    for i, m in enumerate(msgs):
        o = int(offs[i])
        slab[o:o + len(m)] = m
    return slab, offs, lens


class Engine:
    """One device context (cuspx_create)."""

    def __init__(self, device=0):
        self.L = lib()
        h = ctypes.c_void_p()
        rc = self.L.cuspx_create(device, ctypes.byref(h))
        if rc != 0:
            raise CuspxError("cuspx_create(%d) failed (%d): no usable CUDA device" % (device, rc))
        self.h = h

    def close(self):
        if self.h:
            self.L.cuspx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise CuspxError("%s failed (%d): %s" % (what, rc, self.L.cuspx_error(self.h).decode()))

    set_id = staticmethod(set_id)
    set_sizes = staticmethod(set_sizes)

    def set_tuning(self, sid, **kw):
        """Change fields of a set's launch mapping (others keep their value)."""
        t = Tuning(0, 0, 0, 0, 0, -1, -1, -1, -1, 0, -1, 0, 0, -1, -1)
        for k, v in kw.items():
            setattr(t, k, int(v))
        self._check(self.L.cuspx_set_tuning(self.h, sid, ctypes.byref(t)), "set_tuning")

    def get_tuning(self, sid):
        t = Tuning()
        self._check(self.L.cuspx_get_tuning(self.h, sid, ctypes.byref(t)), "get_tuning")
        return t.as_dict()

    def set_tuning_for(self, sid, op, min_count, max_count, **kw):
        """Mapping of (set, op) for batches of min_count..max_count items
        (fields not given keep the set's base mapping)."""
        t = Tuning(0, 0, 0, 0, 0, -1, -1, -1, -1, 0, -1, 0, 0, -1, -1)
        for k, v in kw.items():
            setattr(t, k, int(v))
        self._check(self.L.cuspx_set_tuning_for(self.h, sid, op, min_count, max_count, ctypes.byref(t)),
                    "set_tuning_for")

    def get_tuning_for(self, sid, op, count):
        """The mapping a batch of `count` items of (set, op) runs with."""
        t = Tuning()
        self._check(self.L.cuspx_get_tuning_for(self.h, sid, op, count, ctypes.byref(t)), "get_tuning_for")
        return t.as_dict()

    def clear_tuning_for(self, sid, op=-1):
        self._check(self.L.cuspx_clear_tuning_for(self.h, sid, op), "clear_tuning_for")

    def load_tuning(self, path):
        """Install a tuning file's entries for this GPU; returns how many."""
        rc = self.L.cuspx_load_tuning(self.h, path.encode())
        if rc < 0:
            raise CuspxError("load_tuning(%s) failed (%d)" % (path, rc))
        return rc

    def keypair_batch(self, sid, seeds):
        z = set_sizes(sid)
        cnt = len(seeds)
        sb = b"".join(bytes(s) for s in seeds)
        assert len(sb) == cnt * z["seed"]
        pk = ctypes.create_string_buffer(cnt * z["pk"])
        sk = ctypes.create_string_buffer(cnt * z["sk"])
        self._check(self.L.cuspx_keypair_batch(self.h, sid, cnt, _buf(sb), _buf(pk), _buf(sk)), "keypair_batch")
        return ([pk.raw[i * z["pk"]:(i + 1) * z["pk"]] for i in range(cnt)],
                [sk.raw[i * z["sk"]:(i + 1) * z["sk"]] for i in range(cnt)])

    def sign_batch(self, sid, sks, msgs, optrand=None):
        import numpy as np
        z = set_sizes(sid)
        cnt = len(msgs)
        assert len(sks) == cnt
        skb = b"".join(bytes(s) for s in sks)
        slab, offs, lens = pack_messages(msgs)
        opt = b"".join(bytes(o) for o in optrand) if optrand is not None else None
        sig = ctypes.create_string_buffer(max(1, cnt * z["sig"]))
        st = np.zeros(cnt, dtype=np.int32)
        self._check(self.L.cuspx_sign_batch(self.h, sid, cnt, _buf(skb), _buf(slab), _buf(offs), _buf(lens),
                                            _buf(opt), _buf(sig), _buf(st)), "sign_batch")
        return [sig.raw[i * z["sig"]:(i + 1) * z["sig"]] for i in range(cnt)], st

    def verify_batch(self, sid, pks, msgs, sigs, siglens=None):
        import numpy as np
        z = set_sizes(sid)
        cnt = len(msgs)
        pkb = b"".join(bytes(p) for p in pks)
        slab, offs, lens = pack_messages(msgs)
        rows = bytearray(cnt * z["sig"])
        sl = np.zeros(cnt, dtype=np.uint64)
        for i, s in enumerate(sigs):
            s = bytes(s)[:z["sig"]]
            rows[i * z["sig"]:i * z["sig"] + len(s)] = s
            sl[i] = len(sigs[i]) if siglens is None else siglens[i]
        v = np.zeros(cnt, dtype=np.int32)
        self._check(self.L.cuspx_verify_batch(self.h, sid, cnt, _buf(pkb), _buf(slab), _buf(offs), _buf(lens),
                                              _buf(rows), _buf(sl), _buf(v)), "verify_batch")
        return v

    def batch(self, op, sid, capacity, msg_capacity=0, key_capacity=0):
        return Batch(self, op, sid, capacity, msg_capacity, key_capacity)


class Batch:
    """A reusable device-resident batch (cuspx_batch_*)."""

    def __init__(self, eng, op, sid, capacity, msg_capacity=0, key_capacity=0):
        self.eng, self.L, self.op, self.sid = eng, eng.L, op, sid
        self.sizes = set_sizes(sid)
        h = ctypes.c_void_p()
        eng._check(self.L.cuspx_batch_create(eng.h, op, sid, capacity, msg_capacity, key_capacity,
                                              ctypes.byref(h)), "batch_create")
        self.h = h
        self.count = 0

    def close(self):
        if self.h:
            self.L.cuspx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, count, keys, nkeys=0, key_index=None, msgs=None, msg_bytes=0, msg_off=None, msg_len=None,
               aux=None, siglens=None):
        self.eng._check(self.L.cuspx_batch_upload(self.h, count, _buf(keys), nkeys, _buf(key_index), _buf(msgs),
                                                  msg_bytes, _buf(msg_off), _buf(msg_len), _buf(aux),
                                                  _buf(siglens)), "batch_upload")
        self.count = count

    def run(self):
        self.eng._check(self.L.cuspx_batch_run(self.h), "batch_run")

    def download(self, out=None, out2=None, status=None):
        self.eng._check(self.L.cuspx_batch_download(self.h, _buf(out), _buf(out2), _buf(status)), "batch_download")

    def download_async(self, out=None, out2=None, status=None):
        """Enqueue the copies of download() on the batch stream without
        waiting; the host buffers must be pinned and stay alive until sync()."""
        self.eng._check(self.L.cuspx_batch_download_async(self.h, _buf(out), _buf(out2), _buf(status)),
                        "batch_download_async")

    def sync(self):
        self.eng._check(self.L.cuspx_batch_sync(self.h), "batch_sync")

    def last_ms(self):
        f = ctypes.c_float()
        self.eng._check(self.L.cuspx_batch_last_ms(self.h, ctypes.byref(f)), "batch_last_ms")
        return f.value

    def stream(self):
        return self.L.cuspx_batch_stream(self.h)

    def profile(self, enable=True):
        self.eng._check(self.L.cuspx_batch_profile(self.h, 1 if enable else 0), "batch_profile")

    def kernel_ms(self):
        n = self.L.cuspx_batch_kernel_ms(self.h, -1, None, None, None)
        out = []
        for i in range(n):
            name = ctypes.c_char_p()
            ms = ctypes.c_double()
            cnt = ctypes.c_long()
            self.L.cuspx_batch_kernel_ms(self.h, i, ctypes.byref(name), ctypes.byref(ms), ctypes.byref(cnt))
            out.append((name.value.decode(), ms.value, cnt.value))
        return out


def randombytes_init(entropy48, personalization=None):
    lib().cuspx_randombytes_init(_buf(bytes(entropy48)), _buf(personalization), 256)


def randombytes(n):
    b = ctypes.create_string_buffer(max(1, n))
    lib().cuspx_randombytes(_buf(b), n)
    return b.raw[:n]


def aes256_ecb(key, block):
    out = ctypes.create_string_buffer(16)
    lib().cuspx_aes256_ecb(_buf(bytes(key)), _buf(bytes(block)), _buf(out))
    return out.raw


def set_deterministic(on):
    lib().cuspx_set_deterministic(1 if on else 0)


def int_peak(device=0, iters=4096, mix=0):
    """Measured integer peak (ops/s): mix 0 the ALU-pipe SHF/LOP3/IADD3 shape
    (Keccak-f), mix 1 a SHA-256 round with one add in eight on the FMA pipe."""
    ops = ctypes.c_double()
    ms = ctypes.c_float()
    rc = lib().cuspx_int_peak_mix(device, iters, mix, ctypes.byref(ops), ctypes.byref(ms))
    if rc != 0:
        raise CuspxError("cuspx_int_peak_mix failed (%d)" % rc)
    return ops.value, ms.value


def device_name(device=0):
    buf = ctypes.create_string_buffer(256)
    if lib().cuspx_device_name(device, buf, 256) != 0:
        raise CuspxError("no CUDA device %d" % device)
    return buf.value.decode()


def cmp_rate(warps_per_sm, device=0, iters=2048):
    """(SHA-256 compressions/s over all SMs, ns per compression of one lane's
    dependent chain) with warps_per_sm warps on every SM."""
    r = ctypes.c_double()
    ns = ctypes.c_double()
    rc = lib().cuspx_cmp_rate(device, warps_per_sm, iters, ctypes.byref(r), ctypes.byref(ns))
    if rc != 0:
        raise CuspxError("cuspx_cmp_rate failed (%d)" % rc)
    return r.value, ns.value


def dropin_path(set_name):
    """Path of the NIST api.h drop-in library for one parameter set."""
    return os.path.join(LIB_DIR, "libspx_%s.so" % set_name)


# ---------------------------------------------------------------------------
# serving face (include/cuspx_serve.h)
# ---------------------------------------------------------------------------
SUBMIT_BORROW, SUBMIT_DETACH = 1, 2
E_BUSY, E_TIMEDOUT, E_NOMEM = -4, -5, -3


class ServeConfig(ctypes.Structure):
    _fields_ = [("mem_budget", ctypes.c_size_t), ("max_batch", ctypes.c_int), ("max_inflight", ctypes.c_int),
                ("window_us", ctypes.c_int), ("max_keys", ctypes.c_int), ("max_queue", ctypes.c_size_t),
                ("max_queue_ms", ctypes.c_double), ("max_launch_ms", ctypes.c_double),
                ("gpu_ops_per_s", ctypes.c_double)]


class ServeCounters(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("submitted", "completed", "refused", "failed", "launches",
                                                 "sign_done", "verify_done")] + \
               [("bytes_inflight", ctypes.c_size_t), ("bytes_peak", ctypes.c_size_t)] + \
               [(f, ctypes.c_double) for f in ("sign_p50_us", "sign_p99_us", "verify_p50_us", "verify_p99_us",
                                                 "mean_batch")] + \
               [(f, ctypes.c_double * 3) for f in ("sign_p50_bucket_us", "sign_p99_bucket_us",
                                                     "verify_p50_bucket_us", "verify_p99_bucket_us")] + \
               [("bucket_count", (ctypes.c_uint64 * 3) * 2)] + \
               [("launch_ms_mean", ctypes.c_double), ("launch_ms_max", ctypes.c_double)]

    def as_dict(self):
        out = {}
        for f, _ in self._fields_:
            v = getattr(self, f)
            if f == "bucket_count":
                v = [list(v[0]), list(v[1])]
            elif isinstance(v, ctypes.Array):
                v = list(v)
            out[f] = v
        return out


class LoadgenSample(ctypes.Structure):
    _fields_ = [("set", ctypes.c_int32), ("key_id", ctypes.c_uint32), ("status", ctypes.c_int32),
                ("pad", ctypes.c_uint32), ("mlen", ctypes.c_uint64), ("msg_off", ctypes.c_uint64),
                ("sig_off", ctypes.c_uint64)]


class LoadgenConfig(ctypes.Structure):
    _fields_ = [("rate", ctypes.c_double), ("seconds", ctypes.c_double), ("verify_frac", ctypes.c_double),
                ("nsets", ctypes.c_int), ("sets", ctypes.POINTER(ctypes.c_int)), ("keys_per_set", ctypes.c_uint32),
                ("min_len", ctypes.c_uint64), ("max_len", ctypes.c_uint64), ("corrupt_frac", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("pool", ctypes.c_int), ("sample_every", ctypes.c_uint32),
                ("sample_max", ctypes.c_uint32), ("samples", ctypes.POINTER(LoadgenSample)),
                ("arena", ctypes.c_void_p), ("arena_bytes", ctypes.c_size_t)]


class LoadgenResult(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("offered", "completed", "refused", "wrong_verdicts", "sign_done",
                                                 "verify_done")] + \
               [(f, ctypes.c_double) for f in ("wall_s", "throughput", "sign_throughput", "verify_throughput",
                                                 "sign_p50_us", "sign_p99_us", "verify_p50_us", "verify_p99_us",
                                                 "mean_batch")] + \
               [(f, ctypes.c_double * 3) for f in ("sign_p50_bucket_us", "sign_p99_bucket_us",
                                                     "verify_p50_bucket_us", "verify_p99_bucket_us")] + \
               [("launch_ms_mean", ctypes.c_double), ("launch_ms_max", ctypes.c_double)] + \
               [("set_sign_done", ctypes.c_uint64 * 8), ("set_verify_done", ctypes.c_uint64 * 8),
                ("set_msg_units", ctypes.c_double * 8), ("sampled", ctypes.c_uint64)]

    def as_dict(self):
        return {f: (list(getattr(self, f)) if isinstance(getattr(self, f), ctypes.Array) else getattr(self, f))
                for f, _ in self._fields_}


SERVE_EXPORTS = ["cuspx_serve_create", "cuspx_serve_destroy", "cuspx_serve_add_keys", "cuspx_serve_prepare",
                 "cuspx_serve_add_pubkeys",
                 "cuspx_serve_submit", "cuspx_serve_wait", "cuspx_serve_stats", "cuspx_serve_reset_stats",
                 "cuspx_serve_loadgen"]


def _bind_serve(L):
    if getattr(L, "_serve_bound", False):
        return L
    c, vp = ctypes, ctypes.c_void_p
    L.cuspx_serve_create.argtypes = [vp, c.POINTER(ServeConfig), c.POINTER(vp)]
    L.cuspx_serve_destroy.argtypes = [vp]
    L.cuspx_serve_destroy.restype = None
    L.cuspx_serve_add_keys.argtypes = [vp, c.c_int, c.c_size_t, vp, c.POINTER(c.c_uint32)]
    L.cuspx_serve_prepare.argtypes = [vp, c.c_int, c.c_int]
    L.cuspx_serve_add_pubkeys.argtypes = [vp, c.c_int, c.c_size_t, vp, c.POINTER(c.c_uint32)]
    L.cuspx_serve_submit.argtypes = [vp, c.c_int, c.c_int, c.c_uint32, vp, c.c_size_t, vp, c.c_size_t, c.c_uint,
                                     c.POINTER(c.c_uint64)]
    L.cuspx_serve_wait.argtypes = [vp, c.c_uint64, c.c_long, vp, c.POINTER(c.c_int32), c.POINTER(c.c_double)]
    L.cuspx_serve_stats.argtypes = [vp, c.POINTER(ServeCounters)]
    L.cuspx_serve_reset_stats.argtypes = [vp]
    L.cuspx_serve_loadgen.argtypes = [vp, c.POINTER(LoadgenConfig), c.POINTER(LoadgenResult)]
    L._serve_bound = True
    return L


class Server:
    """A serving loop on one engine context (cuspx_serve_*)."""

    def __init__(self, eng, mem_budget=0, max_batch=0, max_inflight=0, window_us=0, max_keys=0, max_queue=0,
                 max_queue_ms=0.0, max_launch_ms=0.0, gpu_ops_per_s=0.0):
        self.eng = eng
        self.L = _bind_serve(eng.L)
        cfg = ServeConfig(mem_budget, max_batch, max_inflight, window_us, max_keys, max_queue, max_queue_ms,
                          max_launch_ms, gpu_ops_per_s)
        h = ctypes.c_void_p()
        eng._check(self.L.cuspx_serve_create(eng.h, ctypes.byref(cfg), ctypes.byref(h)), "serve_create")
        self.h = h
        self._keep = {}

    def close(self):
        if self.h:
            self.L.cuspx_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_keys(self, sid, sks):
        b = b"".join(bytes(x) for x in sks)
        first = ctypes.c_uint32()
        self.eng._check(self.L.cuspx_serve_add_keys(self.h, sid, len(sks), _buf(b), ctypes.byref(first)),
                        "serve_add_keys")
        return list(range(first.value, first.value + len(sks)))

    def prepare(self, op, sid):
        """Create every launch slot of (op, set) now rather than on first use."""
        self.eng._check(self.L.cuspx_serve_prepare(self.h, op, sid), "serve_prepare")

    def add_pubkeys(self, sid, pks):
        b = b"".join(bytes(x) for x in pks)
        first = ctypes.c_uint32()
        self.eng._check(self.L.cuspx_serve_add_pubkeys(self.h, sid, len(pks), _buf(b), ctypes.byref(first)),
                        "serve_add_pubkeys")
        return list(range(first.value, first.value + len(pks)))

    def submit(self, op, sid, key_id, msg, sig=None):
        """Returns a ticket, or raises CuspxError with the refusal code."""
        t = ctypes.c_uint64()
        msg = bytes(msg)
        sig = bytes(sig) if sig is not None else None
        rc = self.L.cuspx_serve_submit(self.h, op, sid, key_id, _buf(msg), len(msg), _buf(sig),
                                       len(sig) if sig is not None else 0, 0, ctypes.byref(t))
        if rc != 0:
            err = CuspxError("serve_submit refused (%d)" % rc)
            err.code = rc
            raise err
        return t.value

    def wait(self, ticket, timeout_us=-1, sig_bytes=0):
        out = ctypes.create_string_buffer(max(1, sig_bytes))
        st = ctypes.c_int32()
        lat = ctypes.c_double()
        rc = self.L.cuspx_serve_wait(self.h, ticket, timeout_us, _buf(out), ctypes.byref(st), ctypes.byref(lat))
        if rc != 0:
            raise CuspxError("serve_wait (%d)" % rc)
        return (out.raw[:sig_bytes] if sig_bytes else None), st.value, lat.value

    def stats(self):
        s = ServeCounters()
        self.L.cuspx_serve_stats(self.h, ctypes.byref(s))
        return s.as_dict()

    def reset_stats(self):
        self.L.cuspx_serve_reset_stats(self.h)

    def loadgen(self, rate, seconds, sets, keys_per_set, verify_frac=0.7, min_len=16, max_len=1 << 20,
                corrupt_frac=0.0, seed=1, pool=64, sample_every=0, sample_max=0, arena_bytes=0):
        """Open-loop Poisson stream.  With sample_every > 0, one timed sign
        request in sample_every keeps its signature (up to sample_max, within
        arena_bytes); out["samples"] lists (set, key_id, status, msg, sig)."""
        arr = (ctypes.c_int * len(sets))(*sets)
        smp = (LoadgenSample * max(1, sample_max))()
        arena = ctypes.create_string_buffer(max(1, arena_bytes))
        cfg = LoadgenConfig(rate, seconds, verify_frac, len(sets), arr, keys_per_set, min_len, max_len,
                            corrupt_frac, seed, pool, sample_every, sample_max,
                            ctypes.cast(smp, ctypes.POINTER(LoadgenSample)), ctypes.cast(arena, ctypes.c_void_p),
                            arena_bytes)
        res = LoadgenResult()
        rc = self.L.cuspx_serve_loadgen(self.h, ctypes.byref(cfg), ctypes.byref(res))
        out = res.as_dict()
        out["rc"] = rc
        raw = arena.raw
        out["samples"] = []
        for i in range(res.sampled):
            e = smp[i]
            sigb = set_sizes(e.set)["sig"]
            out["samples"].append((e.set, e.key_id, e.status, raw[e.msg_off:e.msg_off + e.mlen],
                                   raw[e.sig_off:e.sig_off + sigb]))
        return out


# ---------------------------------------------------------------------------
# mixed parameter sets in one graph launch (cuspx_group_run)
# ---------------------------------------------------------------------------
def _bind_group(L):
    if not getattr(L, "_group_bound", False):
        L.cuspx_group_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_float)]
        L._group_bound = True
    return L


def group_run(eng, batches):
    """Run several uploaded batches as one CUDA graph; returns device ms."""
    L = _bind_group(eng.L)
    arr = (ctypes.c_void_p * len(batches))(*[b.h.value for b in batches])
    ms = ctypes.c_float()
    eng._check(L.cuspx_group_run(eng.h, arr, len(batches), ctypes.byref(ms)), "group_run")
    return ms.value


class MixedSigner:
    """Sign requests of several parameter sets, each with its own key, in one
    graph launch: requests are grouped per set into device-resident batches
    (keys uploaded once per batch) that run concurrently in one graph."""

    def __init__(self, eng):
        self.eng = eng
        self.batches = {}

    def sign(self, set_ids, sks, msgs, optrand=None):
        import numpy as np
        order = {}
        for i, sid in enumerate(set_ids):
            order.setdefault(sid, []).append(i)
        runs = []
        for sid, idx in order.items():
            z = set_sizes(sid)
            slab, offs, lens = pack_messages([msgs[i] for i in idx])
            keys = b"".join(bytes(sks[i]) for i in idx)
            cap = len(idx)
            b = self.batches.get(sid)
            if b is None or b._cap < cap or b._mcap < len(slab):
                if b is not None:
                    b.close()
                b = self.eng.batch(OP_SIGN, sid, max(cap, 1), max(len(slab), 1 << 16), max(cap, 1))
                b._cap, b._mcap = max(cap, 1), max(len(slab), 1 << 16)
                self.batches[sid] = b
            opt = b"".join(bytes(optrand[i]) for i in idx) if optrand is not None else None
            b.upload(cap, keys, cap, None, slab, len(slab), offs, lens, opt)
            runs.append((sid, idx, b, z))
        ms = group_run(self.eng, [r[2] for r in runs])
        sigs = [None] * len(msgs)
        status = np.zeros(len(msgs), dtype=np.int32)
        for sid, idx, b, z in runs:
            out = np.zeros(len(idx) * z["sig"], dtype=np.uint8)
            st = np.zeros(len(idx), dtype=np.int32)
            b.download(out, None, st)
            for j, i in enumerate(idx):
                sigs[i] = out[j * z["sig"]:(j + 1) * z["sig"]].tobytes()
                status[i] = st[j]
        return sigs, status, ms

    def close(self):
        for b in self.batches.values():
            b.close()
        self.batches = {}
