"""cuspx_sign_noalloc -- signing for callers that cannot allocate device
memory while they run (cudaFree waits for the whole device; some hosts own
all device memory through their own allocator).  The caller provides device
buffers for inputs and outputs; the pipeline's scratch is a fixed array in
the library.  This file is collected last so that a failure here comes after
every other test has run; it must also pass alone in a fresh process."""
import ctypes
import random

import pytest

pytestmark = pytest.mark.gpu

CUSPX_ETOOBIG = -6


def _bind():
    import cuspx_gb300 as c
    L = c.lib()
    L.cuspx_sign_noalloc.argtypes = [ctypes.c_int, ctypes.c_size_t] + [ctypes.c_void_p] * 7 + [ctypes.c_void_p]
    L.cuspx_sign_noalloc.restype = ctypes.c_int
    return L


def _device_inputs(torch, sks, msgs):
    import numpy as np
    import cuspx_gb300 as c
    slab, offs, lens = c.pack_messages(msgs)
    d_sk = torch.from_numpy(np.frombuffer(b"".join(sks), dtype=np.uint8).copy()).cuda()
    d_msg = torch.from_numpy(np.frombuffer(bytes(slab), dtype=np.uint8).copy()).cuda()
    d_off = torch.from_numpy(offs.astype(np.int64)).cuda()
    d_len = torch.from_numpy(lens.astype(np.int64)).cuda()
    return d_sk, d_msg, d_off, d_len


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "shake256-192f-simple", "sha256-128s-simple",
                                     "shake256-128f-robust"])
def test_noalloc_matches_batch_entry_point_twice(engine, setname):
    torch = pytest.importorskip("torch")
    import cuspx_gb300 as c
    L = _bind()
    sid = c.set_id(setname)
    z = c.set_sizes(sid)
    rng = random.Random(2024)
    seeds = [bytes(rng.randrange(256) for _ in range(z["seed"])) for _ in range(3)]
    _, keys = engine.keypair_batch(sid, seeds)
    stream = torch.cuda.current_stream().cuda_stream
    for call, count in enumerate((9, 5)):   # two calls in a row, different inputs
        sks = [keys[(i + call) % 3] for i in range(count)]
        msgs = [bytes(rng.randrange(256) for _ in range(rng.randrange(0, 700))) for _ in range(count)]
        want, wst = engine.sign_batch(sid, sks, msgs)   # the existing entry point
        assert list(wst) == [0] * count
        d_sk, d_msg, d_off, d_len = _device_inputs(torch, sks, msgs)
        d_sig = torch.zeros(count * z["sig"], dtype=torch.uint8, device="cuda")
        d_st = torch.full((count,), 77, dtype=torch.int32, device="cuda")
        rc = L.cuspx_sign_noalloc(sid, count, d_sk.data_ptr(), d_msg.data_ptr(), d_off.data_ptr(),
                                  d_len.data_ptr(), None, d_sig.data_ptr(), d_st.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        got = d_sig.cpu().numpy().tobytes()
        assert got == b"".join(want), "call %d differs from cuspx_sign_batch" % call
        assert d_st.cpu().tolist() == [0] * count


def test_noalloc_rejects_batches_beyond_the_scratch(engine):
    torch = pytest.importorskip("torch")
    import cuspx_gb300 as c
    L = _bind()
    sid = c.set_id("sha256-128f-simple")
    d = torch.zeros(16, dtype=torch.uint8, device="cuda")
    p = d.data_ptr()
    # 42 signatures of 128f need more than the 8 MiB scratch (41 fit)
    assert L.cuspx_sign_noalloc(sid, 42, p, p, p, p, None, p, p, None) == CUSPX_ETOOBIG
    assert L.cuspx_sign_noalloc(sid, 1 << 30, p, p, p, p, None, p, p, None) == CUSPX_ETOOBIG
    assert L.cuspx_sign_noalloc(99, 1, p, p, p, p, None, p, p, None) == -1


def test_noalloc_refuses_misaligned_or_missing_buffers(engine):
    """Pointers the kernels would read with vector loads at a misaligned
    address, and a missing message slab, are refused before any launch."""
    torch = pytest.importorskip("torch")
    import cuspx_gb300 as c
    L = _bind()
    sid = c.set_id("sha256-128f-simple")
    d = torch.zeros(1 << 16, dtype=torch.uint8, device="cuda")
    p = d.data_ptr()   # 256-byte aligned
    ok = [p, p + 1024, p + 2048, p + 3072, None, p + 4096, p + 8192]
    for i, bump in ((0, 4), (1, 8), (2, 4), (3, 4), (5, 4), (6, 2)):
        args = list(ok)
        args[i] = args[i] + bump
        assert L.cuspx_sign_noalloc(sid, 1, *args, None) == -1, (i, bump)
    args = list(ok)
    args[4] = p + 12288 + 4   # optrand
    assert L.cuspx_sign_noalloc(sid, 1, *args, None) == -1
    args = list(ok)
    args[1] = None   # messages
    assert L.cuspx_sign_noalloc(sid, 1, *args, None) == -1
    torch.cuda.synchronize()
