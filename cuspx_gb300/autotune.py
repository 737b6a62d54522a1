"""Per-parameter-set launch-mapping autotuner.

The reference fixes its mapping at compile time (all_option.h:7-68:
HP_PARALLELISM, block-size and load-balancing switches).  Here the mapping is
a runtime cuspx_tuning per parameter set, and this module picks it by timing
real batches on the device:

  sign:   chain_mode_max (lane per chain vs lane per leaf for this batch
          size), fors_lanes_log2 (lanes per FORS tree), tree_mode,
          leaf_block, fors_block, tree_warps
  verify: verify_mode (layered kernels or one persistent launch), and for
          each the chains per warp / items per warp and block size

Search is coordinate descent: each knob is swept with the others held, the
best value kept, for two passes.  Every candidate is timed with CUDA events
on the batch stream (min of `reps` runs after a warm-up).  Results are cached
per (GPU name, set, op, batch-size bucket) in a JSON file
($CUSPX_TUNE_CACHE, default ~/.cache/cuspx/tune.json).
"""
import json
import os

import numpy as np

from . import OP_SIGN, OP_VERIFY, pack_messages, set_name, set_sizes

SIGN_SPACE = {
    "chain_mode_max": [0, 256],
    "fors_lanes_log2": [0, 1, 2, 3, 5],
    "tree_mode": [0, 1],
    "leaf_block": [64, 128, 256],
    "fors_block": [64, 128, 256],
    "tree_warps": [1, 2, 4],
}
VERIFY_SPACE = {
    "verify_mode": [0, 1, 2],
    "verify_slots": [2, 3, 4, 6, 8],
    "chains_per_warp": [32, 64, 128, 256, 512],
    "verify_block": [32, 64, 128],
}


def _cache_path():
    return os.environ.get("CUSPX_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "cuspx", "tune.json"))


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "gpu"


def _bucket(n):
    b = 1
    while b < n:
        b *= 4
    return b


def _load_cache():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_cache(c):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(c, f, indent=1)
    except OSError:
        pass


def _time(batch, reps):
    batch.run()
    batch.sync()
    best = None
    for _ in range(reps):
        batch.run()
        batch.sync()
        ms = batch.last_ms()
        best = ms if best is None else min(best, ms)
    return best


def tune(eng, sid, op=OP_SIGN, count=1024, mlen=64, reps=2, passes=2, use_cache=True, verbose=False):
    """Pick and install the fastest mapping of `op` for set `sid` at `count`
    items of `mlen`-byte messages.  Returns (mapping dict, best ms)."""
    key = "%s|%s|%s|%d" % (_gpu_name(), set_name(sid), "sign" if op == OP_SIGN else "verify", _bucket(count))
    cache = _load_cache() if use_cache else {}
    if key in cache:
        eng.set_tuning(sid, **cache[key]["mapping"])
        return cache[key]["mapping"], cache[key]["ms"]
    z = set_sizes(sid)
    rng = np.random.default_rng(1234)
    pks, sks = eng.keypair_batch(sid, [rng.bytes(z["seed"])])
    msgs = [rng.bytes(mlen) for _ in range(count)]
    slab, offs, lens = pack_messages(msgs)
    kidx = np.zeros(count, dtype=np.uint32)
    sb = eng.batch(OP_SIGN, sid, count, len(slab), 1)
    sb.upload(count, sks[0], 1, kidx, slab, len(slab), offs, lens)
    batch = sb
    if op == OP_VERIFY:
        sb.run()
        sigs = np.zeros(count * z["sig"], dtype=np.uint8)
        sb.download(sigs)
        vb = eng.batch(OP_VERIFY, sid, count, len(slab), 1)
        vb.upload(count, pks[0], 1, kidx, slab, len(slab), offs, lens, sigs)
        batch = vb
    space = SIGN_SPACE if op == OP_SIGN else VERIFY_SPACE
    cur = {k: v for k, v in eng.get_tuning(sid).items() if k in space}
    best_ms = _time(batch, reps)
    for _ in range(passes):
        improved = False
        for knob, values in space.items():
            for v in values:
                if v == cur[knob]:
                    continue
                trial = dict(cur, **{knob: v})
                eng.set_tuning(sid, **trial)
                ms = _time(batch, reps)
                if verbose:
                    print("  %s=%s %.3f ms" % (knob, v, ms))
                if ms < best_ms * 0.995:
                    best_ms, cur, improved = ms, trial, True
            eng.set_tuning(sid, **cur)
        if not improved:
            break
    eng.set_tuning(sid, **cur)
    batch.close()
    if op == OP_VERIFY:
        sb.close()
    if use_cache:
        cache = _load_cache()
        cache[key] = {"mapping": cur, "ms": best_ms, "count": count, "mlen": mlen}
        _save_cache(cache)
    return cur, best_ms
