"""Per-parameter-set, per-batch-size launch-mapping autotuner.

The reference fixes its mapping at compile time (all_option.h:7-68:
HP_PARALLELISM, block-size and load-balancing switches).  Here the mapping is
a runtime cuspx_tuning per parameter set, refined per (operation, batch-size
bucket), and this module picks it by timing real batches on the device:

  sign:   chain_mode_max (lane per chain vs lane per leaf for this batch
          size), fors_lanes_log2 (lanes per FORS tree), tree_mode,
          leaf_block, fors_block, tree_warps
  verify: verify_item_max (one item per block at this size or not),
          verify_mode (layered kernels, one persistent launch, or layered
          kernels over length-sorted chains), and for each the chains per
          warp / items per warp, block size, the persistent kernel's claim
          threshold and the sorted mode's item groups

Search is coordinate descent: each knob is swept with the others held, the
best value kept, for two passes.  Every candidate is timed with CUDA events
on the batch stream (min of `reps` runs after a warm-up).

The result is installed in the library, not only in Python: the engine gets
a per-size entry (cuspx_set_tuning_for) for batches in the bucket's range
(b/4 + 1 .. b items for the power of 4 b at or above the tuned count), and
the result is written to a tab-separated tuning file ($CUSPX_TUNE_CACHE,
default ~/.cache/cuspx/tune.tsv), one line per (GPU name, set, op, bucket).
cuspx_create reads that file, so every later
context -- the api.h drop-ins, the one-shot calls and the serving loop
included -- runs the tuned mappings without Python.
"""
import os

import numpy as np

from . import OP_SIGN, OP_VERIFY, device_name, pack_messages, set_name, set_sizes

SIGN_SPACE = {
    "chain_mode_max": [0, 256],
    "fors_lanes_log2": [0, 1, 2, 3, 5],
    "tree_mode": [0, 1],
    "leaf_block": [64, 128, 256],
    "fors_block": [64, 128, 256],
    "tree_warps": [1, 2, 4],
}
VERIFY_SPACE = {
    "verify_item_max": [0, None],   # None: this bucket's size (one item per block)
    "verify_sorted_min": [0, 1],    # 1: every batch of this bucket verifies as verify_mode 3
    "verify_spec_max": [0, None],   # None: this bucket's size (speculative chains, up to 64 items)
    "verify_mode": [0, 1, 2, 3],
    "verify_slots": [2, 3, 4, 6, 8],
    "chains_per_warp": [32, 64, 128, 256, 512],
    "verify_block": [32, 64, 128],
    "verify_claim_min": [1, 2, 3, 4],
    "verify_groups": [2, 4, 6, 8],
}
OP_NAMES = {OP_SIGN: "sign", OP_VERIFY: "verify"}
SPEC_MAX_ITEMS = 64   # largest verify_spec_max the library accepts


def cache_path():
    return os.environ.get("CUSPX_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "cuspx", "tune.tsv"))


def bucket(n):
    """Batch-size bucket: the power of 4 at or above n.  An entry tuned for
    bucket b applies to batches of b/4 + 1 .. b items (1 item for b = 1)."""
    b = 1
    while b < n:
        b *= 4
    return b


def bucket_range(b):
    return (b // 4 + 1 if b > 1 else 1), b


def load_cache(path=None):
    """{(gpu, set, op, bucket): (ms, mapping)} from the tuning file (one line
    per entry: gpu, set, op, min_count, max_count = bucket, ms, knobs)."""
    out = {}
    try:
        with open(path or cache_path()) as f:
            for line in f:
                col = line.rstrip("\n").split("\t")
                if len(col) != 7:
                    continue
                mapping = dict((k, int(v)) for k, v in (kv.split("=") for kv in col[6].split(",") if kv))
                out[(col[0], col[1], col[2], int(col[4]))] = (float(col[5]), mapping)
    except (OSError, ValueError):
        pass
    return out


def save_entry(key, ms, mapping, path=None):
    """Write (or replace) one line of the tuning file."""
    path = path or cache_path()
    cache = load_cache(path)
    cache[key] = (ms, mapping)
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            for (gpu, sname, op, b), (m, mp) in sorted(cache.items()):
                lo, hi = bucket_range(b)
                f.write("%s\t%s\t%s\t%d\t%d\t%.4f\t%s\n" % (gpu, sname, op, lo, hi, m,
                                                            ",".join("%s=%d" % kv for kv in sorted(mp.items()))))
        os.replace(tmp, path)
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


def search_space(op, b):
    """The knob values swept for `op` in batch-size bucket b (None in the
    tables stands for b itself)."""
    space = {k: [b if v is None else v for v in vals]
             for k, vals in (SIGN_SPACE if op == OP_SIGN else VERIFY_SPACE).items()}
    if "verify_spec_max" in space and b > SPEC_MAX_ITEMS:   # the speculative path covers up to 64 items
        space["verify_spec_max"] = [0]
    return space


def tune(eng, sid, op=OP_SIGN, count=1024, mlen=64, msgs=None, reps=2, passes=2, use_cache=True, verbose=False):
    """Pick the fastest mapping of `op` for set `sid` on a batch of `count`
    `mlen`-byte random messages, or on the given `msgs` (their count and
    lengths), install it in the engine for that batch-size bucket and record
    it in the tuning file.  Returns (mapping dict, best ms)."""
    if msgs is not None:
        count = len(msgs)
    b = bucket(count)
    key = (device_name(), set_name(sid), OP_NAMES[op], b)
    if use_cache:
        hit = load_cache().get(key)
        if hit:
            eng.set_tuning_for(sid, op, *bucket_range(b), **hit[1])
            return hit[1], hit[0]
    z = set_sizes(sid)
    rng = np.random.default_rng(1234)
    pks, sks = eng.keypair_batch(sid, [rng.bytes(z["seed"])])
    if msgs is None:
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
    space = search_space(op, b)
    cur = {k: v for k, v in eng.get_tuning_for(sid, op, count).items() if k in space}
    eng.set_tuning_for(sid, op, *bucket_range(b), **cur)
    best_ms = _time(batch, reps)
    for _ in range(passes):
        improved = False
        for knob, values in space.items():
            for v in values:
                if v == cur[knob]:
                    continue
                trial = dict(cur, **{knob: v})
                eng.set_tuning_for(sid, op, *bucket_range(b), **trial)
                ms = _time(batch, reps)
                if verbose:
                    print("  %s=%s %.3f ms" % (knob, v, ms))
                if ms < best_ms * 0.995:
                    best_ms, cur, improved = ms, trial, True
            eng.set_tuning_for(sid, op, *bucket_range(b), **cur)
        if not improved:
            break
    eng.set_tuning_for(sid, op, *bucket_range(b), **cur)
    batch.close()
    if op == OP_VERIFY:
        sb.close()
    if use_cache:
        save_entry(key, best_ms, cur)
    return cur, best_ms
