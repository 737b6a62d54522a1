"""Benchmark: batched SPHINCS+-SHA-256-128f-simple signing on one GB300.

Workload (the batched configuration the headline metric is quoted on): one
keypair, 4096 messages of 64 uniform random bytes, all signed in one
graph-launched batch, then all 4096 verified in one batch; the signatures of a
seeded 64-message subset are byte-compared with the CPU oracle.

A step is one sign batch of 4096 messages.  `value` is signs/s with inputs
already resident in HBM (device time from CUDA events on the batch stream);
`e2e` is the same through the C ABI with pinned host buffers, the
host->device copy of messages/key and the device->host copy of all
signatures inside every timed step, streamed over two batch objects (step i
launches while step i-1's signatures copy back); `e2e.serial` is the same
one call at a time.  Verify throughput, the plain
one-signature-per-call path and the roofline of the dominant kernel
(k_leaves) ride along on the same JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 runs under torchrun as independent replicas (the path shards by request,
no collective): every rank signs its own 4096 messages, value sums the ranks.
"""
import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# many concurrent streams (serving, mixed-set graphs): 32 hardware queues,
# set before anything creates the CUDA context
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

SET = "sha256-128f-simple"
BATCH = 4096
MLEN = 64
SUBSET = 64
METRIC = "sign/s & verify/s, SHA2-128f, 1 GB300: batched+served vs plain; p50/p99 latency"
OPS_PER_CMP = 1384   # INT ops of one SHA-256 compression (64 rounds x 14 + 48 x 10 + 8)
# SHA-256 compressions per 128f operation, message hashing excluded (<1% at the
# message lengths used here): sign = FORS + d x (2^hp leaves + tree) + T_k,
# verify = FORS roots + T_k + d x (chains + T_len + auth path)
SIGN_CMP_128F = 113265
VERIFY_CMP_128F = 6400
KEYGEN_CMP_128F = 4567   # top-layer XMSS tree: 8 leaves x 570 + 7 H
# message hashing of a 64-B message at n = 16: PRF_msg 5 (HMAC) + H_msg 4
MSG_CMP_64B_SIGN = 9


def int_frac(signs, verifies, peak_ops):
    """Fraction of the measured SHA-256-mix integer peak that `signs`/s and
    `verifies`/s of SHA-256-128f-simple amount to."""
    return (signs * SIGN_CMP_128F + verifies * VERIFY_CMP_128F) * OPS_PER_CMP / peak_ops


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = []
        mx = 0.0
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for i, nm in enumerate(names):
                    if r[5 + i].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs(rank):
    import numpy as np
    import cuspx_gb300 as c
    rng = np.random.default_rng(20260 + rank)
    seed = rng.bytes(48)
    msgs = rng.integers(0, 256, size=(BATCH, MLEN), dtype=np.uint8)
    return seed, msgs


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the baseline lines."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        names = [ln.split(":", 1)[1].strip() for ln in out.splitlines() if ln.strip().startswith("Model name")]
        if names:
            return " / ".join(dict.fromkeys(names))
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu part")):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_baseline_port(seconds, verify=True):
    """The C restatement of the reference CPU path, all host cores, bounded."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import spx_oracle
    o = spx_oracle.Oracle(SET)
    threads = os.cpu_count() or 1
    done, secs = o.throughput(0, threads, MLEN, seconds)
    out = {"value": done / secs if secs else 0.0, "unit": "sign/s", "cores": threads, "kind": "port",
           "cpu_model": cpu_model(),
           "sample": "%d signatures of %d-B messages (%s) on %d threads in %.1f s, each worker its own key" %
                     (done, MLEN, SET, threads, secs),
           "signatures": done, "seconds": secs,
           "compressions_per_s": (done / secs if secs else 0.0) * (SIGN_CMP_128F + MSG_CMP_64B_SIGN)}
    if verify:
        vdone, vsecs = o.throughput(1, threads, MLEN, max(1.0, seconds / 4))
        out["verify_per_s"] = vdone / vsecs if vsecs else 0.0
    return out


def run_reference(args):
    """The reference arm.  A step is one bounded sample: 2 s of signing 64-B
    messages on every host core (about 670 signatures); ms_per_step is the
    measured wall time of a step and value the median signing rate."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    per_step, step_ms = [], []
    info = None
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        info = cpu_baseline_port(2.0, verify=False)
        if i >= args.warmup:
            per_step.append(info["value"])
            step_ms.append((time.perf_counter() - t0) * 1e3)
    value = statistics.median(per_step)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "sign/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms),
            "step": "one 2-s sample of signing on all host cores (%d signatures in the last)" % info["signatures"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded uniform random 64-B messages)",
            "config": {"workload": "batched SHA-256-128f-simple sign, 4096 x 64-B messages, one key",
                       "set": SET, "batch": BATCH, "mlen": MLEN,
                       "reference_code": "C restatement of the reference CPU path (oracle/spx_oracle.c); the "
                                         "reference's own sources are absent on the GPU host"},
            "cpu_baseline": {"value": value, "unit": "sign/s", "cores": info["cores"], "kind": "port",
                             "cpu_model": info["cpu_model"], "sample": info["sample"]},
            "e2e": {"value": value, "unit": "sign/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the uneven-mixed and verify-heavy workloads")
    ap.add_argument("--profile-case", type=int, default=0,
                    help="run one sign and one verify batch of this many messages (for ncu) and exit")
    ap.add_argument("--profile-set", default=SET)
    args = ap.parse_args()
    if args.profile_case:
        return profile_case(args.profile_case, args.profile_set)
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch
    import cuspx_gb300 as c

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    eng = c.Engine(local)
    sid = c.set_id(SET)
    z = c.set_sizes(sid)
    # roofline denominators: the SHA-256 round's pipe mix (7 ALU : 1 FMA), and
    # the ALU pipe alone (reported beside it)
    peak_ops, _ = c.int_peak(local, 8192, mix=1)
    peak_alu, _ = c.int_peak(local, 8192, mix=0)
    # dependent SHA-256 compressions by warps per SM: the latency of one
    # (1 warp) and how many warps the ALU pipe needs
    cmp_curve = {w: {"cmp_per_s": r, "ns_per_cmp": ns}
                 for w in (1, 4, 8, 16) for r, ns in [c.cmp_rate(w, local, 2048 if w <= 8 else 1024)]}
    # per-set launch mapping for this batch shape (autotuner, cached per GPU)
    from cuspx_gb300 import autotune
    tuned = {"sign": autotune.tune(eng, sid, c.OP_SIGN, count=BATCH, mlen=MLEN)[0],
             "verify": autotune.tune(eng, sid, c.OP_VERIFY, count=BATCH, mlen=MLEN)[0]}

    seed, msgs = make_inputs(rank)
    pks, sks = eng.keypair_batch(sid, [seed])
    pk, sk = pks[0], sks[0]
    slab = np.ascontiguousarray(msgs.reshape(-1))
    offs = np.arange(BATCH, dtype=np.uint64) * MLEN
    lens = np.full(BATCH, MLEN, dtype=np.uint64)
    kidx = np.zeros(BATCH, dtype=np.uint32)
    skb = np.frombuffer(sk, dtype=np.uint8).copy()
    pkb = np.frombuffer(pk, dtype=np.uint8).copy()

    # pinned host buffers for the end-to-end path
    def pinned(nbytes):
        return torch.empty(max(1, nbytes), dtype=torch.uint8, pin_memory=True).numpy()
    h_msgs = pinned(slab.nbytes); h_msgs[:] = slab
    h_offs = pinned(offs.nbytes).view(np.uint64); h_offs[:] = offs
    h_lens = pinned(lens.nbytes).view(np.uint64); h_lens[:] = lens
    h_kidx = pinned(kidx.nbytes).view(np.uint32); h_kidx[:] = kidx
    h_sk = pinned(skb.nbytes); h_sk[:] = skb
    h_sigs = pinned(BATCH * z["sig"])
    h_status = pinned(BATCH * 4).view(np.int32)

    sb = eng.batch(c.OP_SIGN, sid, BATCH, slab.nbytes, 1)
    vb = eng.batch(c.OP_VERIFY, sid, BATCH, slab.nbytes, 1)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2

    # ---- correctness gate: seeded 64-message subset against the oracle ----
    sb.upload(BATCH, h_sk, 1, h_kidx, h_msgs, slab.nbytes, h_offs, h_lens)
    sb.run()
    sb.download(h_sigs, None, h_status)
    assert (h_status == 0).all(), "sign status"
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import spx_oracle
    o = spx_oracle.Oracle(SET)
    rs = np.random.default_rng(64)
    subset = sorted(rs.choice(BATCH, SUBSET, replace=False).tolist())
    for i in subset:
        ref = o.sign(bytes(msgs[i]), sk)
        got = bytes(h_sigs[i * z["sig"]:(i + 1) * z["sig"]])
        assert got == ref, "signature %d differs from the CPU oracle" % i
    vb.upload(BATCH, pkb, 1, h_kidx, h_msgs, slab.nbytes, h_offs, h_lens, h_sigs)
    vb.run()
    vv = np.zeros(BATCH, dtype=np.int32)
    vb.download(None, None, vv)
    assert (vv == 0).all(), "verify rejected a valid signature"

    # ---- device-resident timing (value) ----
    for _ in range(args.warmup):
        sb.run(); vb.run()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    sign_ms, verify_ms = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        sb.run(); sb.sync(); sign_ms.append(sb.last_ms())
        flush.zero_()
        torch.cuda.synchronize()
        vb.run(); vb.sync(); verify_ms.append(vb.last_ms())
    barrier()
    wall = time.perf_counter() - t0
    ck = clocks.stop()
    sign_total = sum(sign_ms)
    verify_total = sum(verify_ms)
    if world > 1:
        t = torch.tensor([sign_total, verify_total], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        sign_total, verify_total = t.tolist()
    value = world * BATCH * args.steps / (sign_total / 1e3)
    verify_value = world * BATCH * args.steps / (verify_total / 1e3)

    # ---- per-kernel times (events around each kernel, same stream) ----
    sb.profile(True)
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        sb.run(); sb.sync()
    kern = sb.kernel_ms()
    sb.profile(False)
    vb.profile(True)
    vb.run(); vb.sync()
    vkern = vb.kernel_ms()
    vb.profile(False)
    tot = sum(m for _, m, _ in kern)
    leaves = [(m / n) for name, m, n in kern if name == "k_leaves"][0]
    P = dict(n=16, d=22, hp=3)
    leaf_ops = BATCH * P["d"] * (1 << P["hp"]) * leaf_units(SET) * OPS_PER_CMP
    achieved = leaf_ops / (leaves * 1e-3) / 1e12
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "k_leaves_sha256-128f_traffic.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            tj = json.load(f)
        traffic = tj.get("dram_bytes_per_launch_scaled_to_4096")

    # ---- verify at 16384 items (4 copies of the batch): batch parallelism
    # beside kernel quality -- the persistent kernel keeps ~4 warps per SM
    # busy per 600 items, and the ALU pipe needs ~8 warps per SM
    # (cuspx_cmp_rate) ----
    verify16k = None
    if rank == 0:
        big = 4 * BATCH
        vb4 = eng.batch(c.OP_VERIFY, sid, big, 4 * slab.nbytes, 1)
        vb4.upload(big, pkb, 1, np.zeros(big, dtype=np.uint32), np.tile(slab, 4), 4 * slab.nbytes,
                   np.arange(big, dtype=np.uint64) * MLEN, np.full(big, MLEN, dtype=np.uint64),
                   np.tile(h_sigs[:BATCH * z["sig"]], 4))
        t16 = []
        for i in range(4):
            flush.zero_()
            torch.cuda.synchronize()
            vb4.run(); vb4.sync()
            if i:
                t16.append(vb4.last_ms())
        vv4 = np.zeros(big, dtype=np.int32)
        vb4.download(None, None, vv4)
        vb4.close()
        v16 = big / (min(t16) / 1e3)
        verify16k = {"value": v16, "unit": "verify/s", "items": big, "ms_per_batch": min(t16),
                     "all_accept": bool((vv4 == 0).all()), "roofline_frac": int_frac(0, v16, peak_ops)}

    # ---- what the kernels execute, beside the model ----
    # The model counts the reference's structure at 1384 INT ops per
    # compression.  This engine skips two of its parts (the FORS secret PRF
    # and wots_sign's chain recomputation: ~6.5k of 113k compressions), and
    # the compiler issues fewer ALU instructions per compression than the
    # model's ops (ncu: ALU instructions of one k_leaves launch / its
    # compressions, profiles/k_leaves_sha256-128f_pipe.json).
    m128 = unit_model(SET)
    executed = {"sign_compressions": m128["executed_sign"] + MSG_CMP_64B_SIGN,
                "step_frac_of_mix_peak": value * (m128["executed_sign"] + MSG_CMP_64B_SIGN) * OPS_PER_CMP / peak_ops}
    pfile = os.path.join(ROOT, "profiles", "k_leaves_sha256-128f_pipe.json")
    if os.path.exists(pfile):
        with open(pfile) as f:
            pj = json.load(f)
        cmps = leaf_ops / OPS_PER_CMP   # compressions of one k_leaves launch
        executed["k_leaves_alu_instr_per_cmp"] = pj["alu_instr_per_cmp"]
        executed["k_leaves_alu_pipe_frac"] = cmps * pj["alu_instr_per_cmp"] / (leaves * 1e-3) / peak_alu
        executed["alu_source"] = "ALU-pipe instructions per compression from ncu (%s) x compressions/s of " \
                                 "k_leaves / the measured ALU-only peak" % pj.get("capture", "k_leaves")

    # ---- batched key generation (crypto_sign_seed_keypair per item) ----
    keygen = keygen_run(c, eng, sid, z, o, flush, args.steps, args.warmup, peak_ops) if rank == 0 else None

    # ---- end-to-end through the C ABI with host buffers ----
    # One call at a time: upload, run, download (which waits), per step.
    gate_digest = hashlib.sha256(h_sigs.tobytes()).hexdigest()
    serial_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        sb.upload(BATCH, h_sk, 1, h_kidx, h_msgs, slab.nbytes, h_offs, h_lens)
        sb.run()
        sb.download(h_sigs, None, h_status)
        s1 = time.perf_counter()
        if i >= args.warmup:
            serial_ms.append((s1 - s0) * 1e3)
    # Streamed (the e2e figure): two batches on their own streams with their
    # own pinned outputs; step i uploads and launches on batch i % 2 while
    # step i-1's signatures copy back.  A batch is synchronised before its
    # buffers are reused, so every step's host->device copy, kernels and
    # device->host copy of all its signatures fall inside the timed region.
    sb2 = eng.batch(c.OP_SIGN, sid, BATCH, slab.nbytes, 1)
    ring = [(sb, h_sigs, h_status), (sb2, pinned(BATCH * z["sig"]), pinned(BATCH * 4).view(np.int32))]

    def streamed(nsteps):
        pending = [False, False]
        for i in range(nsteps):
            b, hs, hst = ring[i % 2]
            if pending[i % 2]:
                b.sync()
            b.upload(BATCH, h_sk, 1, h_kidx, h_msgs, slab.nbytes, h_offs, h_lens)
            b.run()
            b.download_async(hs, None, hst)
            pending[i % 2] = True
        for j in (0, 1):
            if pending[j]:
                ring[j][0].sync()

    streamed(max(args.warmup, 2))
    barrier()
    s0 = time.perf_counter()
    streamed(args.steps)
    e2e_total = (time.perf_counter() - s0) * 1e3
    for _, hs, hst in ring:
        assert (hst == 0).all() and hashlib.sha256(hs.tobytes()).hexdigest() == gate_digest, \
            "streamed signatures differ from the checked batch"
    serial_total = sum(serial_ms)
    if world > 1:
        t = torch.tensor([e2e_total, serial_total], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_total, serial_total = t.tolist()
    e2e_value = world * BATCH * args.steps / (e2e_total / 1e3)
    sb2.close()
    h2d = slab.nbytes + skb.nbytes + offs.nbytes + lens.nbytes + kidx.nbytes
    d2h = BATCH * z["sig"] + BATCH * 4

    # ---- plain one-signature-per-call path (NIST api.h drop-in) ----
    plain = None
    if rank == 0:
        plain = plain_path(c)

    served = None
    if rank == 0 and not args.no_served:
        served = served_runs(c, eng, peak_ops, peak_alu)
    extra = {}
    if rank == 0 and not args.no_extra:
        extra["uneven_mixed"] = uneven_mixed(c, eng, peak_ops)
        extra["verify_heavy"] = verify_heavy(c, eng, peak_alu)
        extra["sign_sets_1024"] = sign_sets(c, eng, peak_alu, peak_ops)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_port(args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "sign/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sign_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded uniform random 64-B messages; one seeded keypair)",
            "config": {"workload": "batched SHA-256-128f-simple: 4096 x 64-B messages signed in one "
                                   "graph-launched batch, then verified in one batch",
                       "set": SET, "batch": BATCH, "mlen": MLEN, "parallelism": "replicas" if world > 1 else "1gpu",
                       "l2": "256 MiB buffer written between timed steps (L2 is 129 MB)",
                       "subset_check": "%d seeded signatures byte-identical to the CPU oracle" % SUBSET,
                       "mapping": tuned},
            "verify": {"value": verify_value, "unit": "verify/s", "ms_per_batch": verify_total / args.steps,
                       "roofline_frac": int_frac(0, verify_value, peak_ops)},
            "verify_16384": verify16k,
            "cmp_rate_by_warps_per_sm": cmp_curve,
            "step_roofline_frac": int_frac(value, 0, peak_ops),
            "compressions_per_s": value * (SIGN_CMP_128F + MSG_CMP_64B_SIGN),
            "executed": executed,
            "keygen": keygen,
            "e2e": {"value": e2e_value, "unit": "sign/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_total / args.steps,
                    "mode": "streamed: two batches, step i launched while step i-1's signatures copy back",
                    "serial": {"value": world * BATCH * args.steps / (serial_total / 1e3),
                               "ms_per_step": serial_total / args.steps,
                               "mode": "one call at a time: upload, run, download per step"}},
            "gpu_launches": (5 + 3) * args.steps,
            "kernels_ms": {name: round(m / n, 4) for name, m, n in kern},
            "verify_kernels_ms": {name: round(m / n, 4) for name, m, n in vkern},
            "roofline": {"bound": "int_alu", "kernel": "k_leaves", "achieved": achieved,
                         "peak": peak_ops / 1e12, "unit": "Tops/s", "frac": achieved / (peak_ops / 1e12),
                         "traffic": traffic,
                         "work": "%d compressions x %d INT ops per launch" %
                                 (BATCH * 176 * leaf_units(SET), OPS_PER_CMP),
                         "peak_source": "measured in this run on all SMs: SHA-256 round mix, 7 ALU ops "
                                        "(SHF/LOP3/IADD3) to 1 IMAD on the FMA pipe (cuspx_int_peak_mix 1)",
                         "peak_alu_only": peak_alu / 1e12,
                         "share_of_step": leaves / (tot / 3)},
            "clocks": ck,
            "wall_s_timed": wall,
        }
        if plain:
            line["plain"] = plain
            line["batched_vs_plain"] = value / plain["sign_per_s"] if plain["sign_per_s"] else None
        line.update(extra)
        if served:
            line.update(served)
            ok = [p for p in served["served_128f"] if p["sign_p99_ms"] < 20.0 and p["wrong_verdicts"] == 0]
            if ok and plain:
                best = max(ok, key=lambda p: p["sign_per_s"] + p["verify_per_s"])
                line["served_vs_plain"] = {
                    "sign": best["sign_per_s"] / plain["sign_per_s"],
                    "verify": best["verify_per_s"] / plain["verify_per_s"],
                    "at_rate": best["rate"], "sign_p99_ms": best["sign_p99_ms"]}
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    sb.close(); vb.close(); eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def keygen_run(c, eng, sid, z, oracle, flush, steps, warmup, peak_ops):
    """4096 SHA-256-128f keypairs from seeded 48-byte seeds in one
    graph-launched batch; three are byte-compared with the oracle's
    crypto_sign_seed_keypair before timing."""
    import numpy as np
    import torch
    rng = np.random.default_rng(4242)
    seeds = rng.integers(0, 256, size=(BATCH, z["seed"]), dtype=np.uint8)
    kb = eng.batch(c.OP_KEYGEN, sid, BATCH)
    kb.upload(BATCH, np.ascontiguousarray(seeds.reshape(-1)))
    kb.run()
    sk = np.zeros(BATCH * z["sk"], dtype=np.uint8)
    pk = np.zeros(BATCH * z["pk"], dtype=np.uint8)
    kb.download(sk, pk)
    for i in (0, 1, BATCH - 1):
        rpk, rsk = oracle.seed_keypair(bytes(seeds[i]))
        assert bytes(sk[i * z["sk"]:(i + 1) * z["sk"]]) == rsk, "keypair %d differs from the CPU oracle" % i
        assert bytes(pk[i * z["pk"]:(i + 1) * z["pk"]]) == rpk, "keypair %d differs from the CPU oracle" % i
    for _ in range(warmup):
        kb.run()
    kb.sync()
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        kb.run(); kb.sync(); ms.append(kb.last_ms())
    kb.close()
    tot = sum(ms)
    v = BATCH * steps / (tot / 1e3)
    return {"value": v, "unit": "keypair/s", "ms_per_batch": tot / steps, "batch": BATCH,
            "subset_check": "3 keypairs byte-identical to the CPU oracle",
            "roofline_frac": v * KEYGEN_CMP_128F * OPS_PER_CMP / peak_ops}


def stream_frac(c, r, sids, wall, peak_mix, peak_alu):
    """Fraction of the GPU's integer peak that a served stream's completed work
    amounts to: per set, signs x sign units + verifies x verify units + the
    message hashing units of the requests (unit_model, msg_units), each hash
    against its own peak (SHA-256: the round mix; Keccak: the ALU pipe)."""
    t = 0.0
    for i, sid in enumerate(sids):
        m = unit_model(c.set_name(sid))
        units = r["set_sign_done"][i] * m["sign"] + r["set_verify_done"][i] * m["verify"] + r["set_msg_units"][i]
        t += units * m["ops_per_unit"] / (peak_alu if m["hash"] == "shake256" else peak_mix)
    return t / wall if wall > 0 else 0.0


def check_samples(c, samples, keys):
    """Byte-compare the load generator's sampled signatures with the oracle
    (in parallel threads; the oracle releases the GIL)."""
    import concurrent.futures
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import spx_oracle

    def one(smp):
        sid, kid, st, msg, sig = smp
        return st == 0 and sig == spx_oracle.Oracle(c.set_name(sid)).sign(msg, keys[sid][kid])
    with concurrent.futures.ThreadPoolExecutor(min(16, os.cpu_count() or 1)) as ex:
        return all(ex.map(one, samples))


def served_runs(c, eng, peak_ops, peak_alu, seconds=2.0):
    """Open-loop Poisson streams through the serving loop (cuspx_serve_*).

    served_128f: SHA-256-128f-simple only, 30% sign / 70% verify, 64 resident
    keys, 16..1024-B messages, 10% of verifies corrupted -- the stream the
    >= 3x-plain / p99 < 20 ms target is stated for.
    served_stream: 70% verify / 30% sign over {SHA-256-128f, SHA-256-192f,
    SHAKE-256-256f} (simple), 1024 resident keys, log-uniform 16 B..1 MiB.
    """
    import numpy as np
    rng = np.random.default_rng(555)
    out = {}
    sid = c.set_id(SET)
    z = c.set_sizes(sid)
    seeds = [rng.bytes(z["seed"]) for _ in range(64)]
    _, sks = eng.keypair_batch(sid, seeds)
    srv = c.Server(eng, max_batch=1024, max_inflight=3, window_us=1000)
    srv.add_keys(sid, sks)
    for op in (c.OP_SIGN, c.OP_VERIFY):
        srv.prepare(op, sid)   # launch slots exist before the first timed request
    pts = []
    # 300k and 400k req/s offered are past what the GPU can serve at this mix
    # (~430k req/s of pure compute): they show the served roofline fraction
    for rate in (5e3, 20e3, 50e3, 100e3, 200e3, 300e3, 400e3):
        r = srv.loadgen(rate, seconds, [sid], 64, verify_frac=0.7, min_len=16, max_len=1024, corrupt_frac=0.1,
                        seed=int(rate), pool=512)
        pts.append({"rate": rate, "sign_per_s": r["sign_throughput"], "verify_per_s": r["verify_throughput"],
                    "sign_p50_ms": r["sign_p50_us"] / 1e3, "sign_p99_ms": r["sign_p99_us"] / 1e3,
                    "verify_p50_ms": r["verify_p50_us"] / 1e3, "verify_p99_ms": r["verify_p99_us"] / 1e3,
                    "completed": r["completed"], "refused": r["refused"], "wrong_verdicts": r["wrong_verdicts"],
                    "mean_batch": r["mean_batch"],
                    "roofline_frac": int_frac(r["sign_throughput"], r["verify_throughput"], peak_ops)})
    srv.close()
    out["served_128f"] = pts
    names = ["sha256-128f-simple", "sha256-192f-simple", "shake256-256f-simple"]
    sids = [c.set_id(n) for n in names]
    # admission: device bytes of pending plus in-flight requests within 2 GiB,
    # and at most 25 ms of estimated GPU work queued or in flight (requests
    # beyond either are refused at submission); a launch carries at most
    # 10 ms of work, so a batch of SHAKE-256-256f signs stays short.  At
    # 200k req/s offered this holds the <= 64 KiB p99 to tens of ms (no
    # limits: 150-170 ms; 50 ms / 20 ms: 50-85 ms), at the price of smaller
    # launches: ~25% fewer signs/s at saturation, verifies/s unchanged.
    budget, queue_ms, launch_ms = 2 << 30, 25.0, 10.0
    srv = c.Server(eng, max_batch=1024, max_inflight=3, window_us=1000, mem_budget=budget, max_queue_ms=queue_ms,
                   max_launch_ms=launch_ms)
    per = 1024 // len(sids) + 1
    stream_keys = {}
    for s2 in sids:
        z2 = c.set_sizes(s2)
        _, sk2 = eng.keypair_batch(s2, [rng.bytes(z2["seed"]) for _ in range(per)])
        stream_keys[s2] = sk2
        srv.add_keys(s2, sk2)
        for op in (c.OP_SIGN, c.OP_VERIFY):
            srv.prepare(op, s2)
    pts = []
    for rate in (5e3, 20e3, 50e3, 100e3, 200e3):
        r = srv.loadgen(rate, seconds, sids, per, verify_frac=0.7, min_len=16, max_len=1 << 20, corrupt_frac=0.0,
                        seed=7 + int(rate), pool=48, sample_every=64, sample_max=12,
                        arena_bytes=12 * ((1 << 20) + 50000))
        ms = lambda v: [round(x / 1e3, 3) for x in v]
        frac = stream_frac(c, r, sids, r["wall_s"], peak_ops, peak_alu)
        sample_ok = check_samples(c, r["samples"], stream_keys)
        pts.append({"rate": rate, "sign_per_s": r["sign_throughput"], "verify_per_s": r["verify_throughput"],
                    "sign_p50_ms": r["sign_p50_us"] / 1e3, "sign_p99_ms": r["sign_p99_us"] / 1e3,
                    "verify_p50_ms": r["verify_p50_us"] / 1e3, "verify_p99_ms": r["verify_p99_us"] / 1e3,
                    "by_length_le1KiB_le64KiB_gt64KiB": {
                        "sign_p50_ms": ms(r["sign_p50_bucket_us"]), "sign_p99_ms": ms(r["sign_p99_bucket_us"]),
                        "verify_p50_ms": ms(r["verify_p50_bucket_us"]),
                        "verify_p99_ms": ms(r["verify_p99_bucket_us"])},
                    "completed": r["completed"], "refused": r["refused"], "wrong_verdicts": r["wrong_verdicts"],
                    "mean_batch": r["mean_batch"], "launch_ms_mean": r["launch_ms_mean"],
                    "launch_ms_max": r["launch_ms_max"], "roofline_frac": frac,
                    "oracle_sample": {"signatures": len(r["samples"]), "identical": sample_ok}})
    srv.close()
    out["served_stream"] = {"sets": names, "keys": per * len(sids), "lengths": "log-uniform 16 B..1 MiB",
                            "mem_budget_bytes": budget, "max_queue_ms": queue_ms, "max_launch_ms": launch_ms,
                            "oracle_sample": "1 in 64 timed signs kept (up to 12 per point), byte-compared "
                                             "with the CPU oracle",
                            "points": pts}
    return out


# (n, h, d, a, k) per size (params.h:33-79)
SIZES = {"128s": (16, 63, 7, 12, 14), "128f": (16, 66, 22, 6, 33), "192s": (24, 63, 7, 14, 17),
         "192f": (24, 66, 22, 8, 33), "256s": (32, 64, 8, 14, 22), "256f": (32, 68, 17, 9, 35)}


def expected_digit_sum(n, samples=20000):
    """E[sum of the len = 2n + 3 WOTS+ digits] of a uniformly random message
    (chain_lengths, wots.cu:84-166: 2n message digits, then the checksum
    sum(15 - d) shifted left by 4 and read as its three top 4-bit digits)."""
    import numpy as np
    d = np.random.default_rng(12345).integers(0, 16, size=(samples, 2 * n))
    csum = (15 - d).sum(axis=1)
    return float(d.sum(axis=1).mean() + ((csum >> 8) & 15).mean() + ((csum >> 4) & 15).mean() +
                 (csum & 15).mean())


def unit_model(name):
    """Hash units (SHA-256 compressions, or Keccak-f[1600] permutations for
    SHAKE sets) of one operation of a parameter set, counted the way the
    reference's CPU path runs it, message hashing excluded:
      sign   = seed state (SHA-256) + FORS (per tree: the signature's secret
               PRF, 2^a leaves of PRF + F, 2^a - 1 H; then T_k) + per layer
               wots_sign (len PRF + sum of digits F) and a treehash of 2^h'
               leaves (len (PRF + 15 F) + T_len) and 2^h' - 1 H
      verify = seed state + FORS (per tree F + a H; T_k) + per layer
               sum of (15 - digit) F, T_len and h' H
    (sign.cu:1924-1994, :3048-3121; fors.cu:107-143, :596-631; wots.cu).
    The digit sums are their expectation over random messages.  A thash over
    m n-byte blocks is (22 + m n + 9) / 64 compressions after the PUB_SEED
    midstate, or (n + 32 + m n) / 136 + 1 permutations; robust adds the mask
    (ceil(m n / 32) MGF1 blocks of (n + 26 + 9) / 64 compressions, or
    ceil(m n / 136) squeezing permutations).  `executed_sign` drops what this
    engine does not recompute: the FORS secret PRF (taken from its leaf) and
    wots_sign (the signing leaf's chain values are recorded)."""
    parts = name.split("-")
    shake, robust = parts[0] == "shake256", parts[2] == "robust"
    n, h, d, a, k = SIZES[parts[1]]
    hp, ln = h // d, 2 * n + 3

    def th(m):
        if shake:
            return (n + 32 + m * n) // 136 + 1 + (-(-m * n // 136) if robust else 0)
        return (22 + m * n + 9 + 63) // 64 + (-(-m * n // 32) * ((n + 26 + 9 + 63) // 64) if robust else 0)

    F, H, prf = th(1), th(2), 1
    seed = 0 if shake else 1
    leaf = ln * (prf + 15 * F) + th(ln)
    xmss = (1 << hp) * leaf + ((1 << hp) - 1) * H
    sign_fixed = seed + k * (prf + (1 << a) * (prf + F) + ((1 << a) - 1) * H) + th(k) + d * xmss
    verify_fixed = seed + k * (F + a * H) + th(k) + d * (th(ln) + hp * H)
    e = expected_digit_sum(n)
    wots_sign = d * (ln * prf + e * F)
    return {"unit": "perm" if shake else "cmp", "ops_per_unit": 4560 if shake else OPS_PER_CMP,
            "sign": sign_fixed + wots_sign, "verify": verify_fixed + d * (ln * 15 - e) * F,
            "sign_fixed": sign_fixed, "verify_fixed": verify_fixed, "wots_sign": wots_sign,
            "verify_chain_steps": d * (ln * 15 - e), "F": F,
            "executed_sign": sign_fixed - k * prf, "hash": "shake256" if shake else "sha256"}


def msg_units(name, op, mlen):
    """Hash units of the message hashing of one request: H_msg for verify,
    PRF_msg and H_msg for sign (hash_sha256.cu:99-145, :200-262;
    hash_shake256.cu:64-77, :96-130)."""
    parts = name.split("-")
    n, h, d, a, k = SIZES[parts[1]]
    hp = h // d
    dgst = (k * a + 7) // 8 + (hp * (d - 1) + 7) // 8 + (hp + 7) // 8
    if parts[0] == "shake256":
        hm = (3 * n + mlen) // 136 + 1
        return hm if op == "verify" else hm + (2 * n + mlen) // 136 + 1
    hm = (3 * n + mlen + 9 + 63) // 64 + (dgst + 31) // 32
    return hm if op == "verify" else hm + 3 + (n + mlen + 9 + 63) // 64


def leaf_units(name):
    """Hash units (SHA-256 compressions or Keccak-f permutations) of one XMSS
    leaf of a simple set: len chains of PRF + 15 F (one unit each at these
    widths) and T_len over the len chain ends.  SHA-256 runs T_len after the
    PUB_SEED midstate on ADRS_c (22 B) || values || padding (9 B min);
    SHAKE-256 absorbs PUB_SEED || ADRS (32 B) || values at rate 136."""
    n = {"128": 16, "192": 24, "256": 32}[name.split("-")[1][:3]]
    ln = 2 * n + 3
    if name.startswith("sha256"):
        t = (22 + ln * n + 9 + 63) // 64
    else:
        t = (n + 32 + ln * n) // 136 + 1
    return ln * 16 + t


def sign_sets(c, eng, peak_alu, peak_mix, count=1024, mlen=256):
    """Sign throughput of other simple sets at `count` signatures of `mlen`
    random bytes (one key each, graph-launched batches), with k_leaves'
    fraction of the integer peak for its hash: the SHA-256-round mix for
    SHA-256, the ALU pipe alone for Keccak-f (which puts nothing on the FMA
    pipe).  One signature per set is byte-compared with the CPU oracle."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import spx_oracle
    hypertree = {"128f": (66, 22), "192f": (66, 22), "256f": (68, 17)}   # (h, d), params.h
    out = {}
    for name in ("sha256-192f-simple", "sha256-256f-simple", "shake256-128f-simple", "shake256-256f-simple"):
        sid = c.set_id(name)
        z = c.set_sizes(sid)
        o = spx_oracle.Oracle(name)
        rng = np.random.default_rng(123)
        _, sks = eng.keypair_batch(sid, [rng.bytes(z["seed"])])
        sk = bytes(sks[0])
        msgs = rng.integers(0, 256, size=(count, mlen), dtype=np.uint8)
        slab = np.ascontiguousarray(msgs.reshape(-1))
        offs = np.arange(count, dtype=np.uint64) * mlen
        lens = np.full(count, mlen, dtype=np.uint64)
        kidx = np.zeros(count, dtype=np.uint32)
        sb = eng.batch(c.OP_SIGN, sid, count, slab.nbytes, 1)
        sb.upload(count, np.frombuffer(sk, dtype=np.uint8), 1, kidx, slab, slab.nbytes, offs, lens)
        sb.run()
        sigs = np.zeros(count * z["sig"], dtype=np.uint8)
        sb.download(sigs)
        ok = bytes(sigs[:z["sig"]]) == o.sign(bytes(msgs[0]), sk)
        sb.run(); sb.sync()
        ms = []
        for _ in range(2):
            sb.run(); sb.sync(); ms.append(sb.last_ms())
        sb.profile(True)
        sb.run(); sb.sync()
        km = {k: m / n for k, m, n in sb.kernel_ms()}
        sb.profile(False)
        sb.close()
        h, d = hypertree[name.split("-")[1]]
        units = count * d * (1 << (h // d)) * leaf_units(name)
        shake = name.startswith("shake")
        ops = units * (4560 if shake else OPS_PER_CMP)
        leaves = km.get("k_leaves")
        peak = peak_alu if shake else peak_mix
        out[name] = {"sign_per_s": count / (min(ms) / 1e3), "ms_per_batch": min(ms),
                     "k_leaves_ms": leaves,
                     "k_leaves_frac": ops / (leaves * 1e-3) / peak if leaves else None,
                     "peak": "alu_only" if shake else "sha256_mix", "oracle_first_sig_agrees": ok}
    return out


def uneven_mixed(c, eng, peak_mix, reps=3):
    """Uneven batch: 256 distinct keypairs (128 per set), 2048 sign requests,
    lengths floor(exp(U(ln 1, ln 65536))) B, sets SHA-256-128s-simple and
    SHA-256-192f-robust drawn 50/50, one graph launch; each set's mapping is
    tuned on its own part of this very batch (its count and lengths) and
    installed in the library for that batch size."""
    import numpy as np
    from cuspx_gb300 import autotune
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import spx_oracle
    names = ["sha256-128s-simple", "sha256-192f-robust"]
    sids = [c.set_id(n) for n in names]
    rng = np.random.default_rng(33)
    keys = {}
    tuned = {}
    for n, sid in zip(names, sids):
        z = c.set_sizes(sid)
        pks, sks = eng.keypair_batch(sid, [rng.bytes(z["seed"]) for _ in range(128)])
        keys[sid] = sks
    set_ids, sks, msgs = [], [], []
    for _ in range(2048):
        sid = sids[int(rng.integers(0, 2))]
        L = int(np.floor(np.exp(rng.uniform(0.0, np.log(65536.0)))))
        set_ids.append(sid)
        sks.append(keys[sid][int(rng.integers(0, 128))])
        msgs.append(rng.bytes(L))
    for n, sid in zip(names, sids):
        part = [m for s2, m in zip(set_ids, msgs) if s2 == sid]
        tuned[n] = autotune.tune(eng, sid, c.OP_SIGN, msgs=part, use_cache=False, passes=1)[0]
    ms = c.MixedSigner(eng)
    sigs, st, _ = ms.sign(set_ids, sks, msgs)
    times = []
    for _ in range(reps):
        _, _, dev = ms.sign(set_ids, sks, msgs)
        times.append(dev)
    ms.close()
    # byte-compare a seeded subset against the CPU oracle
    chk = [int(i) for i in np.random.default_rng(34).choice(2048, 6, replace=False)]
    ok = all(st == 0)
    for i in chk:
        o = spx_oracle.Oracle(c.set_name(set_ids[i]))
        ok &= sigs[i] == o.sign(msgs[i], sks[i])
    best = min(times)
    units = sum(unit_model(c.set_name(s2))["sign"] + msg_units(c.set_name(s2), "sign", len(m))
                for s2, m in zip(set_ids, msgs))
    return {"workload": "2048 sign requests, 256 keys, lengths log-uniform 1 B..64 KiB, sets %s 50/50, one "
                        "graph launch" % "+".join(names),
            "sign_per_s": 2048 / (best / 1e3), "ms_per_launch": best, "tuning": tuned,
            "tuned_on": "each set's own part of this batch (its count and message lengths)",
            "compressions_per_launch": units,
            "roofline_frac": units * OPS_PER_CMP / (best * 1e-3) / peak_mix,
            "oracle_subset_identical": bool(ok), "subset": len(chk)}


def verify_heavy(c, eng, peak_alu, reps=3):
    """16384 SHAKE-256-256f signatures (simple and robust) over 256-B
    messages, 10% with one seeded random byte xored with a nonzero byte; every
    verdict must be the expected one and a subset must match the CPU oracle."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import spx_oracle
    out = {}
    for name in ("shake256-256f-simple", "shake256-256f-robust"):
        sid = c.set_id(name)
        z = c.set_sizes(sid)
        rng = np.random.default_rng(44)
        count = 16384
        pks, sks = eng.keypair_batch(sid, [rng.bytes(z["seed"]) for _ in range(16)])
        kidx = (np.arange(count) % 16).astype(np.uint32)
        msgs = rng.integers(0, 256, size=(count, 256), dtype=np.uint8)
        slab = np.ascontiguousarray(msgs.reshape(-1))
        offs = np.arange(count, dtype=np.uint64) * 256
        lens = np.full(count, 256, dtype=np.uint64)
        skb = np.frombuffer(b"".join(sks), dtype=np.uint8).copy()
        pkb = np.frombuffer(b"".join(pks), dtype=np.uint8).copy()
        sb = eng.batch(c.OP_SIGN, sid, count, slab.nbytes, 16)
        sb.upload(count, skb, 16, kidx, slab, slab.nbytes, offs, lens)
        sb.run()
        sigs = np.zeros(count * z["sig"], dtype=np.uint8)
        st = np.zeros(count, dtype=np.int32)
        sb.download(sigs, None, st)
        sb.close()
        bad = rng.random(count) < 0.10
        for i in np.nonzero(bad)[0]:
            pos = int(rng.integers(0, z["sig"]))
            sigs[i * z["sig"] + pos] ^= np.uint8(int(rng.integers(1, 256)))
        vb = eng.batch(c.OP_VERIFY, sid, count, slab.nbytes, 16)
        vb.upload(count, pkb, 16, kidx, slab, slab.nbytes, offs, lens, sigs)
        times = []
        for _ in range(reps + 1):
            vb.run()
            vb.sync()
            times.append(vb.last_ms())
        v = np.zeros(count, dtype=np.int32)
        vb.download(None, None, v)
        vb.close()
        expect = np.where(bad, -1, 0)
        o = spx_oracle.Oracle(name)
        sub = [int(i) for i in np.random.default_rng(45).choice(count, 48, replace=False)] + \
              [int(i) for i in np.nonzero(bad)[0][:16]]
        oracle_ok = all(o.verify(sigs[i * z["sig"]:(i + 1) * z["sig"]].tobytes(), msgs[i].tobytes(),
                                 pks[int(kidx[i])]) == int(v[i]) for i in sub)
        best = min(times[1:])
        perms = count * (unit_model(name)["verify"] + msg_units(name, "verify", 256))
        out[name] = {"verify_per_s": count / (best / 1e3), "ms_per_launch": best, "corrupted": int(bad.sum()),
                     "permutations_per_s": perms / (best * 1e-3),
                     "roofline_frac": perms * 4560 / (best * 1e-3) / peak_alu,
                     "all_verdicts_expected": bool((v == expect).all()), "oracle_subset_agrees": bool(oracle_ok),
                     "oracle_subset": len(sub)}
    return out


def profile_case(count, setname):
    """One sign batch and one verify batch of `count` 64-B messages, kernels
    launched directly on the batch stream (no graph): the small case that
    ncu captures."""
    import numpy as np
    import cuspx_gb300 as c
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import spx_oracle
    eng = c.Engine(0)
    sid = c.set_id(setname)
    z = c.set_sizes(sid)
    rng = np.random.default_rng(11)
    # key from the CPU oracle, so the first GPU launches are the signing ones
    pk0, sk0 = spx_oracle.Oracle(setname).seed_keypair(rng.bytes(z["seed"]))
    pks, sks = [pk0], [sk0]
    msgs = [rng.bytes(MLEN) for _ in range(count)]
    slab, offs, lens = c.pack_messages(msgs)
    kidx = np.zeros(count, dtype=np.uint32)
    sb = eng.batch(c.OP_SIGN, sid, count, len(slab), 1)
    sb.profile(True)
    sb.upload(count, sks[0], 1, kidx, slab, len(slab), offs, lens)
    sb.run()
    sigs = np.zeros(count * z["sig"], dtype=np.uint8)
    st = np.zeros(count, dtype=np.int32)
    sb.download(sigs, None, st)
    vb = eng.batch(c.OP_VERIFY, sid, count, len(slab), 1)
    vb.profile(True)
    vb.upload(count, pks[0], 1, kidx, slab, len(slab), offs, lens, sigs)
    vb.run()
    vv = np.zeros(count, dtype=np.int32)
    vb.download(None, None, vv)
    ok = bool((st == 0).all() and (vv == 0).all())
    # the two roofline calibration kernels, short, after the batches, so a
    # capture can read their pipe split next to the hash kernels'
    peaks = {"int_peak_mix%d" % mix: round(c.int_peak(0, 256, mix=mix)[0] / 1e12, 3) for mix in (0, 1)}
    print(json.dumps({"profile_case": setname, "count": count, "ok": ok,
                      "sign_kernels_ms": {k: round(m, 3) for k, m, _ in sb.kernel_ms()},
                      "verify_kernels_ms": {k: round(m, 3) for k, m, _ in vb.kernel_ms()}, **peaks}))
    sb.close(); vb.close(); eng.close()
    return 0 if ok else 1


def plain_path(c):
    """The plain configuration: one keypair, 16 messages of 32..1024 B,
    keypair/sign/verify one call at a time through the NIST api.h drop-in
    library."""
    import ctypes
    import numpy as np
    L = ctypes.CDLL(c.dropin_path(SET))
    L.crypto_sign_signature.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_char_p,
                                        ctypes.c_size_t, ctypes.c_char_p]
    L.crypto_sign_verify.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t,
                                     ctypes.c_char_p]
    L.crypto_sign_seed_keypair.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p]
    rng = np.random.default_rng(7)
    seed = rng.bytes(48)
    pk = ctypes.create_string_buffer(32)
    sk = ctypes.create_string_buffer(64)
    assert L.crypto_sign_seed_keypair(pk, sk, seed) == 0   # context creation and first launch
    kp_lat = []
    for _ in range(5):
        t0 = time.perf_counter()
        assert L.crypto_sign_seed_keypair(pk, sk, seed) == 0
        kp_lat.append((time.perf_counter() - t0) * 1e3)
    kp_ms = statistics.median(kp_lat)
    msgs = [rng.bytes(int(x)) for x in rng.integers(32, 1025, size=16)]
    sig = ctypes.create_string_buffer(17088)
    sl = ctypes.c_size_t()
    L.crypto_sign_signature(sig, ctypes.byref(sl), msgs[0], len(msgs[0]), sk.raw)   # warm the path
    s_lat, v_lat = [], []
    for m in msgs:
        t0 = time.perf_counter()
        assert L.crypto_sign_signature(sig, ctypes.byref(sl), m, len(m), sk.raw) == 0
        t1 = time.perf_counter()
        assert L.crypto_sign_verify(sig.raw, sl.value, m, len(m), pk.raw) == 0
        t2 = time.perf_counter()
        s_lat.append((t1 - t0) * 1e3)
        v_lat.append((t2 - t1) * 1e3)
    return {"workload": "1 key, 16 messages 32..1024 B, one crypto_sign_signature / crypto_sign_verify "
                        "call at a time through libspx_%s.so" % SET,
            "sign_per_s": 1e3 * len(s_lat) / sum(s_lat), "verify_per_s": 1e3 * len(v_lat) / sum(v_lat),
            "sign_ms_p50": statistics.median(s_lat), "verify_ms_p50": statistics.median(v_lat),
            "keypair_ms": kp_ms, "keypair_note": "median of 5 calls after a first (context-creating) call",
            "threads8": threaded_dropin(L, sk.raw, pk.raw, msgs)}


def threaded_dropin(L, sk, pk, msgs, nthreads=8, seconds=1.0):
    """The same drop-in called from 8 host threads at once, each looping over
    crypto_sign_signature (then crypto_sign_verify) for about a second:
    concurrent calls share launches.  Python threads run the calls in
    parallel because ctypes releases the GIL during each call."""
    import ctypes
    import threading

    def run(fn):
        counts = [0] * nthreads
        barrier = threading.Barrier(nthreads + 1)
        stop = [False]

        def worker(t):
            sig = ctypes.create_string_buffer(17088)
            sl = ctypes.c_size_t()
            barrier.wait()
            i = t
            while not stop[0]:
                fn(sig, sl, msgs[i % len(msgs)])
                counts[t] += 1
                i += 1

        ths = [threading.Thread(target=worker, args=(t,)) for t in range(nthreads)]
        for th in ths:
            th.start()
        barrier.wait()
        t0 = time.perf_counter()
        time.sleep(seconds)
        stop[0] = True
        for th in ths:
            th.join()
        return sum(counts) / (time.perf_counter() - t0)

    sigs = {}
    for m in msgs:
        sig = ctypes.create_string_buffer(17088)
        sl = ctypes.c_size_t()
        L.crypto_sign_signature(sig, ctypes.byref(sl), m, len(m), sk)
        sigs[m] = sig.raw
    sign_rate = run(lambda sig, sl, m: L.crypto_sign_signature(sig, ctypes.byref(sl), m, len(m), sk))
    verify_rate = run(lambda sig, sl, m: L.crypto_sign_verify(sigs[m], 17088, m, len(m), pk))
    return {"threads": nthreads, "sign_per_s": sign_rate, "verify_per_s": verify_rate,
            "note": "api.h calls from 8 threads at once; concurrent one-shot calls are combined into shared launches"}


if __name__ == "__main__":
    sys.exit(main())
