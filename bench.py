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


def cpu_baseline_port(seconds):
    """The C restatement of the reference CPU path, all host cores, bounded."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import spx_oracle
    o = spx_oracle.Oracle(SET)
    threads = os.cpu_count() or 1
    done, secs = o.throughput(0, threads, MLEN, seconds)
    vdone, vsecs = o.throughput(1, threads, MLEN, max(1.0, seconds / 4))
    return {"value": done / secs if secs else 0.0, "unit": "sign/s", "cores": threads, "kind": "port",
            "sample": "%d signatures of %d-B messages (%s) on %d threads in %.1f s, each worker its own key" %
                      (done, MLEN, SET, threads, secs),
            "verify_per_s": vdone / vsecs if vsecs else 0.0}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    per_step = []
    info = None
    for i in range(args.warmup + args.steps):
        sample_s = 2.0
        info = cpu_baseline_port(sample_s)
        if i >= args.warmup:
            per_step.append(info["value"])
    value = statistics.median(per_step)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "sign/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * BATCH / value if value else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded uniform random 64-B messages)",
            "config": {"workload": "batched SHA-256-128f-simple sign, 4096 x 64-B messages, one key",
                       "set": SET, "batch": BATCH, "mlen": MLEN,
                       "reference_code": "C restatement of the reference CPU path (oracle/spx_oracle.c); the "
                                         "reference's own sources are absent on the GPU host"},
            "cpu_baseline": {"value": value, "unit": "sign/s", "cores": info["cores"], "kind": "port",
                             "sample": info["sample"]},
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
        served = served_runs(c, eng, peak_ops)
    extra = {}
    if rank == 0 and not args.no_extra:
        extra["uneven_mixed"] = uneven_mixed(c, eng)
        extra["verify_heavy"] = verify_heavy(c, eng)
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
            "step_roofline_frac": int_frac(value, 0, peak_ops),
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


def served_runs(c, eng, peak_ops, seconds=2.0):
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
    srv = c.Server(eng, max_batch=1024, max_inflight=3, window_us=1000, mem_budget=24 << 30)
    per = 1024 // len(sids) + 1
    for s2 in sids:
        z2 = c.set_sizes(s2)
        _, sk2 = eng.keypair_batch(s2, [rng.bytes(z2["seed"]) for _ in range(per)])
        srv.add_keys(s2, sk2)
        for op in (c.OP_SIGN, c.OP_VERIFY):
            srv.prepare(op, s2)
    pts = []
    for rate in (5e3, 20e3, 50e3, 100e3, 200e3):
        r = srv.loadgen(rate, seconds, sids, per, verify_frac=0.7, min_len=16, max_len=1 << 20, corrupt_frac=0.0,
                        seed=7 + int(rate), pool=48)
        ms = lambda v: [round(x / 1e3, 3) for x in v]
        pts.append({"rate": rate, "sign_per_s": r["sign_throughput"], "verify_per_s": r["verify_throughput"],
                    "sign_p50_ms": r["sign_p50_us"] / 1e3, "sign_p99_ms": r["sign_p99_us"] / 1e3,
                    "verify_p50_ms": r["verify_p50_us"] / 1e3, "verify_p99_ms": r["verify_p99_us"] / 1e3,
                    "by_length_le1KiB_le64KiB_gt64KiB": {
                        "sign_p50_ms": ms(r["sign_p50_bucket_us"]), "sign_p99_ms": ms(r["sign_p99_bucket_us"]),
                        "verify_p50_ms": ms(r["verify_p50_bucket_us"]),
                        "verify_p99_ms": ms(r["verify_p99_bucket_us"])},
                    "completed": r["completed"], "refused": r["refused"], "wrong_verdicts": r["wrong_verdicts"],
                    "mean_batch": r["mean_batch"], "launch_ms_mean": r["launch_ms_mean"],
                    "launch_ms_max": r["launch_ms_max"]})
    srv.close()
    out["served_stream"] = {"sets": names, "keys": per * len(sids), "lengths": "log-uniform 16 B..1 MiB",
                            "points": pts}
    return out


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


def uneven_mixed(c, eng, reps=3):
    """Uneven batch: 256 distinct keypairs (128 per set), 2048 sign requests,
    lengths floor(exp(U(ln 1, ln 65536))) B, sets SHA-256-128s-simple and
    SHA-256-192f-robust drawn 50/50, autotuned mapping, one graph launch."""
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
        tuned[n] = autotune.tune(eng, sid, c.OP_SIGN, count=1024, mlen=64)[0]
    set_ids, sks, msgs = [], [], []
    for _ in range(2048):
        sid = sids[int(rng.integers(0, 2))]
        L = int(np.floor(np.exp(rng.uniform(0.0, np.log(65536.0)))))
        set_ids.append(sid)
        sks.append(keys[sid][int(rng.integers(0, 128))])
        msgs.append(rng.bytes(L))
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
    return {"workload": "2048 sign requests, 256 keys, lengths log-uniform 1 B..64 KiB, sets %s 50/50, one "
                        "graph launch" % "+".join(names),
            "sign_per_s": 2048 / (best / 1e3), "ms_per_launch": best, "tuning": tuned,
            "oracle_subset_identical": bool(ok), "subset": len(chk)}


def verify_heavy(c, eng, reps=3):
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
        out[name] = {"verify_per_s": count / (best / 1e3), "ms_per_launch": best, "corrupted": int(bad.sum()),
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
            "keypair_ms": kp_ms, "keypair_note": "median of 5 calls after a first (context-creating) call"}


if __name__ == "__main__":
    sys.exit(main())
