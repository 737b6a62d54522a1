"""Serving face on the GPU: a request's result is the same alone and in a
busy mixed stream, admission respects the memory budget and the queue
limit, and the open-loop load generator's verdicts are all correct."""
import random

import pytest

pytestmark = pytest.mark.gpu


def _setup(engine, names, nkeys, seed=5):
    import cuspx_gb300 as c
    rng = random.Random(seed)
    keys = {}
    for name in names:
        sid = c.set_id(name)
        z = c.set_sizes(sid)
        seeds = [bytes(rng.randrange(256) for _ in range(z["seed"])) for _ in range(nkeys)]
        pks, sks = engine.keypair_batch(sid, seeds)
        keys[sid] = (pks, sks, z)
    return keys


def test_same_result_alone_and_in_the_mix(engine):
    import cuspx_gb300 as c
    import spx_oracle
    names = ["sha256-128f-simple", "sha256-192f-simple", "shake256-256f-simple"]
    keys = _setup(engine, names, 4)
    rng = random.Random(11)
    probe_set = c.set_id("sha256-128f-simple")
    pks, sks, z = keys[probe_set]
    probe_msg = bytes(rng.randrange(256) for _ in range(777))
    oracle_sig = spx_oracle.Oracle("sha256-128f-simple").sign(probe_msg, sks[2])

    srv = c.Server(engine, max_batch=64, max_inflight=2, window_us=200)
    try:
        ids = {sid: srv.add_keys(sid, v[1]) for sid, v in keys.items()}
        # alone
        t = srv.submit(c.OP_SIGN, probe_set, ids[probe_set][2], probe_msg)
        alone, st, _ = srv.wait(t, 60_000_000, z["sig"])
        assert st == 0 and alone == oracle_sig
        # in the mix: many signs and verifies of other sets and keys around it
        tickets = []
        for i in range(150):
            sid = rng.choice(list(keys))
            pk_, sk_, zz = keys[sid]
            k = rng.randrange(4)
            m = bytes(rng.randrange(256) for _ in range(rng.randrange(0, 3000)))
            tickets.append((c.OP_SIGN, sid, k, m, srv.submit(c.OP_SIGN, sid, ids[sid][k], m)))
            if i == 75:
                tp = srv.submit(c.OP_SIGN, probe_set, ids[probe_set][2], probe_msg)
        mixed, st, _ = srv.wait(tp, 120_000_000, z["sig"])
        assert st == 0 and mixed == alone
        # verify everything that was signed in the mix, each verdict alone-correct
        vt = []
        for op, sid, k, m, t in tickets:
            sig, st, _ = srv.wait(t, 120_000_000, keys[sid][2]["sig"])
            assert st == 0
            bad = bytearray(sig)
            bad[len(bad) // 3] ^= 4
            vt.append((srv.submit(c.OP_VERIFY, sid, ids[sid][k], m, sig), 0))
            vt.append((srv.submit(c.OP_VERIFY, sid, ids[sid][k], m, bytes(bad)), -1))
        for t, want in vt:
            _, st, _ = srv.wait(t, 120_000_000)
            assert st == want
        s = srv.stats()
        assert s["failed"] == 0 and s["launches"] >= 2
    finally:
        srv.close()


def test_memory_budget_admission(engine):
    """Admission by device-memory budget: each request counts the device
    bytes its launch will need from submission on, so with a 1 MB budget
    (one 128f signing item needs ~230 KB) only a few requests are admitted at
    a time and the rest are refused with E_BUSY; every admitted request
    completes, the in-flight bytes never exceed the budget, and once the
    queue drains new requests are admitted again."""
    import cuspx_gb300 as c
    keys = _setup(engine, ["sha256-128f-simple"], 2)
    sid = c.set_id("sha256-128f-simple")
    pks, sks, z = keys[sid]
    srv = c.Server(engine, mem_budget=1 << 20, max_batch=256, max_inflight=2, window_us=100)
    try:
        ids = srv.add_keys(sid, sks)
        ts, refused = [], 0
        for i in range(40):
            try:
                ts.append(srv.submit(c.OP_SIGN, sid, ids[i % 2], b"m%d" % i))
            except c.CuspxError as e:
                assert e.code == c.E_BUSY
                refused += 1
        # ~4 fit at once; a few more may be admitted as early ones complete
        assert len(ts) >= 1 and refused >= 20 and refused == 40 - len(ts)
        for t in ts:
            _, st, _ = srv.wait(t, 120_000_000, z["sig"])
            assert st == 0
        s = srv.stats()
        assert s["bytes_peak"] <= 1 << 20 and s["refused"] == refused
        # drained: admitted again, and the signature is the engine's one-shot one
        t = srv.submit(c.OP_SIGN, sid, ids[0], b"again")
        sig, st, _ = srv.wait(t, 120_000_000, z["sig"])
        want, _ = engine.sign_batch(sid, [sks[0]], [b"again"])
        assert st == 0 and sig == want[0]
        # a request that could never fit the budget is refused outright
        with pytest.raises(c.CuspxError) as ei:
            srv.submit(c.OP_SIGN, sid, ids[0], bytes(1 << 20))
        assert ei.value.code == c.E_NOMEM
    finally:
        srv.close()


def test_queue_limit_refuses(engine):
    import cuspx_gb300 as c
    keys = _setup(engine, ["sha256-128f-simple"], 1)
    sid = c.set_id("sha256-128f-simple")
    srv = c.Server(engine, max_queue=4, max_batch=2, max_inflight=1, window_us=1_000_000)
    try:
        kid = srv.add_keys(sid, keys[sid][1])[0]
        refused = 0
        tickets = []
        for i in range(64):
            try:
                tickets.append(srv.submit(c.OP_SIGN, sid, kid, b"x" * i))
            except c.CuspxError as e:
                assert e.code == c.E_BUSY
                refused += 1
        assert refused > 0
        for t in tickets:
            srv.wait(t, 120_000_000, keys[sid][2]["sig"])
        # signing with an unknown key is refused up front
        with pytest.raises(c.CuspxError):
            srv.submit(c.OP_SIGN, sid, 999, b"x")
    finally:
        srv.close()


def test_loadgen_short_run(engine):
    import cuspx_gb300 as c
    names = ["sha256-128f-simple", "shake256-256f-simple"]
    keys = _setup(engine, names, 2)
    srv = c.Server(engine, max_batch=256, window_us=300)
    try:
        for sid, v in keys.items():
            srv.add_keys(sid, v[1])
        r = srv.loadgen(rate=2000, seconds=0.5, sets=list(keys), keys_per_set=2, verify_frac=0.7,
                        min_len=16, max_len=4096, corrupt_frac=0.1, seed=3, pool=16)
        assert r["rc"] == 0, r
        assert r["wrong_verdicts"] == 0
        assert r["completed"] + r["refused"] == r["offered"] and r["offered"] > 500
    finally:
        srv.close()


def test_prepared_slots_serve_the_same_bytes(engine):
    """cuspx_serve_prepare creates a set's launch slots (and its key table)
    before any key or request; keys added afterwards are served through the
    prepared slots, short and long messages alike, with the oracle's bytes."""
    import cuspx_gb300 as c
    import spx_oracle
    name = "sha256-128f-simple"
    sid = c.set_id(name)
    keys = _setup(engine, [name], 2, seed=21)
    pks, sks, z = keys[sid]
    o = spx_oracle.Oracle(name)
    rng = random.Random(23)
    srv = c.Server(engine, max_batch=32, max_inflight=2, window_us=200)
    try:
        for op in (c.OP_SIGN, c.OP_VERIFY):
            srv.prepare(op, sid)
            srv.prepare(op, sid)   # a second call finds every slot there
        ids = srv.add_keys(sid, sks)
        msgs = [bytes(rng.randrange(256) for _ in range(L)) for L in (10, 3000, 20000)]
        tickets = [srv.submit(c.OP_SIGN, sid, ids[1], m) for m in msgs]
        for m, t in zip(msgs, tickets):
            sig, st, _ = srv.wait(t, 60_000_000, z["sig"])
            assert st == 0 and sig == o.sign(m, sks[1])
            tv = srv.submit(c.OP_VERIFY, sid, ids[1], m, sig)
            _, vst, _ = srv.wait(tv, 60_000_000, 0)
            assert vst == 0
    finally:
        srv.close()


MIB = 1 << 20


def test_long_class_packs_megabyte_messages(engine):
    """Messages of about 1 MiB go to the long length class.  With one launch
    slot, the first request launches alone and the next ones queue behind it
    and then share one launch (more than 2 MiB of messages packed into one
    message slab).  Every signature equals the oracle's, and the long verify
    class accepts them all and rejects a corrupted one."""
    import cuspx_gb300 as c
    import spx_oracle
    name = "sha256-128f-simple"
    sid = c.set_id(name)
    keys = _setup(engine, [name], 2, seed=31)
    pks, sks, z = keys[sid]
    o = spx_oracle.Oracle(name)
    rng = random.Random(37)
    lens = [MIB, MIB - 1, MIB + 1, MIB + 17, 3 * MIB // 2]
    msgs = [rng.randbytes(L) for L in lens]
    srv = c.Server(engine, max_batch=64, max_inflight=1, window_us=200)
    try:
        ids = srv.add_keys(sid, sks)
        tickets = [srv.submit(c.OP_SIGN, sid, ids[i % 2], m) for i, m in enumerate(msgs)]
        sigs = []
        for t in tickets:
            sig, st, _ = srv.wait(t, 120_000_000, z["sig"])
            assert st == 0
            sigs.append(sig)
        s = srv.stats()
        assert s["launches"] < len(msgs), s["launches"]   # some launch held >= 2 MiB of messages
        for i, (m, sig) in enumerate(zip(msgs, sigs)):
            assert sig == o.sign(m, sks[i % 2]), len(m)
        bad = bytearray(sigs[2])
        bad[len(bad) // 2] ^= 0x40
        vt = [srv.submit(c.OP_VERIFY, sid, ids[i % 2], m, sig) for i, (m, sig) in enumerate(zip(msgs, sigs))]
        vt.append(srv.submit(c.OP_VERIFY, sid, ids[0], msgs[2], bytes(bad)))
        got = [srv.wait(t, 120_000_000)[1] for t in vt]
        assert got == [0] * len(msgs) + [o.verify(bytes(bad), msgs[2], pks[0])] == [0] * len(msgs) + [-1]
    finally:
        srv.close()


def test_middle_class_does_not_wait_for_megabyte_launches(engine):
    """A 64 KiB request submitted behind a launch of 1 MiB messages is batched
    in the middle length class and completes first (its own launch hashes
    64 KiB, not 1 MiB)."""
    import cuspx_gb300 as c
    import spx_oracle
    name = "sha256-128f-simple"
    sid = c.set_id(name)
    keys = _setup(engine, [name], 1, seed=41)
    pks, sks, z = keys[sid]
    rng = random.Random(43)
    srv = c.Server(engine, max_batch=64, max_inflight=2, window_us=200)
    try:
        for op in (c.OP_SIGN, c.OP_VERIFY):
            srv.prepare(op, sid)
        kid = srv.add_keys(sid, sks)[0]
        longs = [srv.submit(c.OP_SIGN, sid, kid, rng.randbytes(MIB)) for _ in range(4)]
        mid_msg = rng.randbytes(64 * 1024)
        tm = srv.submit(c.OP_SIGN, sid, kid, mid_msg)
        sig, st, lat_mid = srv.wait(tm, 120_000_000, z["sig"])
        assert st == 0 and sig == spx_oracle.Oracle(name).sign(mid_msg, sks[0])
        lat_long = [srv.wait(t, 120_000_000, z["sig"])[2] for t in longs]
        assert lat_mid < max(lat_long), (lat_mid, lat_long)
    finally:
        srv.close()


def test_one_waiter_per_ticket(engine):
    """A second thread waiting on a ticket that already has a waiter is
    refused at once (the first waiter frees the request when it returns)."""
    import threading
    import cuspx_gb300 as c
    name = "sha256-128f-simple"
    sid = c.set_id(name)
    keys = _setup(engine, [name], 1, seed=47)
    z = keys[sid][2]
    srv = c.Server(engine, max_batch=8, max_inflight=1, window_us=100)
    try:
        kid = srv.add_keys(sid, keys[sid][1])[0]
        # one long-class slot: the first 1 MiB request launches alone, the
        # next two wait for it (~33 ms), so the ticket is pending below
        block = [srv.submit(c.OP_SIGN, sid, kid, bytes(MIB)) for _ in range(2)]
        t = srv.submit(c.OP_SIGN, sid, kid, b"waited twice".ljust(MIB, b"."))
        first = {}

        def waiter():
            first["r"] = srv.wait(t, 120_000_000, z["sig"])

        th = threading.Thread(target=waiter)
        th.start()
        import time
        time.sleep(0.005)
        with pytest.raises(c.CuspxError):
            srv.wait(t, 120_000_000, z["sig"])
        th.join()
        assert first["r"][1] == 0
        with pytest.raises(c.CuspxError):   # released by the first waiter
            srv.wait(t, 0)
        for b in block:
            srv.wait(b, 120_000_000, z["sig"])
    finally:
        srv.close()


def test_loadgen_sample_matches_oracle(engine):
    """The load generator keeps one in every few of its timed sign requests:
    each sampled signature, from a stream mixing two parameter sets and
    message lengths up to 256 KiB (all three length classes), equals the
    oracle's signature of the same message under the same key."""
    import cuspx_gb300 as c
    import spx_oracle
    names = ["sha256-128f-simple", "sha256-192f-simple"]
    keys = _setup(engine, names, 3, seed=53)
    srv = c.Server(engine, max_batch=128, window_us=300)
    try:
        for sid, v in keys.items():
            srv.add_keys(sid, v[1])
        r = srv.loadgen(rate=1500, seconds=0.4, sets=list(keys), keys_per_set=3, verify_frac=0.5,
                        min_len=16, max_len=256 * 1024, corrupt_frac=0.1, seed=9, pool=8,
                        sample_every=4, sample_max=24, arena_bytes=24 * (256 * 1024 + 40000))
        assert r["rc"] == 0 and r["wrong_verdicts"] == 0, r
        assert r["sampled"] >= 8 and len(r["samples"]) == r["sampled"]
        assert sum(r["set_sign_done"]) == r["sign_done"] and sum(r["set_verify_done"]) == r["verify_done"]
        assert all(u > 0 for u in r["set_msg_units"][:2])
        oracles = {c.set_id(n): spx_oracle.Oracle(n) for n in names}
        for sid, kid, st, msg, sig in r["samples"]:
            assert st == 0
            assert sig == oracles[sid].sign(msg, keys[sid][1][kid]), (sid, len(msg))
    finally:
        srv.close()


def test_work_based_admission_and_launch_cap(engine):
    """With max_queue_ms the server refuses a submission once the estimated
    GPU work pending or in flight exceeds that many ms of the stated capacity
    (here 1e13 integer ops/s: one SHAKE-256-256f sign is ~1.6e9 ops, 0.16 ms);
    with max_launch_ms a launch carries at most that much work.  Every
    admitted request completes with the right bytes."""
    import cuspx_gb300 as c
    import spx_oracle
    name = "shake256-256f-simple"
    sid = c.set_id(name)
    keys = _setup(engine, [name], 1, seed=61)
    pks, sks, z = keys[sid]
    srv = c.Server(engine, max_batch=256, max_inflight=1, window_us=100_000, max_queue_ms=1.0,
                   max_launch_ms=0.35, gpu_ops_per_s=1e13)
    try:
        for op in (c.OP_SIGN, c.OP_VERIFY):
            srv.prepare(op, sid)
        kid = srv.add_keys(sid, sks)[0]
        ts, refused = [], 0
        for i in range(40):
            try:
                ts.append((i, srv.submit(c.OP_SIGN, sid, kid, b"w%d" % i)))
            except c.CuspxError as e:
                assert e.code == c.E_BUSY
                refused += 1
        # ~1 ms / 0.16 ms per sign: about six admitted while the first ones run
        assert 3 <= len(ts) <= 16 and refused >= 24, (len(ts), refused)
        sigs = {}
        for i, t in ts:
            sig, st, _ = srv.wait(t, 120_000_000, z["sig"])
            assert st == 0
            sigs[i] = sig
        s = srv.stats()
        # 0.35 ms per launch: at most two of these signs in one launch
        assert s["launches"] >= (len(ts) + 1) // 2, s
        i0 = ts[0][0]
        assert sigs[i0] == spx_oracle.Oracle(name).sign(b"w%d" % i0, sks[0])
        # drained: admitted again
        t = srv.submit(c.OP_SIGN, sid, kid, b"again")
        assert srv.wait(t, 120_000_000, z["sig"])[1] == 0
    finally:
        srv.close()
