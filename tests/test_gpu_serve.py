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
    import cuspx_gb300 as c
    keys = _setup(engine, ["sha256-128f-simple"], 2)
    sid = c.set_id("sha256-128f-simple")
    pks, sks, z = keys[sid]
    # one signing item of 128f needs ~230 KB of device scratch: a 1 MB budget
    # admits only a handful per launch, yet every request completes
    srv = c.Server(engine, mem_budget=1 << 20, max_batch=256, max_inflight=2, window_us=100)
    try:
        ids = srv.add_keys(sid, sks)
        ts = [srv.submit(c.OP_SIGN, sid, ids[i % 2], b"m%d" % i) for i in range(40)]
        for t in ts:
            _, st, _ = srv.wait(t, 120_000_000, z["sig"])
            assert st == 0
        s = srv.stats()
        assert s["bytes_peak"] <= 1 << 20
        assert s["launches"] >= 40 // 4
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
