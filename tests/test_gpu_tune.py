"""The autotuner's result lives in the library: tune() installs a per-size
mapping in the engine, records it in the tuning file, and a new context
(cuspx_create) reads that file, so every caller of the C ABI -- drop-ins,
one-shot calls, serving -- runs the tuned mapping."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _verify_batch_ms(eng, c, sid, n, reps=5):
    z = c.set_sizes(sid)
    rng = np.random.default_rng(77)
    pks, sks = eng.keypair_batch(sid, [rng.bytes(z["seed"])])
    msgs = [rng.bytes(64) for _ in range(n)]
    sigs, _ = eng.sign_batch(sid, [sks[0]] * n, msgs)
    slab, offs, lens = c.pack_messages(msgs)
    b = eng.batch(c.OP_VERIFY, sid, n, len(slab), 1)
    b.upload(n, pks[0], 1, np.zeros(n, dtype=np.uint32), slab, len(slab), offs, lens,
             np.frombuffer(b"".join(sigs), dtype=np.uint8))
    best = None
    for _ in range(reps):
        b.run()
        b.sync()
        best = b.last_ms() if best is None else min(best, b.last_ms())
    v = np.zeros(n, dtype=np.int32)
    b.download(None, None, v)
    b.close()
    assert (v == 0).all()
    return best


def test_tune_is_installed_in_the_library_and_round_trips(tmp_path, monkeypatch):
    import cuspx_gb300 as c
    from cuspx_gb300 import autotune
    path = tmp_path / "tune.tsv"
    monkeypatch.setenv("CUSPX_TUNE_CACHE", str(path))
    eng = c.Engine(0)
    try:
        sid = c.set_id("sha256-128f-simple")
        n = 256
        default_ms = _verify_batch_ms(eng, c, sid, n)
        mapping, best = autotune.tune(eng, sid, c.OP_VERIFY, count=n, reps=2, passes=1)
        # the engine runs the tuned mapping for this size, the base is untouched
        got = eng.get_tuning_for(sid, c.OP_VERIFY, n)
        assert {k: got[k] for k in mapping} == mapping
        tuned_ms = _verify_batch_ms(eng, c, sid, n)
        assert tuned_ms <= default_ms * 1.15, (tuned_ms, default_ms, mapping)
        assert path.exists()
        assert autotune.load_cache(str(path))[(c.device_name(), "sha256-128f-simple", "verify", 256)][1] == mapping
    finally:
        eng.close()
    # a new context reads the file at creation
    eng2 = c.Engine(0)
    try:
        got = eng2.get_tuning_for(sid, c.OP_VERIFY, n)
        assert {k: got[k] for k in mapping} == mapping
        # sizes outside the entry's bucket (65..256 items) and other ops keep the base mapping
        assert eng2.get_tuning_for(sid, c.OP_VERIFY, 64) == eng2.get_tuning(sid)
        assert eng2.get_tuning_for(sid, c.OP_VERIFY, 257) == eng2.get_tuning(sid)
        assert {k: eng2.get_tuning_for(sid, c.OP_VERIFY, 65)[k] for k in mapping} == mapping
        assert eng2.get_tuning_for(sid, c.OP_SIGN, n) == eng2.get_tuning(sid)
        eng2.clear_tuning_for(sid)
        assert eng2.get_tuning_for(sid, c.OP_VERIFY, n) == eng2.get_tuning(sid)
        assert eng2.load_tuning(str(path)) == 1
    finally:
        eng2.close()


def test_per_size_entries_cover_their_ranges(monkeypatch, tmp_path):
    import cuspx_gb300 as c
    monkeypatch.setenv("CUSPX_TUNE_CACHE", str(tmp_path / "none.tsv"))
    eng = c.Engine(0)
    try:
        sid = c.set_id("shake256-128f-simple")
        base = eng.get_tuning(sid)["leaf_block"]
        eng.set_tuning_for(sid, c.OP_SIGN, 1, 64, leaf_block=64)
        eng.set_tuning_for(sid, c.OP_SIGN, 65, 1024, leaf_block=256)
        assert eng.get_tuning_for(sid, c.OP_SIGN, 1)["leaf_block"] == 64
        assert eng.get_tuning_for(sid, c.OP_SIGN, 64)["leaf_block"] == 64
        assert eng.get_tuning_for(sid, c.OP_SIGN, 65)["leaf_block"] == 256
        assert eng.get_tuning_for(sid, c.OP_SIGN, 99999)["leaf_block"] == base
        with pytest.raises(c.CuspxError):   # overlaps 65..1024
            eng.set_tuning_for(sid, c.OP_SIGN, 1000, 2000, leaf_block=128)
        # every entry gives the oracle's bytes
        import spx_oracle
        o = spx_oracle.Oracle("shake256-128f-simple")
        pk, sk = o.seed_keypair(bytes(range(48)))
        for count in (3, 70):
            msgs = [bytes([i]) * (i + 1) for i in range(count)]
            sigs, st = eng.sign_batch(sid, [sk] * count, msgs)
            assert list(st) == [0] * count
            assert sigs[0] == o.sign(msgs[0], sk) and sigs[-1] == o.sign(msgs[-1], sk)
    finally:
        eng.close()


def test_sorted_verify_knobs(monkeypatch, tmp_path):
    """verify_groups / verify_sorted_min / verify_spec_max: per-set defaults, range checks,
    0 and -1 for the size threshold (off / keep), and the C reader of the
    tuning file parses both."""
    import cuspx_gb300 as c
    monkeypatch.setenv("CUSPX_TUNE_CACHE", str(tmp_path / "none.tsv"))
    eng = c.Engine(0)
    try:
        s128 = c.set_id("sha256-128f-simple")
        s256 = c.set_id("shake256-256f-simple")
        assert eng.get_tuning(s128)["verify_sorted_min"] == 1024
        assert eng.get_tuning(s256)["verify_sorted_min"] == 2048
        assert eng.get_tuning(s128)["verify_groups"] == 4
        assert eng.get_tuning(s128)["verify_spec_max"] == 32
        assert eng.get_tuning(c.set_id("sha256-192f-robust"))["verify_spec_max"] == 64
        for bad in ({"verify_groups": 9}, {"verify_mode": 4}, {"verify_spec_max": 65}):
            with pytest.raises(c.CuspxError):
                eng.set_tuning(s128, **bad)
        eng.set_tuning(s128, verify_sorted_min=0, verify_groups=8)
        assert eng.get_tuning(s128)["verify_sorted_min"] == 0 and eng.get_tuning(s128)["verify_groups"] == 8
        eng.set_tuning(s128, verify_groups=0, verify_sorted_min=-1)   # both keep
        assert eng.get_tuning(s128)["verify_sorted_min"] == 0 and eng.get_tuning(s128)["verify_groups"] == 8
        eng.set_tuning(s128, verify_sorted_min=1024, verify_groups=4)
        path = tmp_path / "tune.tsv"
        path.write_text("%s\tsha256-128f-simple\tverify\t1025\t4096\t2.0\tverify_groups=6,verify_sorted_min=512\n"
                        % c.device_name())
        assert eng.load_tuning(str(path)) == 1
        got = eng.get_tuning_for(s128, c.OP_VERIFY, 4096)
        assert got["verify_groups"] == 6 and got["verify_sorted_min"] == 512
        assert eng.get_tuning_for(s128, c.OP_VERIFY, 1024)["verify_groups"] == 4
    finally:
        eng.close()
