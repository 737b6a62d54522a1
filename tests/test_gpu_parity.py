"""GPU parity: the engine (through the C ABI) against the reference's own
outputs (tests/golden, written by tests/golden/make_golden.py from the
reference CPU code) and against the C restatement in oracle/ for cases the
fixtures do not hold (distinct keys, robust sets, long messages).

Everything here is integer/byte work, so the bar is byte equality.
"""
import hashlib
import os
import random

import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

SIMPLE_SETS = ["sha256-128f", "sha256-128s", "sha256-192f", "sha256-192s", "sha256-256f", "sha256-256s",
               "shake256-128f", "shake256-128s", "shake256-192f", "shake256-192s", "shake256-256f", "shake256-256s"]


def _oracle(name):
    import spx_oracle
    return spx_oracle.Oracle(name)


@pytest.mark.parametrize("setname", SIMPLE_SETS)
def test_keypair_matches_reference(engine, setname):
    g = load_golden(setname)
    sid = engine.set_id(setname)
    seeds = [bytes.fromhex(g["seed"]), bytes(range(g["seed_bytes"]))]
    pks, sks = engine.keypair_batch(sid, seeds)
    assert pks[0].hex() == g["pk"] and sks[0].hex() == g["sk"]
    # crypto_sign_keypair under the shipped DEBUG_MODE uses seed 0..3n-1
    assert pks[1].hex() == g["debug_keypair"]["pk"] and sks[1].hex() == g["debug_keypair"]["sk"]


@pytest.mark.parametrize("setname", SIMPLE_SETS)
def test_sign_matches_reference(engine, setname):
    g = load_golden(setname)
    sid = engine.set_id(setname)
    sk = bytes.fromhex(g["sk"])
    msgs = [bytes.fromhex(c["msg"]) for c in g["cases"]]
    sigs, status = engine.sign_batch(sid, [sk] * len(msgs), msgs)
    assert list(status) == [0] * len(msgs)
    for c, sig in zip(g["cases"], sigs):
        assert len(sig) == g["sig_bytes"]
        assert sig[:64].hex() == c["sig_head"], "mlen=%d" % c["mlen"]
        assert hashlib.sha256(sig).hexdigest() == c["sig_sha256"], "mlen=%d" % c["mlen"]
        if "sig_file" in c:
            with open(os.path.join(GOLDEN, c["sig_file"]), "rb") as f:
                assert sig == f.read()


@pytest.mark.parametrize("setname", SIMPLE_SETS)
def test_verify_matches_reference(engine, setname):
    """Good signatures accept; every corruption the reference rejected is rejected."""
    g = load_golden(setname)
    sid = engine.set_id(setname)
    sk, pk = bytes.fromhex(g["sk"]), bytes.fromhex(g["pk"])
    msgs = [bytes.fromhex(c["msg"]) for c in g["cases"]]
    sigs, _ = engine.sign_batch(sid, [sk] * len(msgs), msgs)
    vs_pk, vs_m, vs_sig, vs_len, want = [], [], [], [], []
    for c, m, sig in zip(g["cases"], msgs, sigs):
        vs_pk.append(pk); vs_m.append(m); vs_sig.append(sig); vs_len.append(len(sig)); want.append(c["verify"])
        for fl in c["corrupt"]:
            bad = bytearray(sig)
            bad[fl["pos"]] ^= fl["xor"]
            vs_pk.append(pk); vs_m.append(m); vs_sig.append(bytes(bad)); vs_len.append(len(sig))
            want.append(fl["verify"])
        if "msgflip_verify" in c:
            bm = bytearray(m)
            bm[len(m) // 2] ^= 0x10
            vs_pk.append(pk); vs_m.append(bytes(bm)); vs_sig.append(sig); vs_len.append(len(sig))
            want.append(c["msgflip_verify"])
        vs_pk.append(pk); vs_m.append(m); vs_sig.append(sig); vs_len.append(len(sig) - 1)
        want.append(c["shortsig_verify"])
    got = engine.verify_batch(sid, vs_pk, vs_m, vs_sig, siglens=vs_len)
    assert list(got) == want


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "shake256-128f-simple", "sha256-192f-robust",
                                     "sha256-128f-robust", "shake256-256f-robust", "shake256-128f-robust"])
def test_distinct_keys_uneven_lengths_vs_oracle(engine, setname):
    """A batch with distinct keys and uneven lengths equals the oracle item by item."""
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(1234)
    n = o.p.n
    seeds = [bytes(rng.randrange(256) for _ in range(3 * n)) for _ in range(4)]
    pks, sks = engine.keypair_batch(sid, seeds)
    for s, pk, sk in zip(seeds, pks, sks):
        opk, osk = o.seed_keypair(s)
        assert (pk, sk) == (opk, osk)
    lens = [0, 1, 17, 55, 56, 64, 100, 333]
    msgs = [bytes(rng.randrange(256) for _ in range(L)) for L in lens]
    key_of = [i % 4 for i in range(len(msgs))]
    optrand = [bytes(rng.randrange(256) for _ in range(n)) for _ in msgs]
    sigs, st = engine.sign_batch(sid, [sks[k] for k in key_of], msgs, optrand=optrand)
    assert list(st) == [0] * len(msgs)
    for m, k, opt, sig in zip(msgs, key_of, optrand, sigs):
        assert sig == o.sign(m, sks[k], opt), "mlen=%d" % len(m)
    v = engine.verify_batch(sid, [pks[k] for k in key_of], msgs, sigs)
    assert list(v) == [0] * len(msgs)
    # wrong key rejects
    v = engine.verify_batch(sid, [pks[(k + 1) % 4] for k in key_of], msgs, sigs)
    assert list(v) == [-1] * len(msgs)


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "shake256-128f-simple"])
def test_long_message_vs_oracle(engine, setname):
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(7)
    seed = bytes(rng.randrange(256) for _ in range(3 * o.p.n))
    pk, sk = o.seed_keypair(seed)
    msgs = [bytes(rng.randrange(256) for _ in range(L)) for L in (65536, 4097, 1000)]
    sigs, _ = engine.sign_batch(sid, [sk] * 3, msgs)
    for m, s in zip(msgs, sigs):
        assert s == o.sign(m, sk)
    assert list(engine.verify_batch(sid, [pk] * 3, msgs, sigs)) == [0, 0, 0]


def test_sign_status_flags_bad_key(engine):
    """A secret key whose ROOT does not match its seeds is reported per item."""
    sid = engine.set_id("sha256-128f-simple")
    g = load_golden("sha256-128f")
    sk = bytearray.fromhex(g["sk"])
    bad = bytearray(sk)
    bad[-1] ^= 1
    _, st = engine.sign_batch(sid, [bytes(sk), bytes(bad)], [b"abc", b"abc"])
    assert list(st) == [0, -2]


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "shake256-256f-simple", "sha256-192f-robust",
                                     "sha256-192f-simple", "sha256-256f-simple", "sha256-128s-simple",
                                     "shake256-128f-simple", "shake256-192s-simple", "shake256-256f-robust",
                                     "shake256-128f-robust", "shake256-192s-robust", "sha256-128f-robust",
                                     "sha256-256f-robust", "sha256-128s-robust"])
def test_verify_mappings_agree(engine, setname):
    """Every verify launch mapping the autotuner may pick returns the same verdicts."""
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(99)
    seeds = [bytes(rng.randrange(256) for _ in range(3 * o.p.n)) for _ in range(3)]
    pks, sks = engine.keypair_batch(sid, seeds)
    msgs = [bytes(rng.randrange(256) for _ in range(rng.randrange(0, 300))) for _ in range(12)]
    kidx = [i % 3 for i in range(12)]
    sigs, _ = engine.sign_batch(sid, [sks[k] for k in kidx], msgs)
    sigs = list(sigs)
    for i in (1, 5, 9):
        b = bytearray(sigs[i])
        b[rng.randrange(len(b))] ^= 1 << rng.randrange(8)
        sigs[i] = bytes(b)
    want = [o.verify(s, m, pks[k]) for s, m, k in zip(sigs, msgs, kidx)]
    assert want.count(-1) == 3
    saved = engine.get_tuning(sid)
    try:
        for m in ({"verify_mode": 0, "chains_per_warp": 32}, {"verify_mode": 0, "chains_per_warp": 64},
                  {"verify_mode": 0, "chains_per_warp": 1024}, {"verify_mode": 1},
                  {"verify_mode": 2, "verify_slots": 1, "verify_block": 32},
                  {"verify_mode": 2, "verify_slots": 3, "verify_block": 64},
                  {"verify_mode": 2, "verify_slots": 8, "verify_block": 128},
                  {"verify_mode": 2, "verify_slots": 4, "verify_block": 64, "verify_claim_min": 6},
                  {"verify_mode": 2, "verify_slots": 2, "verify_block": 32, "verify_claim_min": 32},
                  {"verify_mode": 3, "verify_groups": 1, "verify_block": 32},
                  {"verify_mode": 3, "verify_groups": 2, "verify_block": 64},
                  {"verify_mode": 3, "verify_groups": 4, "verify_block": 128},
                  {"verify_spec_max": 16}):
            engine.set_tuning(sid, **dict({"verify_item_max": 0, "verify_claim_min": 1, "verify_sorted_min": 0,
                                            "verify_spec_max": 0}, **m))
            got = engine.verify_batch(sid, [pks[k] for k in kidx], msgs, sigs)
            assert list(got) == want, m
        # one item per block (the small-batch kernel)
        engine.set_tuning(sid, verify_item_max=64, verify_spec_max=0)
        assert list(engine.verify_batch(sid, [pks[k] for k in kidx], msgs, sigs)) == want
        # a batch large enough that the persistent kernel packs several
        # items into each warp (1300 items on 152 SMs: 3 per warp), and the
        # same batch one item per block (several blocks share each SM)
        rep = 1300
        for m in ({"verify_mode": 2, "verify_slots": 8, "verify_block": 64, "verify_item_max": 0,
                   "verify_sorted_min": 0},
                  {"verify_mode": 2, "verify_slots": 4, "verify_block": 64, "verify_item_max": 0,
                   "verify_claim_min": 8, "verify_sorted_min": 0},
                  {"verify_mode": 2, "verify_item_max": 0, "verify_sorted_min": 1000},
                  {"verify_mode": 3, "verify_groups": 3, "verify_block": 64, "verify_item_max": 0},
                  {"verify_item_max": 2000}):
            engine.set_tuning(sid, **m)
            got = engine.verify_batch(sid, [pks[kidx[i % 12]] for i in range(rep)],
                                      [msgs[i % 12] for i in range(rep)], [sigs[i % 12] for i in range(rep)])
            assert list(got) == [want[i % 12] for i in range(rep)], m
    finally:
        engine.set_tuning(sid, **saved)


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "shake256-256f-robust", "sha256-192s-robust"])
def test_sorted_verify_group_split(engine, setname):
    """The sorted layered verify (verify_mode 3) splits a batch into item
    groups on their own streams: batches smaller than the group count, one
    item, uneven splits and a wrong-length signature inside a group all give
    the CPU's verdicts, and so do batches the size threshold sends there
    whatever verify_mode says."""
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(31)
    seed = bytes(rng.randrange(256) for _ in range(3 * o.p.n))
    pk, sk = o.seed_keypair(seed)
    msgs = [bytes(rng.randrange(256) for _ in range(5 + 11 * i)) for i in range(4)]
    sigs = [o.sign(m, sk) for m in msgs]
    bad = bytearray(sigs[1])
    bad[len(bad) // 2] ^= 0x40
    cases = [(sigs[0], msgs[0], len(sigs[0])), (bytes(bad), msgs[1], len(bad)),
             (sigs[2], msgs[2], len(sigs[2]) - 8), (sigs[3], msgs[3], len(sigs[3]))]
    want = [o.verify(s, m, pk) if ln == len(s) else -1 for s, m, ln in cases]   # wrong length: rejected
    assert want == [0, -1, -1, 0]
    saved = engine.get_tuning(sid)
    try:
        for count, m in ((1, {"verify_mode": 3, "verify_groups": 4}),
                         (2, {"verify_mode": 3, "verify_groups": 4}),
                         (5, {"verify_mode": 3, "verify_groups": 3}),
                         (37, {"verify_mode": 3, "verify_groups": 4, "verify_block": 128}),
                         (37, {"verify_mode": 2, "verify_sorted_min": 30, "verify_groups": 2})):
            engine.set_tuning(sid, **dict({"verify_item_max": 0, "verify_spec_max": 0}, **m))
            pick = [(i * 7 + 3) % len(cases) for i in range(count)]
            got = engine.verify_batch(sid, [pk] * count, [cases[j][1] for j in pick], [cases[j][0] for j in pick],
                                      siglens=[cases[j][2] for j in pick])
            assert list(got) == [want[j] for j in pick], (count, m)
    finally:
        engine.set_tuning(sid, **saved)


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "sha256-192f-robust", "shake256-256f-robust",
                                     "shake256-128s-simple"])
def test_speculative_verify(engine, setname):
    """Tiny batches verified from speculative chain runs (every chain of every
    layer from each of its 16 start steps, then the serial T_len / auth-path
    walk): one item, a few, the 64-item maximum, corrupted and wrong-length
    signatures, all equal to the CPU's verdicts."""
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(61)
    pk, sk = o.seed_keypair(bytes(rng.randrange(256) for _ in range(3 * o.p.n)))
    msgs = [bytes(rng.randrange(256) for _ in range(3 + 29 * i)) for i in range(4)]
    sigs = [o.sign(m, sk) for m in msgs]
    bad = bytearray(sigs[1])
    bad[rng.randrange(len(bad))] ^= 0x02
    cases = [(sigs[0], msgs[0], len(sigs[0])), (bytes(bad), msgs[1], len(bad)),
             (sigs[2], msgs[2], len(sigs[2]) + 1), (sigs[3], msgs[3], len(sigs[3]))]
    want = [o.verify(sg, m, pk) if ln == len(sg) else -1 for sg, m, ln in cases]   # wrong length: rejected
    assert want == [0, -1, -1, 0]
    saved = engine.get_tuning(sid)
    try:
        engine.set_tuning(sid, verify_spec_max=64, verify_item_max=0)
        for count in (1, 3, 64):
            pick = [(i * 5 + 3) % len(cases) for i in range(count)] if count > 1 else [0]
            got = engine.verify_batch(sid, [pk] * count, [cases[j][1] for j in pick], [cases[j][0] for j in pick],
                                      siglens=[cases[j][2] for j in pick])
            assert list(got) == [want[j] for j in pick], count
    finally:
        engine.set_tuning(sid, **saved)


def test_persistent_verify_refills_slots(engine):
    """A batch larger than all resident warp slots together: warps take new
    items from the counter as items finish; every verdict is still the CPU's
    (intact, corrupted and wrong-length signatures interleaved)."""
    setname = "sha256-128f-simple"
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(7)
    seed = bytes(rng.randrange(256) for _ in range(3 * o.p.n))
    pk, sk = o.seed_keypair(seed)
    msgs = [bytes(rng.randrange(256) for _ in range(40 + 7 * i)) for i in range(3)]
    sigs = [o.sign(m, sk) for m in msgs]
    bad = []
    for s in sigs:
        b = bytearray(s)
        b[rng.randrange(len(b))] ^= 1 << rng.randrange(8)
        bad.append(bytes(b))
    cases = []   # (sig, msg, siglen, expected)
    for i in range(3):
        cases.append((sigs[i], msgs[i], len(sigs[i]), o.verify(sigs[i], msgs[i], pk)))
        cases.append((bad[i], msgs[i], len(bad[i]), o.verify(bad[i], msgs[i], pk)))
        cases.append((sigs[i], msgs[i], len(sigs[i]) - 1, -1))
    assert [c[3] for c in cases].count(0) == 3
    count = 6000   # > 152 SMs x 32 resident one-warp blocks x 1 slot
    pick = [rng.randrange(len(cases)) for _ in range(count)]
    saved = engine.get_tuning(sid)
    try:
        for m in ({"verify_mode": 2, "verify_slots": 1, "verify_block": 32, "verify_item_max": 0,
                   "verify_sorted_min": 0},
                  {"verify_mode": 2, "verify_slots": 4, "verify_block": 128, "verify_item_max": 0,
                   "verify_sorted_min": 0},
                  {"verify_mode": 3, "verify_groups": 2, "verify_block": 64, "verify_item_max": 0}):
            engine.set_tuning(sid, **m)
            got = engine.verify_batch(sid, [pk] * count, [cases[j][1] for j in pick], [cases[j][0] for j in pick],
                                      siglens=[cases[j][2] for j in pick])
            assert list(got) == [cases[j][3] for j in pick], m
    finally:
        engine.set_tuning(sid, **saved)


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "shake256-256f-simple", "sha256-128s-simple"])
def test_sign_mappings_agree(engine, setname):
    """Every sign launch mapping the autotuner may pick gives the same bytes."""
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(31)
    seed = bytes(rng.randrange(256) for _ in range(3 * o.p.n))
    pk, sk = o.seed_keypair(seed)
    msgs = [bytes(rng.randrange(256) for _ in range(rng.randrange(0, 200))) for _ in range(5)]
    want = [o.sign(m, sk) for m in msgs[:2]]
    saved = engine.get_tuning(sid)
    ref = None
    try:
        for g, tm, lb, fb, cm in ((5, 0, 128, 128, 0), (0, 1, 64, 64, 64), (2, 1, 256, 96, 0),
                                  (3, 0, 96, 256, 256)):
            engine.set_tuning(sid, fors_lanes_log2=g, tree_mode=tm, leaf_block=lb, fors_block=fb,
                              chain_mode_max=cm)
            sigs, st = engine.sign_batch(sid, [sk] * len(msgs), msgs)
            assert list(st) == [0] * len(msgs)
            assert list(sigs[:2]) == want, (g, tm, lb, fb, cm)
            if ref is None:
                ref = sigs
            assert sigs == ref, (g, tm, lb, fb, cm)
    finally:
        engine.set_tuning(sid, **saved)


def test_empty_batches_and_length_edges(engine):
    """Zero-item keygen, sign and verify calls and batch runs return at once
    with empty results; in a verify batch an empty message verifies like any
    other, and a signature of length 0, SPX_BYTES - 1 or SPX_BYTES + 1 is
    rejected (crypto_sign_verify, sign.cu:3064: siglen != SPX_BYTES -> -1)
    without disturbing its neighbours."""
    import cuspx_gb300 as c
    for name in ("sha256-128f-simple", "shake256-128f-simple"):
        o = _oracle(name)
        sid = engine.set_id(name)
        z = c.set_sizes(sid)
        pks, sks = engine.keypair_batch(sid, [])
        assert pks == [] and sks == []
        sigs, st = engine.sign_batch(sid, [], [])
        assert sigs == [] and len(st) == 0
        assert len(engine.verify_batch(sid, [], [], [])) == 0
        b = engine.batch(c.OP_SIGN, sid, 4, 64, 1)
        b.upload(0, None)
        b.run()
        b.sync()
        b.close()
        rng = random.Random(8)
        pk, sk = o.seed_keypair(bytes(rng.randrange(256) for _ in range(z["seed"])))
        msgs = [b"", b"x" * 33]
        sigs, st = engine.sign_batch(sid, [sk] * 2, msgs)
        assert list(st) == [0, 0]
        assert sigs[0] == o.sign(b"", sk) and sigs[1] == o.sign(msgs[1], sk)
        vm = [msgs[0], msgs[1], msgs[0], msgs[1], msgs[0]]
        vs = [sigs[0], sigs[1], b"", sigs[1], sigs[0]]
        vl = [z["sig"], z["sig"], 0, z["sig"] - 1, z["sig"] + 1]
        got = engine.verify_batch(sid, [pk] * 5, vm, vs, siglens=vl)
        assert list(got) == [0, 0, -1, -1, -1]


def test_keygen_mappings_agree(engine):
    """Key generation gives the same keys one lane per WOTS+ chain (taken for
    any batch the chain scratch holds) and one lane per leaf (chain_mode_max
    0), and they are the oracle's crypto_sign_seed_keypair keys."""
    o = _oracle("sha256-128f-simple")
    sid = engine.set_id("sha256-128f-simple")
    rng = random.Random(53)
    seeds = [bytes(rng.randrange(256) for _ in range(48)) for _ in range(300)]
    saved = engine.get_tuning(sid)
    try:
        pks_c, sks_c = engine.keypair_batch(sid, seeds)
        engine.set_tuning(sid, chain_mode_max=0)
        pks_l, sks_l = engine.keypair_batch(sid, seeds)
    finally:
        engine.set_tuning(sid, **saved)
    assert list(pks_c) == list(pks_l) and list(sks_c) == list(sks_l)
    for i in (0, 157, 299):
        pk, sk = o.seed_keypair(seeds[i])
        assert pks_c[i] == pk and sks_c[i] == sk, i


def test_mixed_sets_one_launch_vs_oracle(engine):
    """Uneven lengths, distinct keys and two parameter sets in one graph launch
    give the same signatures as the oracle item by item."""
    import cuspx_gb300 as c
    rng = random.Random(77)
    names = ["sha256-128f-simple", "sha256-192f-robust", "shake256-128f-simple"]
    oracles = {n: _oracle(n) for n in names}
    keys = {}
    for n in names:
        o = oracles[n]
        keys[n] = [o.seed_keypair(bytes(rng.randrange(256) for _ in range(3 * o.p.n))) for _ in range(3)]
    set_ids, sks, msgs, expect = [], [], [], []
    for i in range(24):
        n = names[i % 3]
        pk, sk = keys[n][rng.randrange(3)]
        m = bytes(rng.randrange(256) for _ in range(int(2 ** rng.uniform(0, 12))))
        set_ids.append(c.set_id(n)); sks.append(sk); msgs.append(m); expect.append((n, sk, m))
    ms = c.MixedSigner(engine)
    try:
        for _ in range(2):   # captured on first use, replayed on the second
            sigs, st, dev_ms = ms.sign(set_ids, sks, msgs)
            assert list(st) == [0] * len(msgs) and dev_ms > 0
        for (n, sk, m), sig in zip(expect, sigs):
            assert sig == oracles[n].sign(m, sk), n
    finally:
        ms.close()


def test_group_run_verify_batches(engine):
    """Verify batches of two sets in one graph launch (cuspx_group_run): one
    through the sorted layered verify (its item groups fork onto the batch's
    side streams inside the capture), one through the persistent kernel;
    verdicts equal the oracle's, on the captured launch and its replay."""
    import numpy as np
    import cuspx_gb300 as c
    rng = random.Random(404)
    plan = [("sha256-128f-simple", {"verify_item_max": 0, "verify_mode": 3, "verify_groups": 3}),
            ("shake256-128f-simple", {"verify_item_max": 0, "verify_mode": 2, "verify_sorted_min": 0})]
    batches, want, saved = [], [], {}
    try:
        for name, tune in plan:
            o = _oracle(name)
            sid = engine.set_id(name)
            saved[sid] = engine.get_tuning(sid)
            engine.set_tuning(sid, **tune)
            pk, sk = o.seed_keypair(bytes(rng.randrange(256) for _ in range(3 * o.p.n)))
            msgs = [bytes(rng.randrange(256) for _ in range(rng.randrange(1, 200))) for _ in range(4)]
            sigs = [o.sign(m, sk) for m in msgs]
            bad = bytearray(sigs[2])
            bad[rng.randrange(len(bad))] ^= 0x08
            sigs[2] = bytes(bad)
            n = 40
            pick = [i % 4 for i in range(n)]
            w = [o.verify(sigs[j], msgs[j], pk) for j in range(4)]
            assert w.count(-1) == 1
            want.append([w[j] for j in pick])
            slab, offs, lens = c.pack_messages([msgs[j] for j in pick])
            b = engine.batch(c.OP_VERIFY, sid, n, len(slab), 1)
            b.upload(n, pk, 1, np.zeros(n, dtype=np.uint32), slab, len(slab), offs, lens,
                     np.frombuffer(b"".join(sigs[j] for j in pick), dtype=np.uint8))
            batches.append(b)
        for _ in range(2):   # captured, then replayed
            assert c.group_run(engine, batches) > 0
            for b, w in zip(batches, want):
                v = np.zeros(len(w), dtype=np.int32)
                b.download(None, None, v)
                assert list(v) == w
    finally:
        for b in batches:
            b.close()
        for sid, t in saved.items():
            engine.set_tuning(sid, **t)


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "sha256-192f-simple", "sha256-256f-simple"])
def test_long_messages_two_warp_hashing(engine, setname):
    """Batches holding messages of 2 KiB and more hash those over two warps
    per message (schedule warp + rounds warp) and the rest one thread each;
    signatures and verdicts equal the CPU oracle's on both sides of the
    threshold, with a corrupted and a wrong-length signature mixed in."""
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(2048)
    seed = bytes(rng.randrange(256) for _ in range(3 * o.p.n))
    pk, sk = o.seed_keypair(seed)
    lens = [0, 100, 2047, 2048, 2049, 3000, 20000, 64]
    msgs = [bytes(rng.randrange(256) for _ in range(L)) for L in lens]
    sigs, st = engine.sign_batch(sid, [sk] * len(msgs), msgs)
    assert list(st) == [0] * len(msgs)
    for m, s in zip(msgs, sigs):
        assert s == o.sign(m, sk), len(m)
    bad = bytearray(sigs[6])
    bad[rng.randrange(len(bad))] ^= 0x10
    vsigs = list(sigs) + [bytes(bad), sigs[4]]
    vmsgs = msgs + [msgs[6], msgs[4]]
    siglens = [len(s) for s in vsigs[:-1]] + [len(sigs[4]) - 1]
    want = [o.verify(s, m, pk) for s, m in zip(vsigs[:-1], vmsgs[:-1])] + [-1]
    assert want.count(-1) == 2
    got = engine.verify_batch(sid, [pk] * len(vmsgs), vmsgs, vsigs, siglens=siglens)
    assert list(got) == want


MIB = 1 << 20


@pytest.mark.parametrize("setname", ["sha256-128f-simple", "shake256-256f-simple"])
def test_megabyte_messages_vs_oracle(engine, setname):
    """Messages of 1 MiB - 1, 1 MiB and 1 MiB + 1 bytes (the longest of the
    served stream) beside a short one in one batch.  PRF_msg and H_msg absorb
    the whole message (hash_sha256.cu:99-145, :200-262; hash_shake256.cu:64-77,
    :96-130), so every signature equals the oracle's, and every verdict the
    oracle's, with a corrupted signature and a flipped last message byte."""
    o = _oracle(setname)
    sid = engine.set_id(setname)
    rng = random.Random(1 << 20)
    seed = bytes(rng.randrange(256) for _ in range(3 * o.p.n))
    pk, sk = o.seed_keypair(seed)
    msgs = [rng.randbytes(L) for L in (MIB - 1, MIB, MIB + 1, 64)]
    sigs, st = engine.sign_batch(sid, [sk] * len(msgs), msgs)
    assert list(st) == [0] * len(msgs)
    for m, s in zip(msgs, sigs):
        assert s == o.sign(m, sk), len(m)
    bad = bytearray(sigs[1])
    bad[rng.randrange(len(bad))] ^= 0x08
    flipped = bytearray(msgs[2])
    flipped[-1] ^= 0x01
    vmsgs = msgs + [msgs[1], bytes(flipped)]
    vsigs = list(sigs) + [bytes(bad), sigs[2]]
    want = [o.verify(s, m, pk) for s, m in zip(vsigs, vmsgs)]
    assert want == [0, 0, 0, 0, -1, -1]
    assert list(engine.verify_batch(sid, [pk] * len(vmsgs), vmsgs, vsigs)) == want


def test_null_message_slab_is_refused(engine):
    """A one-shot call with no message buffer but a non-empty message length
    returns CUSPX_EINVAL (nothing is read or launched); with every length 0
    no buffer is needed."""
    import ctypes
    import numpy as np
    import cuspx_gb300 as c
    sid = engine.set_id("sha256-128f-simple")
    z = c.set_sizes(sid)
    _, sks = engine.keypair_batch(sid, [bytes(48)])
    off = np.zeros(1, dtype=np.uint64)
    sig = ctypes.create_string_buffer(z["sig"])
    st = np.zeros(1, dtype=np.int32)
    for ln in (5, 0):
        lens = np.array([ln], dtype=np.uint64)
        rc = engine.L.cuspx_sign_batch(engine.h, sid, 1, sks[0], None, off.ctypes.data, lens.ctypes.data, None, sig,
                                       st.ctypes.data)
        assert rc == (-1 if ln else 0), ln
        v = np.zeros(1, dtype=np.int32)
        rc = engine.L.cuspx_verify_batch(engine.h, sid, 1, bytes(32), None, off.ctypes.data, lens.ctypes.data,
                                         sig, None, v.ctypes.data)
        assert rc == (-1 if ln else 0), ln


@pytest.mark.parametrize("setname", ["shake256-128f-simple", "shake256-256f-simple", "shake256-192f-robust"])
def test_long_messages_warp_sponge(engine, setname):
    """SHAKE messages of 2 KiB and more are hashed one warp per message (the
    sponge state spread over the lanes); signatures and verdicts equal the
    oracle's on both sides of the threshold and on every 136-byte block edge
    of PRF_msg (prefix 2n bytes) and H_msg (prefix 3n bytes), with a
    corrupted and a wrong-length signature mixed in."""
    o = _oracle(setname)
    sid = engine.set_id(setname)
    n = o.p.n
    rng = random.Random(136)
    seed = bytes(rng.randrange(256) for _ in range(3 * n))
    pk, sk = o.seed_keypair(seed)
    lens = [0, 100, 2047, 2048, 2049]
    for pre in (2 * n, 3 * n):
        for d in (-2, -1, 0, 1):
            lens.append(136 * 16 - pre + d)   # the padding byte at a block's last byte, or a new block
    lens += [20000, 64]
    msgs = [rng.randbytes(L) for L in lens]
    sigs, st = engine.sign_batch(sid, [sk] * len(msgs), msgs)
    assert list(st) == [0] * len(msgs)
    for m, s in zip(msgs, sigs):
        assert s == o.sign(m, sk), len(m)
    bad = bytearray(sigs[-2])
    bad[rng.randrange(len(bad))] ^= 0x10
    vsigs = list(sigs) + [bytes(bad), sigs[4]]
    vmsgs = msgs + [msgs[-2], msgs[4]]
    siglens = [len(s) for s in vsigs[:-1]] + [len(sigs[4]) - 1]
    want = [o.verify(s, m, pk) for s, m in zip(vsigs[:-1], vmsgs[:-1])] + [-1]
    assert want.count(-1) == 2
    got = engine.verify_batch(sid, [pk] * len(vmsgs), vmsgs, vsigs, siglens=siglens)
    assert list(got) == want
