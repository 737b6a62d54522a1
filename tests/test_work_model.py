"""The work model behind bench.py's roofline fractions.

`leaf_units` counts the hash units (SHA-256 compressions or Keccak-f
permutations) of one XMSS leaf.  A key generation is one treehash of the top
layer (crypto_sign_seed_keypair, sign.cu:154-182): 2^hp leaves and 2^hp - 1
H calls, so the leaf model is pinned by the keygen unit counts of the
reference's structure, counted per call site: SHA-256 H is one compression at
n = 16 and two at n = 24 (22 + 2n + 9 > 64 bytes after the midstate); a
SHAKE-256 H absorbs 32 + 3n <= 135 bytes in one permutation.
"""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_model", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name,hp,h_units,keygen_units", [
    ("sha256-128f-simple", 3, 1, 4567),
    ("sha256-192f-simple", 3, 2, 6702),
    ("shake256-256f-simple", 4, 1, 17439),
])
def test_leaf_units_match_keygen_work(name, hp, h_units, keygen_units):
    b = _bench()
    assert (1 << hp) * b.leaf_units(name) + ((1 << hp) - 1) * h_units == keygen_units


def test_headline_constants_follow_the_model():
    b = _bench()
    assert b.leaf_units("sha256-128f-simple") == 35 * 16 + 10
    assert b.KEYGEN_CMP_128F == 8 * b.leaf_units("sha256-128f-simple") + 7


@pytest.mark.parametrize("name", ["sha256-128f-simple", "sha256-192f-robust", "shake256-128f-robust",
                                  "shake256-192f-simple"])
def test_unit_model_matches_oracle_counts(name):
    """unit_model against the hash units the oracle counts while it runs the
    reference's crypto_sign_signature / crypto_sign_verify: the message-
    independent part of a signature is exact once message hashing (msg_units)
    and wots_sign are taken out, and the message-dependent parts (wots_sign's
    chains, verify's chain steps) match their expectation over messages."""
    import random
    import statistics
    import spx_oracle as so
    b = _bench()
    o = so.Oracle(name)
    m = b.unit_model(name)
    rng = random.Random(5)
    pk, sk = o.seed_keypair(bytes(rng.randrange(256) for _ in range(o.p.seed_bytes)))
    idx = 1 if m["hash"] == "shake256" else 0
    wots, steps = [], []
    for t in range(6):
        msg = bytes(rng.randrange(256) for _ in range(40 + 173 * t))
        so.units_reset()
        sig = o.sign(msg, sk)
        u = so.units()
        assert u[idx] - u[2] - b.msg_units(name, "sign", len(msg)) == m["sign_fixed"], t
        assert u[1 - idx] == 0
        wots.append(u[2])
        so.units_reset()
        assert o.verify(sig, msg, pk) == 0
        u = so.units()
        steps.append((u[idx] - b.msg_units(name, "verify", len(msg)) - m["verify_fixed"]) / m["F"])
    assert abs(statistics.mean(wots) / m["wots_sign"] - 1) < 0.05
    assert abs(statistics.mean(steps) / m["verify_chain_steps"] - 1) < 0.05


@pytest.mark.parametrize("name,mlen", [("sha256-128f-simple", 0), ("sha256-128f-simple", 1000),
                                       ("sha256-256f-simple", 55), ("shake256-256f-simple", 5000)])
def test_message_units_match_oracle(name, mlen):
    """msg_units against the oracle's PRF_msg and H_msg over one message."""
    import spx_oracle as so
    b = _bench()
    o = so.Oracle(name)
    n = o.p.n
    idx = 1 if name.startswith("shake") else 0
    msg = bytes(range(256)) * (mlen // 256) + bytes(mlen % 256)
    so.units_reset()
    o.L.spxo_gen_message_random(o.p, bytes(n), bytes(n), bytes(n), msg, len(msg))
    prf = so.units()[idx]
    so.units_reset()
    o.hash_message(bytes(n), bytes(2 * n), msg)
    hm = so.units()[idx]
    assert hm == b.msg_units(name, "verify", mlen)
    assert prf + hm == b.msg_units(name, "sign", mlen)
