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
