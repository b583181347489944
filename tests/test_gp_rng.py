"""The perturbation sequence restated in tests/gp_rng.py against the C++
library's own draws (tests/golden/gp_rng.json, tests/golden/make_gp_rng.py)."""
import json
import os

import gp_rng


def test_restated_sequence_matches_the_cxx_library():
    path = os.path.join(os.path.dirname(__file__), "golden", "gp_rng.json")
    want = [float.fromhex(x) for x in json.load(open(path))["draws_hex"]]
    got = gp_rng.draws(len(want))
    assert all(a == b for a, b in zip(got, want))
    assert all(-1.0 <= x < 1.0 for x in got)
