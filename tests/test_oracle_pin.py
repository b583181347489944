"""Re-derive the fixtures from the reference itself where its checkout exists.

Skipped on hosts without the reference sources (the GPU host): there the
committed fixtures (test_oracle_golden.py) stand in for it.
"""
import os

import numpy as np
import pytest

import golden_cases as G
import oracle

REF_ROOT = os.environ.get("MCUT_REF_ROOT", "/root/reference")
pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "source")),
                                reason="reference checkout not present")

CASES = G.all_cases()


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build(ref=True, ref_root=REF_ROOT)


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_is_reference_output(name):
    c = CASES[name]
    r = oracle.front_end(c["src"], c["cut"], impl="ref", float_input=bool(c["float_input"]))
    assert r["status"] == int(c["status"])
    for k in G.FE_KEYS:
        assert G.same_bits(r[k], c[k]), k


def test_port_equals_reference_on_mid_size_case():
    from mcut_gb300 import meshgen
    s, c = meshgen.sphere_heightfield(16.0, level=5, n=160)
    a = oracle.front_end(s, c, impl="ref")
    b = oracle.front_end(s, c, impl="port")
    assert a["status"] == b["status"]
    for k in G.FE_KEYS + ["face_boxes", "src_xyz", "cut_xyz"]:
        assert G.same_bits(a[k], b[k]), k
