"""Re-derive the fixtures from the reference itself where its checkout exists.

Skipped on hosts without the reference sources (the GPU host): there the
committed fixtures (test_oracle_golden.py) stand in for it.
"""
import os

import numpy as np
import pytest

import golden_cases as G
import oracle

pytestmark = pytest.mark.skipif(not oracle.ref_available(),
                                reason="reference harness not built and MCUT_REF_ROOT unset")

CASES = G.all_cases()


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build(ref=True)


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


def _same(a, b):
    assert a["status"] == b["status"] and G.same_bits(a["cut_eps"], b["cut_eps"])
    for k in ("pairs", "tests", "test_info", "rec_ids", "rec_pts", "cut_xyz", "face_boxes"):
        assert G.same_bits(a[k], b[k]), k


@pytest.mark.parametrize("absolute", [False, True])
def test_perturbed_pass_matches_reference(absolute):
    """One general-position enforcement attempt (the cut vertices of the
    narrow phase plus the perturbation, the unperturbed pairs and boxes):
    the restatement against the reference's own functions, for the
    reference's perturbation test case and its first perturbations."""
    import gp_rng
    m = G.perturbation_cube()
    const = 1.5e-5 if absolute else 1e-4
    base = oracle.front_end(m, m, impl="port", float_input=True, gp_constant=const, gp_absolute=absolute)
    assert base["status"] == 1  # general position violated
    for p in gp_rng.perturbations(3, base["cut_eps"]):
        a = oracle.front_end(m, m, impl="port", float_input=True, gp_constant=const, gp_absolute=absolute,
                             perturbation=p)
        b = oracle.front_end(m, m, impl="ref", float_input=True, gp_constant=const, gp_absolute=absolute,
                             perturbation=p)
        _same(a, b)
        assert G.same_bits(a["face_boxes"], base["face_boxes"]) and G.same_bits(a["pairs"], base["pairs"])


@pytest.mark.parametrize("name", ["two_spheres", "crack3"])
def test_perturbed_pass_matches_reference_on_fixtures(name):
    import gp_rng
    c = CASES[name]
    fin = bool(c["float_input"])
    base = oracle.front_end(c["src"], c["cut"], impl="port", float_input=fin)
    p = gp_rng.perturbations(1, base["cut_eps"])[0]
    _same(oracle.front_end(c["src"], c["cut"], impl="port", float_input=fin, perturbation=p),
          oracle.front_end(c["src"], c["cut"], impl="ref", float_input=fin, perturbation=p))
