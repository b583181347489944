"""General-position enforcement (MCGPU_ENFORCE_GENERAL_POSITION[_ABSOLUTE]):
the reference's perturbation re-entry (preproc.cpp:2590-2699, 2933-2945) on
the device. The perturbation must be the reference's sequence (tests/gp_rng.py,
pinned to the C++ library), continued across the dispatches of a context as
the reference's thread_local engines continue across the dispatches of an API
thread, and every attempt's result must equal the oracle's perturbed pass
(pinned to the reference's own functions in test_oracle_pin.py)."""
import ctypes as C

import numpy as np
import pytest

import golden_cases as G
import gp_rng
import oracle
from gpu_util import canonical_records, canonical_tests, sort_rows


def _check(r, want):
    assert r.status == int(want["status"])
    assert r.bad_face == int(want["bad_face"])
    assert G.same_bits(r.cut_eps, want["cut_eps"])
    assert G.same_bits(sort_rows(r.pairs, [0, 1]), want["pairs"])
    t, info = canonical_tests(r.tests, r.test_info)
    assert G.same_bits(t, want["tests"]) and G.same_bits(info, want["test_info"])
    ids, pts = canonical_records(r.record_ids, r.record_points)
    assert G.same_bits(ids, want["rec_ids"]) and G.same_bits(pts, want["rec_pts"])


@pytest.mark.gpu
@pytest.mark.parametrize("absolute", [False, True])
def test_enforced_general_position_on_the_reference_cube(absolute):
    from mcut_gb300 import Context
    m = G.perturbation_cube()
    const = 1.5e-5 if absolute else 1e-4
    ctx = Context(0)  # a fresh perturbation sequence
    try:
        ctx.set_general_position(const, 4)
        assert ctx.general_position() == (const, 4)
        plain = ctx.dispatch(m, m, float_input=True)
        assert plain.status_name == "GP_VIOLATION" and plain.perturbations == 0
        mode = "absolute" if absolute else True
        used = 0
        for _ in range(2):  # the second dispatch continues the sequence
            r = ctx.dispatch(m, m, float_input=True, keep_tests=True, keep_pairs=True,
                             enforce_general_position=mode)
            assert r.status == 0 and r.perturbations >= 1
            used += r.perturbations
            assert r.perturbation == gp_rng.perturbations(used, r.cut_eps)[-1]
            if absolute:
                assert r.cut_eps == const and max(abs(x) for x in r.perturbation) <= const
            want = oracle.front_end(m, m, impl="port", float_input=True, gp_constant=const,
                                    gp_absolute=absolute, perturbation=r.perturbation)
            _check(r, want)
    finally:
        ctx.close()


@pytest.mark.gpu
def test_enforcement_settings_and_scope():
    from mcut_gb300 import Context
    from mcut_gb300 import _lib as L
    ctx = Context(0)
    try:
        assert ctx.general_position() == (1e-4, 4)
        lib = L.load()
        assert lib.mcgpu_context_set_general_position(ctx._h, 0.0, 4) == L.INVALID_VALUE
        assert lib.mcgpu_context_set_general_position(ctx._h, 1e-4, 0) == L.INVALID_VALUE
        # enforcement is per pair: a batch of two is refused
        m = G.perturbation_cube()
        from mcut_gb300.frontend import _as_mesh
        a, ka = _as_mesh(m, True)
        ms = (L.Mesh * 2)(a, a)
        sums = (L.Summary * 2)()
        rc = lib.mcgpu_dispatch_batch(ctx._h, L.RECENTRE | L.VERTEX_ARRAY_FLOAT | L.ENFORCE_GENERAL_POSITION, 2,
                                      ms, ms, None, sums)
        assert rc == L.INVALID_VALUE
        del ka
    finally:
        ctx.close()
