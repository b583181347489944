"""The device's adaptive orient2d returns the reference's value, bit for bit.

Polygon faces rank their vertex triplets by |orient2d| (the reference's
determine_three_noncollinear_vertices, math.cpp:289-389), so the VALUE of
Shewchuk's adaptive orient2d matters, not only its sign. This module restates
the device's orient2d / orient2d_adapt (mcut_gb300/csrc/fe_common.cuh)
operation for operation on Python doubles. It compares the returned double
with the reference's own compiled orient2d (where the reference checkout
exists) and with the oracle's (pinned to it) on inputs that reach every
adaptive stage: collinear up to rounding, lattice points, large offsets and
tiny differences.
"""
import os

import numpy as np
import pytest

import oracle
from expansions import fast_expansion_sum_zeroelim, two_product, two_two_diff

HAVE_REF = oracle.ref_available()
EPS = 1.1102230246251565e-16
CCW_A = 3.3306690738754716e-16


def two_diff_tail(a, b, x):
    bv = a - x
    av = x + bv
    return (a - av) + (bv - b)


def orient2d_adapt(pa, pb, pc, detsum):
    ccw_b = (2.0 + 12.0 * EPS) * EPS
    ccw_c = (9.0 + 64.0 * EPS) * EPS * EPS
    res = (3.0 + 8.0 * EPS) * EPS
    acx, bcx, acy, bcy = pa[0] - pc[0], pb[0] - pc[0], pa[1] - pc[1], pb[1] - pc[1]
    dl, dlt = two_product(acx, bcy)
    dr, drt = two_product(acy, bcx)
    B = two_two_diff(dl, dlt, dr, drt)
    det = B[0]
    for i in range(1, 4):
        det += B[i]
    eb = ccw_b * detsum
    if det >= eb or -det >= eb:
        return det
    acxt, bcxt = two_diff_tail(pa[0], pc[0], acx), two_diff_tail(pb[0], pc[0], bcx)
    acyt, bcyt = two_diff_tail(pa[1], pc[1], acy), two_diff_tail(pb[1], pc[1], bcy)
    if acxt == 0.0 and acyt == 0.0 and bcxt == 0.0 and bcyt == 0.0:
        return det
    eb = ccw_c * detsum + res * abs(det)
    det += (acx * bcyt + bcy * acxt) - (acy * bcxt + bcx * acyt)
    if det >= eb or -det >= eb:
        return det
    s1, s0 = two_product(acxt, bcy)
    t1, t0 = two_product(acyt, bcx)
    C1 = fast_expansion_sum_zeroelim(B, two_two_diff(s1, s0, t1, t0))
    s1, s0 = two_product(acx, bcyt)
    t1, t0 = two_product(acy, bcxt)
    C2 = fast_expansion_sum_zeroelim(C1, two_two_diff(s1, s0, t1, t0))
    s1, s0 = two_product(acxt, bcyt)
    t1, t0 = two_product(acyt, bcxt)
    D = fast_expansion_sum_zeroelim(C2, two_two_diff(s1, s0, t1, t0))
    assert len(C1) <= 8 and len(C2) <= 12 and len(D) <= 16  # the device's buffers
    return D[-1]


def orient2d(pa, pb, pc):
    dl = (pa[0] - pc[0]) * (pb[1] - pc[1])
    dr = (pa[1] - pc[1]) * (pb[0] - pc[0])
    det = dl - dr
    if dl > 0.0:
        if dr <= 0.0:
            return det
        ds = dl + dr
    elif dl < 0.0:
        if dr >= 0.0:
            return det
        ds = -dl - dr
    else:
        return det
    eb = CCW_A * ds
    if det >= eb or -det >= eb:
        return det
    return orient2d_adapt(pa, pb, pc, ds)


def _inputs(rng):
    out = []
    for k in (-30, -5, 0, 8, 30):
        s = 2.0 ** k
        a, b = s * rng.standard_normal((400, 2)), s * rng.standard_normal((400, 2))
        t = rng.random((400, 1))
        c = a + t * (b - a)  # collinear up to rounding: the adaptive stages
        out += list(zip(a, b, c))
        c2 = c + np.spacing(np.abs(c)) * rng.integers(-3, 4, size=(400, 2))
        out += list(zip(a, b, c2))
    for off in (1e3, 1e8, 2.0 ** 45):
        a = off + rng.standard_normal((400, 2))
        b = off + rng.standard_normal((400, 2))
        c = a + 0.5 * (b - a)
        out += list(zip(a, b, c))
    lat = rng.integers(-4, 5, size=(1200, 3, 2)).astype(np.float64) * 0.125
    out += [(p[0], p[1], p[2]) for p in lat]
    return [tuple(tuple(float(v) for v in p) for p in trip) for trip in out]


def _bits(x):
    return np.float64(x).view(np.uint64)


@pytest.mark.parametrize("impl", ["port", "ref"])
def test_value_matches(impl):
    if impl == "ref" and not HAVE_REF:
        pytest.skip("reference harness not built and MCUT_REF_ROOT unset")
    if impl == "ref":
        oracle.build(ref=True)
    fn = oracle.ref_orient2d if impl == "ref" else oracle.port_orient2d
    rng = np.random.default_rng(41)
    adaptive = 0
    for pa, pb, pc in _inputs(rng):
        got = orient2d(pa, pb, pc)
        want = fn(pa, pb, pc)
        assert _bits(got) == _bits(want), (pa, pb, pc, got, want)
        dl = (pa[0] - pc[0]) * (pb[1] - pc[1])
        dr = (pa[1] - pc[1]) * (pb[0] - pc[0])
        adaptive += abs(dl - dr) < CCW_A * (abs(dl) + abs(dr))
    assert adaptive > 500  # the adaptive stages ran
