"""The device's whole orient3d cascade, restated, against exact arithmetic.

orient3d_sign_filtered (mcut_gb300/csrc/fe_common.cuh) runs three stages: the
fp32 filter, the fp64 stage A (Shewchuk's o3derrboundA), and an exact sign
from expansion arithmetic over the raw coordinates (Shewchuk, DCG 18, 1997:
Two-Sum, Two-Product by Veltkamp splitting, zero-eliminating expansion sums
and scalings). This module restates the fp64 and exact stages operation for
operation on Python floats (IEEE doubles, round to nearest, no fused
multiply-add, as the device build is). With the fp32 filter from
test_fp32_filter.py, it checks every cascade sign against the sign of the
determinant computed in rational arithmetic. The inputs are adversarial:
- coplanar up to rounding, where the exact stage decides;
- exact lattice zeros;
- nearly degenerate configurations at large offsets;
- magnitudes up to 2^60.
The expansion lengths never exceed the device's fixed buffers.
"""
from fractions import Fraction

import numpy as np

import test_fp32_filter as F32
from expansions import (fast_expansion_sum_zeroelim, scale_expansion_zeroelim, two_product,
                        two_two_diff)

O3D_A = 7.7715611723761027e-16


# the device's buffer sizes: t8 8, abc/bcd/cda/dab 12, adet.. 24, abd/cdd 48, det 96
CAP = {"t8": 8, "tri": 12, "scaled": 24, "half": 48, "det": 96}


def orient3d_exact_sign(pa, pb, pc, pd):
    def cross2(p, q):
        a1, a0 = two_product(p[0], q[1])
        b1, b0 = two_product(q[0], p[1])
        return two_two_diff(a1, a0, b1, b0)

    def chk(x, cap):
        assert len(x) <= CAP[cap], (cap, len(x))
        return x
    ab, bc, cd = cross2(pa, pb), cross2(pb, pc), cross2(pc, pd)
    da, ac, bd = cross2(pd, pa), cross2(pa, pc), cross2(pb, pd)
    t8 = chk(fast_expansion_sum_zeroelim(cd, da), "t8")
    cda = chk(fast_expansion_sum_zeroelim(t8, ac), "tri")
    t8 = chk(fast_expansion_sum_zeroelim(da, ab), "t8")
    dab = chk(fast_expansion_sum_zeroelim(t8, bd), "tri")
    bd = [-x for x in bd]
    ac = [-x for x in ac]
    t8 = chk(fast_expansion_sum_zeroelim(ab, bc), "t8")
    abc = chk(fast_expansion_sum_zeroelim(t8, ac), "tri")
    t8 = chk(fast_expansion_sum_zeroelim(bc, cd), "t8")
    bcd = chk(fast_expansion_sum_zeroelim(t8, bd), "tri")
    adet = chk(scale_expansion_zeroelim(bcd, pa[2]), "scaled")
    bdet = chk(scale_expansion_zeroelim(cda, -pb[2]), "scaled")
    cdet = chk(scale_expansion_zeroelim(dab, pc[2]), "scaled")
    ddet = chk(scale_expansion_zeroelim(abc, -pd[2]), "scaled")
    abd = chk(fast_expansion_sum_zeroelim(adet, bdet), "half")
    cdd = chk(fast_expansion_sum_zeroelim(cdet, ddet), "half")
    det = chk(fast_expansion_sum_zeroelim(abd, cdd), "det")
    top = det[-1]
    return 1 if top > 0.0 else (-1 if top < 0.0 else 0)


def stage_a(pa, pb, pc, pd):
    adx, bdx, cdx = pa[0] - pd[0], pb[0] - pd[0], pc[0] - pd[0]
    ady, bdy, cdy = pa[1] - pd[1], pb[1] - pd[1], pc[1] - pd[1]
    adz, bdz, cdz = pa[2] - pd[2], pb[2] - pd[2], pc[2] - pd[2]
    bdxcdy, cdxbdy, cdxady, adxcdy = bdx * cdy, cdx * bdy, cdx * ady, adx * cdy
    adxbdy, bdxady = adx * bdy, bdx * ady
    det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) + cdz * (adxbdy - bdxady)
    perm = (abs(bdxcdy) + abs(cdxbdy)) * abs(adz) + (abs(cdxady) + abs(adxcdy)) * abs(bdz) \
        + (abs(adxbdy) + abs(bdxady)) * abs(cdz)
    eb = O3D_A * perm
    if det > eb:
        return 1
    if -det > eb:
        return -1
    return None


def exact(pa, pb, pc, pd):
    a = [Fraction(x) - Fraction(y) for x, y in zip(pa, pd)]
    b = [Fraction(x) - Fraction(y) for x, y in zip(pb, pd)]
    c = [Fraction(x) - Fraction(y) for x, y in zip(pc, pd)]
    det = a[2] * (b[0] * c[1] - c[0] * b[1]) + b[2] * (c[0] * a[1] - a[0] * c[1]) + c[2] * (a[0] * b[1] - b[0] * a[1])
    return (det > 0) - (det < 0)


def _cascade_check(a, b, c, d):
    """Per row: the cascade's sign and the stage that decided it; each equals
    the exact sign. Returns the count per stage."""
    decided, sign32, _ = F32.filter_sign(a, b, c, d)
    stages = [0, 0, 0]
    for i in range(len(a)):
        pa, pb, pc, pd = (tuple(float(v) for v in p[i]) for p in (a, b, c, d))
        want = exact(pa, pb, pc, pd)
        if decided[i]:
            got, st = int(sign32[i]), 0
        else:
            got, st = stage_a(pa, pb, pc, pd), 1
            if got is None:
                got, st = orient3d_exact_sign(pa, pb, pc, pd), 2
        assert got == want, (pa, pb, pc, pd, st)
        stages[st] += 1
    return stages


def test_cascade_on_coplanar_points():
    rng = np.random.default_rng(31)
    stages = [0, 0, 0]
    for k in (-30, -10, 0, 10, 30):
        a, b, c, d = F32._near_coplanar(rng, 300, 2.0 ** k)
        stages = [s + t for s, t in zip(stages, _cascade_check(a, b, c, d))]
    assert stages[2] > 100  # most of these need the exact stage


def test_cascade_on_lattice_zeros_and_near_threshold():
    rng = np.random.default_rng(32)
    a, b, c, d = (rng.integers(-3, 4, size=(800, 3)).astype(np.float64) for _ in range(4))
    st = _cascade_check(a, b, c, d)
    assert st[2] > 0
    a, b, c, d = F32._off_plane(rng, 1500, 1.0)
    st = _cascade_check(a, b, c, d)
    assert st[0] > 0 and st[1] > 0


def test_cascade_at_large_offsets_and_magnitudes():
    rng = np.random.default_rng(33)
    for off, scale in ((1e6, 1e-3), (3e9, 1.0), (2.0 ** 50, 2.0 ** 10)):
        a, b, c, d = F32._near_coplanar(rng, 300, scale, offset=off)
        _cascade_check(a, b, c, d)
    big = 2.0 ** 60
    a, b, c, d = (big * rng.standard_normal((300, 3)) for _ in range(4))
    d = a + 0.5 * (b - a) + 0.25 * (c - a)
    _cascade_check(a, b, c, d)
