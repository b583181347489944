"""The device's whole orient3d cascade, restated, against exact arithmetic.

orient3d_sign_filtered (mcut_gb300/csrc/fe_common.cuh) runs four stages: the
fp32 filter, the fp64 stage A (Shewchuk's o3derrboundA), Shewchuk's adaptive
stages B and C (orient3dadapt, shewchuk.c:1962-2085: the rounded
differences' determinant as an expansion, exact when no difference rounded,
then the tails' first-order terms), and an exact sign from expansion
arithmetic over the raw coordinates (Shewchuk, DCG 18, 1997: Two-Sum,
Two-Product by Veltkamp splitting, zero-eliminating expansion sums and
scalings). This module restates the fp64, B/C and exact stages operation for
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
EPS = 1.1102230246251565e-16
O3D_B = (3.0 + 28.0 * EPS) * EPS
O3D_C = (26.0 + 288.0 * EPS) * EPS * EPS
RES = (3.0 + 8.0 * EPS) * EPS


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


def _sign(x):
    return 1 if x > 0.0 else (-1 if x < 0.0 else 0)


def _diff_tail(a, b, x):
    bv = a - x
    av = x + bv
    return (a - av) + (bv - b)


def stage_bc(pa, pb, pc, pd):
    """orient3d_sign_bc: the sign, or None when neither B nor C decides."""
    adx, bdx, cdx = pa[0] - pd[0], pb[0] - pd[0], pc[0] - pd[0]
    ady, bdy, cdy = pa[1] - pd[1], pb[1] - pd[1], pc[1] - pd[1]
    adz, bdz, cdz = pa[2] - pd[2], pb[2] - pd[2], pc[2] - pd[2]
    bdxcdy, cdxbdy, cdxady, adxcdy = bdx * cdy, cdx * bdy, cdx * ady, adx * cdy
    adxbdy, bdxady = adx * bdy, bdx * ady
    perm = (abs(bdxcdy) + abs(cdxbdy)) * abs(adz) + (abs(cdxady) + abs(adxcdy)) * abs(bdz) \
        + (abs(adxbdy) + abs(bdxady)) * abs(cdz)

    def minor2(p, q, r, s):
        a1, a0 = two_product(p, q)
        b1, b0 = two_product(r, s)
        return two_two_diff(a1, a0, b1, b0)
    adet = scale_expansion_zeroelim(minor2(bdx, cdy, cdx, bdy), adz)
    bdet = scale_expansion_zeroelim(minor2(cdx, ady, adx, cdy), bdz)
    cdet = scale_expansion_zeroelim(minor2(adx, bdy, bdx, ady), cdz)
    abdet = fast_expansion_sum_zeroelim(adet, bdet)
    fin = fast_expansion_sum_zeroelim(abdet, cdet)
    assert len(adet) <= 8 and len(abdet) <= 16 and len(fin) <= 24
    det = fin[0]
    for x in fin[1:]:
        det += x
    eb = O3D_B * perm
    if det >= eb or -det >= eb:
        return _sign(det), "B"
    adxt, bdxt, cdxt = _diff_tail(pa[0], pd[0], adx), _diff_tail(pb[0], pd[0], bdx), _diff_tail(pc[0], pd[0], cdx)
    adyt, bdyt, cdyt = _diff_tail(pa[1], pd[1], ady), _diff_tail(pb[1], pd[1], bdy), _diff_tail(pc[1], pd[1], cdy)
    adzt, bdzt, cdzt = _diff_tail(pa[2], pd[2], adz), _diff_tail(pb[2], pd[2], bdz), _diff_tail(pc[2], pd[2], cdz)
    if all(t == 0.0 for t in (adxt, bdxt, cdxt, adyt, bdyt, cdyt, adzt, bdzt, cdzt)):
        return _sign(fin[-1]), "exact differences"
    eb = O3D_C * perm + RES * abs(det)
    det += (adz * ((bdx * cdyt + cdy * bdxt) - (bdy * cdxt + cdx * bdyt)) + adzt * (bdx * cdy - bdy * cdx)) \
        + (bdz * ((cdx * adyt + ady * cdxt) - (cdy * adxt + adx * cdyt)) + bdzt * (cdx * ady - cdy * adx)) \
        + (cdz * ((adx * bdyt + bdy * adxt) - (ady * bdxt + bdx * adyt)) + cdzt * (adx * bdy - ady * bdx))
    if det >= eb or -det >= eb:
        return _sign(det), "C"
    return None, None


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


BC = {"B": 0, "exact differences": 0, "C": 0}


def _cascade_check(a, b, c, d):
    """Per row: the cascade's sign and the stage that decided it; each equals
    the exact sign. Returns the count per stage (fp32, A, B/C, full exact);
    BC counts which of B, the exact-differences return and C decided."""
    decided, sign32, _ = F32.filter_sign(a, b, c, d)
    stages = [0, 0, 0, 0]
    for i in range(len(a)):
        pa, pb, pc, pd = (tuple(float(v) for v in p[i]) for p in (a, b, c, d))
        want = exact(pa, pb, pc, pd)
        full = orient3d_exact_sign(pa, pb, pc, pd)
        assert full == want, (pa, pb, pc, pd)
        if decided[i]:
            got, st = int(sign32[i]), 0
        else:
            got, st = stage_a(pa, pb, pc, pd), 1
            if got is None:
                got, how = stage_bc(pa, pb, pc, pd)
                st = 2
                if got is None:
                    got, st = full, 3
                else:
                    BC[how] += 1
        assert got == want, (pa, pb, pc, pd, st)
        stages[st] += 1
    return stages


def test_cascade_on_coplanar_points():
    rng = np.random.default_rng(31)
    stages = [0, 0, 0, 0]
    for k in (-30, -10, 0, 10, 30):
        a, b, c, d = F32._near_coplanar(rng, 300, 2.0 ** k)
        stages = [s + t for s, t in zip(stages, _cascade_check(a, b, c, d))]
    assert stages[2] + stages[3] > 100  # most of these go past stage A


def test_cascade_on_lattice_zeros_and_near_threshold():
    rng = np.random.default_rng(32)
    a, b, c, d = (rng.integers(-3, 4, size=(800, 3)).astype(np.float64) for _ in range(4))
    st = _cascade_check(a, b, c, d)
    assert st[2] > 0  # lattice zeros: exact differences, decided after B
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


def test_stages_b_and_c_each_decide():
    """Every adaptive exit is taken: B's estimate, the exact-differences
    return (coplanar lattice points at a dyadic offset) and C's corrected
    estimate (differences that rounded, a determinant just past B's bound)."""
    rng = np.random.default_rng(34)
    BC.update({k: 0 for k in BC})
    a, b, c, d = (rng.integers(-40, 41, size=(600, 3)).astype(np.float64) / 8.0 + 2.0 ** 20 for _ in range(4))
    d[:300] = a[:300] + (b[:300] - a[:300]) * 0.5 + (c[:300] - a[:300]) * 0.25
    _cascade_check(a, b, c, d)
    for k in (-20, 0, 20):
        a, b, c, d = F32._near_coplanar(rng, 300, 2.0 ** k, offset=1.0 / 3.0)
        _cascade_check(a, b, c, d)
    assert all(v > 0 for v in BC.values()), BC


def test_exact_zeros_with_rounded_differences_reach_the_full_stage():
    """Points on the plane z = x mixing 2^60-scale and fractional
    coordinates: the differences round, but each row keeps x == z, so B's
    determinant and C's correction are both exactly zero and only the full
    expansion over the raw coordinates decides (zero)."""
    rng = np.random.default_rng(35)
    n = 200
    pts = []
    for _ in range(4):
        x = np.where(rng.random(n) < 0.5, 2.0 ** 60 + 256.0 * rng.integers(-4, 5, n),
                     rng.integers(-64, 65, n) / 4.0)
        y = rng.integers(-64, 65, n) / 8.0
        pts.append(np.stack([x, y, x], axis=1))
    st = _cascade_check(*pts)
    assert st[3] > 0, st
