"""The resident-tree walk never misses a candidate pair: CPU restatement of
k_traverse_resident's query mapping.

A resident cut mesh's tree holds fp32 boxes (rounded outward) of its faces
in user coordinates x; a pair sees the cut vertices as x' = (x - com) + t
(two fp64 roundings, preproc.cpp:147-181) and its cut boxes enlarged by eps.
The walk maps a pair-frame query box q back with the shift com - t, widens
it by eps and by the margin 2^-48 (|q.lo| + |q.hi| + eps + 2 |com| + 2 |t|
+ 2 mag), and rounds it outward to fp32. Whenever q meets a cut face's
enlarged pair-frame box (the closed fp64 test the leaves then make), the
mapped box must meet the face's fp32 user box. Checked here on random
faces, frames of every magnitude and query boxes that touch the enlarged
box exactly on one side, in fp64 arithmetic as the device does it.
"""
import numpy as np

INF = np.inf


def f32_down(x):
    f = x.astype(np.float32)
    return np.where(f.astype(np.float64) > x, np.nextafter(f, np.float32(-INF)), f)


def f32_up(x):
    f = x.astype(np.float32)
    return np.where(f.astype(np.float64) < x, np.nextafter(f, np.float32(INF)), f)


def _trial(rng, n, scale, off_scale):
    # user coordinates of n triangles near `off`, the frame com, t
    off = rng.uniform(-off_scale, off_scale, size=(n, 1, 3))
    x = off + rng.uniform(-scale, scale, size=(n, 3, 3))
    com = rng.uniform(-off_scale, off_scale, size=(n, 1, 3)) + off * rng.uniform(0.9, 1.1, size=(n, 1, 1))
    t = rng.uniform(-1, 1, size=(n, 1, 3)) * scale * rng.uniform(1, 100, size=(n, 1, 1))
    xp = (x - com) + t                                   # pair frame, two roundings
    eps = np.abs(rng.normal(0, 1e-4, size=(n, 1))) * scale * rng.integers(0, 2, size=(n, 1))
    lo_p, hi_p = xp.min(axis=1), xp.max(axis=1)          # exact pair-frame box
    lo_e, hi_e = lo_p - eps, hi_p + eps                  # enlarged (fp64)
    # a query box touching the enlarged box on one side of one axis, else overlapping
    q_lo = lo_e + rng.uniform(-scale, 0, size=(n, 3)) * rng.integers(0, 2, size=(n, 3))
    q_hi = hi_e - rng.uniform(-scale, 0, size=(n, 3)) * rng.integers(0, 2, size=(n, 3))
    ax = rng.integers(0, 3, size=n)
    side = rng.integers(0, 2, size=n)
    r = np.arange(n)
    w = rng.uniform(0, scale, size=n)
    # q entirely below (q_hi == lo_e) or above (q_lo == hi_e) on axis ax: a touch
    q_hi[r[side == 0], ax[side == 0]] = lo_e[r[side == 0], ax[side == 0]]
    q_lo[r[side == 0], ax[side == 0]] = lo_e[r[side == 0], ax[side == 0]] - w[side == 0]
    q_lo[r[side == 1], ax[side == 1]] = hi_e[r[side == 1], ax[side == 1]]
    q_hi[r[side == 1], ax[side == 1]] = hi_e[r[side == 1], ax[side == 1]] + w[side == 1]
    meets = np.all((q_lo <= hi_e) & (q_hi >= lo_e), axis=1)
    # the walk's mapped query box
    c3, t3 = com[:, 0, :], t[:, 0, :]
    sh = c3 - t3
    mag = np.abs(x).max(axis=1)                          # a bound on the mesh's |coordinates| per axis
    m = 2.0 ** -48 * (np.abs(q_lo) + np.abs(q_hi) + eps + 2.0 * (np.abs(c3) + np.abs(t3)) + 2.0 * mag)
    ql = f32_down(((q_lo - eps) + sh) - m)
    qh = f32_up(((q_hi + eps) + sh) + m)
    # the face's fp32 user box (the tree's leaf box contains it)
    ul, uh = f32_down(x.min(axis=1)), f32_up(x.max(axis=1))
    hit = np.all((ql <= uh) & (qh >= ul), axis=1)
    return meets, hit


def test_mapped_query_boxes_are_conservative():
    rng = np.random.default_rng(20261204)
    total = 0
    for scale in (1e-3, 1.0, 37.5, 1e4):
        for off_scale in (0.0, 1.0, 1e3, 1e6):
            meets, hit = _trial(rng, 20000, scale, max(off_scale, scale))
            assert meets.sum() > 1000
            # every pair the exact test keeps is reached by the walk
            assert np.all(hit[meets]), (scale, off_scale, np.count_nonzero(meets & ~hit))
            total += int(meets.sum())
    assert total > 100000


def test_margin_is_far_below_fp32_rounding():
    """The margin costs nothing measurable: it is below the fp32 outward
    rounding of the boxes by a factor of about 2^20 at any magnitude."""
    for v in (1e-3, 1.0, 1e3, 1e6):
        m = 2.0 ** -48 * 8 * v
        assert m < np.spacing(np.float32(v)) * 2.0 ** -17
