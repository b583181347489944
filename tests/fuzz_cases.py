"""Seeded random mesh pairs shared by the port-vs-reference pin and the GPU
parity run over the same inputs.

Each family returns a list of (src, cut, kwargs) with kwargs for the front
end (float_input, gp_constant, gp_absolute):

    fracture   noisy icosphere vs rotated, displaced grid
    lattice    the same snapped to a 1/8 lattice: coplanar faces, vertices on
               faces, edges through edges (mostly general-position violations)
    collapsed  snapped to a 1/2 lattice: faces collapse (degenerate status)
    quads      quad meshes (face sizes given), planar or warped
    float32    float vertex arrays; with vary_constant, the cut-box constant
               varied, relative and absolute
"""
import numpy as np

from mcut_gb300 import meshgen as M


def _lattice(m, step):
    return dict(v=np.round(m["v"] / step) * step, f=m["f"], fs=m["fs"])


def _quads(n, h, rng, warp):
    g = M.grid(n, h)
    i = np.arange(n - 1)
    I, J = np.meshgrid(i, i, indexing="xy")
    a = (J * n + I).ravel()
    f = np.stack([a, a + 1, a + n + 1, a + n], 1).astype(np.uint32)
    v = g["v"].copy()
    v[:, 2] += rng.uniform(-warp, warp, len(v))
    return dict(v=v, f=f.ravel(), fs=np.full(len(f), 4, np.uint32))


def fracture(seed, count=25):
    rng = np.random.default_rng(M.SEED_BASE + 100 + seed)
    return [M.crack_pair(rng, level=int(rng.integers(1, 4)), n=int(rng.integers(4, 24))) + ({},)
            for _ in range(count)]


def lattice(seed, count=25):
    rng = np.random.default_rng(M.SEED_BASE + 200 + seed)
    out = []
    for _ in range(count):
        s, c = M.crack_pair(rng, level=int(rng.integers(1, 3)), n=int(rng.integers(3, 9)))
        out.append((_lattice(s, 0.125), _lattice(c, 0.125), {}))
    return out


def collapsed(count=40):
    rng = np.random.default_rng(M.SEED_BASE + 300)
    out = []
    for _ in range(count):
        s, c = M.crack_pair(rng, level=int(rng.integers(1, 3)), n=int(rng.integers(3, 9)))
        out.append((_lattice(s, 0.5), _lattice(c, 0.5), {}))
    return out


def quads(warp, count=10):
    rng = np.random.default_rng(M.SEED_BASE + 400)
    out = []
    for _ in range(count):
        s = M.icosphere(int(rng.integers(1, 3)), 1.0)
        c = _quads(int(rng.integers(3, 10)), 1.5, rng, warp)
        c["v"] = c["v"] @ M._rotation(rng).T + rng.uniform(-0.3, 0.3, 3)
        out.append((s, c, {}))
    return out


def float32(absolute, vary_constant=True, count=12):
    rng = np.random.default_rng(M.SEED_BASE + 500 + int(absolute))
    out = []
    for _ in range(count):
        s, c = M.crack_pair(rng, level=2, n=int(rng.integers(4, 16)))
        const = float(rng.choice([1e-4, 1e-3, 1e-2]))
        kw = dict(float_input=True)
        if vary_constant:
            kw.update(gp_absolute=absolute, gp_constant=const)
        out.append((s, c, kw))
    return out
