"""Seeded synthetic meshes for the intersection front end.

Every workload here is generated: there is no public mesh suite behind the
reference's numbers. A mesh is a dict with
    v  : float64 [V, 3]  vertex coordinates (user space)
    f  : uint32  [sum of face sizes] flattened face-vertex indices
    fs : uint32  [F] face sizes, or None for an all-triangle mesh (the
         reference's ``pFaceSizes == nullptr`` convention, preproc.cpp:206)

Workloads (sizes from the reference's configuration list):
    two_spheres()        level-3 icosphere pair (642 verts / 1280 tris each)
    sphere_heightfield() level-7 noisy icosphere vs 1024x1024 height field
    cube_coplanar()      512^2-per-face lattice cube vs 256^2 coplanar grid
    batch_pairs()        4096 independent sphere / crack-grid pairs
Each takes ``scale`` (a power of two, exact in fp64). The reference rejects
faces with |Newell normal|^2 < 1e-9 (math.cpp:151-152) as degenerate, which
the two large workloads hit at scale 1; scale=16 is their valid variant.
"""
from __future__ import annotations

import math

import numpy as np

SEED_BASE = 0xC0FFEE


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
         (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
         (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
         (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(v, dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, np.array(f, dtype=np.int64)


def icosphere(level: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Subdivided icosahedron projected to the sphere: 10*4^L+2 verts, 20*4^L tris.

    Subdivision is vectorised: every face splits into four, midpoints of
    shared edges are deduplicated by their sorted endpoint pair.
    """
    v, f = _icosahedron()
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1) + nv  # m[0]=mid(01) m[1]=mid(12) m[2]=mid(20)
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], m[0], m[2]], 1),
            np.stack([f[:, 1], m[1], m[0]], 1),
            np.stack([f[:, 2], m[2], m[1]], 1),
            np.stack([m[0], m[1], m[2]], 1)])
    v = v * radius + np.asarray(center, dtype=np.float64)
    return dict(v=np.ascontiguousarray(v), f=f.astype(np.uint32).ravel(), fs=None)


def grid(n: int, half_extent: float, z=None):
    """n x n vertex grid over [-h, h]^2 in the z=0 plane (2(n-1)^2 tris)."""
    xs = np.linspace(-half_extent, half_extent, n)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    Z = np.zeros_like(X) if z is None else z(X, Y)
    v = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    i = np.arange(n - 1)
    I, J = np.meshgrid(i, i, indexing="xy")
    a = (J * n + I).ravel()
    b, c, d = a + 1, a + n, a + n + 1
    f = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)]).astype(np.uint32)
    return dict(v=np.ascontiguousarray(v), f=f.ravel(), fs=None)


def _scale(m, s):
    return dict(v=m["v"] * s, f=m["f"], fs=m["fs"])


def two_spheres(scale: float = 1.0):
    """Level-3 icosphere r=1 at the origin vs r=0.8 at (0.5, 0.3, 0.1)."""
    src = icosphere(3, 1.0)
    cut = icosphere(3, 0.8, (0.5, 0.3, 0.1))
    return _scale(src, scale), _scale(cut, scale)


def sphere_heightfield(scale: float = 1.0, level: int = 7, n: int = 1024, seed: int = SEED_BASE + 2):
    """Noisy level-7 icosphere vs an open height field cutting through it."""
    rng = np.random.default_rng(seed)
    src = icosphere(level, 1.0)
    r = 1.0 + rng.normal(0.0, 0.01, size=src["v"].shape[0])
    src["v"] = src["v"] * r[:, None]
    amp = 0.05
    k = rng.uniform(1.0, 8.0, size=(8, 2)) * rng.choice([-1.0, 1.0], size=(8, 2))
    phi = rng.uniform(0.0, 2.0 * np.pi, size=8)

    def height(X, Y):
        z = np.zeros_like(X)
        for j in range(8):
            z += amp * np.sin(k[j, 0] * X + k[j, 1] * Y + phi[j])
        return z + 0.1

    cut = grid(n, 1.5, height)
    return _scale(src, scale), _scale(cut, scale)


def cube_lattice(m: int):
    """Closed cube surface [0,m]^3 on the integer lattice, m x m quads per side, 2 tris each, outward."""
    # all lattice points of the (m+1)^3 cube, keep the surface ones
    g = np.arange(m + 1)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    on = (X == 0) | (X == m) | (Y == 0) | (Y == m) | (Z == 0) | (Z == m)
    lut = -np.ones((m + 1,) * 3, dtype=np.int64)
    lut[on] = np.arange(int(on.sum()))
    v = np.stack([X[on], Y[on], Z[on]], 1).astype(np.float64)
    fl = []
    i = np.arange(m)
    I, J = np.meshgrid(i, i, indexing="ij")
    I, J = I.ravel(), J.ravel()
    for axis in range(3):
        u, w = [a for a in range(3) if a != axis]
        for side in (0, m):
            corners = []
            for (di, dj) in ((0, 0), (1, 0), (1, 1), (0, 1)):
                p = [None, None, None]
                p[axis] = np.full_like(I, side)
                p[u] = I + di
                p[w] = J + dj
                corners.append(lut[p[0], p[1], p[2]])
            q = np.stack(corners, 1)
            if (side == 0) ^ (axis == 1):
                q = q[:, ::-1]
            fl.append(np.stack([q[:, 0], q[:, 1], q[:, 2]], 1))
            fl.append(np.stack([q[:, 0], q[:, 2], q[:, 3]], 1))
    f = np.concatenate(fl).astype(np.uint32)
    return dict(v=v, f=f.ravel(), fs=None)


def cube_coplanar(scale: float = 1.0, m: int = 512, n: int = 256, seed: int = SEED_BASE + 3):
    """Lattice cube (m^2 quads per side, lattice * 2^-9) vs an n x n grid lying
    in its top face plane, each grid vertex nudged by U(-1e-12, 1e-12) in z."""
    rng = np.random.default_rng(seed)
    src = cube_lattice(m)
    src["v"] = src["v"] * (1.0 / 512.0)
    top = m / 512.0
    lo, hi = -0.125 * top, 1.125 * top
    cut = grid(n, 0.5, None)
    v = cut["v"]
    v[:, 0] = (v[:, 0] + 0.5) * (hi - lo) + lo
    v[:, 1] = (v[:, 1] + 0.5) * (hi - lo) + lo
    v[:, 2] = top + rng.uniform(-1e-12, 1e-12, size=v.shape[0])
    return _scale(src, scale), _scale(cut, scale)


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def crack_pair(rng, level=None, n=None, target_tris=None):
    """One fracture-like pair: noisy icosphere vs a rotated, z-displaced grid."""
    if target_tris is not None:
        # split the budget between the two meshes
        level = int(np.clip(round(math.log(max(target_tris / 2, 20) / 20.0, 4)), 1, 7))
        n = int(np.clip(round(math.sqrt(max(target_tris / 2, 8) / 2.0)) + 1, 4, 1024))
    if level is None:
        level = int(rng.integers(2, 6))
    if n is None:
        n = int(rng.integers(8, 129))
    r = rng.uniform(0.5, 1.5)
    src = icosphere(level, r)
    src["v"] = src["v"] * (1.0 + rng.normal(0.0, 0.005, size=src["v"].shape[0]))[:, None]
    cut = grid(n, 1.5 * r)
    cut["v"][:, 2] = rng.normal(0.0, 0.02, size=cut["v"].shape[0])
    R = _rotation(rng)
    off = rng.uniform(-0.3, 0.3, size=3)
    cut["v"] = cut["v"] @ R.T + off
    return src, cut


def batch_pairs(count: int = 4096, seed: int = SEED_BASE + 4):
    """The batched workload: ``count`` independent crack pairs."""
    rng = np.random.default_rng(seed)
    return [crack_pair(rng) for _ in range(count)]


def read_off(path):
    """Minimal OFF reader (vertex count, face count, then 'n i0 .. in-1' rows)."""
    toks = []
    with open(path) as fh:
        for line in fh:
            line = line.split("#", 1)[0].strip()
            if line:
                toks.append(line.split())
    assert toks[0][0] == "OFF"
    head = toks[1] if len(toks[0]) == 1 else toks[0][1:]
    body = toks[2:] if len(toks[0]) == 1 else toks[1:]
    nv, nf = int(head[0]), int(head[1])
    v = np.array([[float(x) for x in r[:3]] for r in body[:nv]], dtype=np.float64).reshape(nv, 3)
    fs, f = [], []
    for r in body[nv:nv + nf]:
        k = int(r[0])
        fs.append(k)
        f.extend(int(x) for x in r[1:1 + k])
    fs = np.array(fs, dtype=np.uint32)
    return dict(v=v, f=np.array(f, dtype=np.uint32), fs=None if np.all(fs == 3) else fs)


def num_faces(m):
    return int(m["fs"].shape[0]) if m["fs"] is not None else int(m["f"].shape[0] // 3)
