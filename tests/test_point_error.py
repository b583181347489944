"""Error of the fp64 intersection points against their exact values.

Each record's point is the reference's segment-plane formula evaluated in
fp64 (compute_segment_plane_intersection, math.cpp:249-287, on the plane of
compute_polygon_plane_coefficients, math.cpp:130-239):

    N = Newell sum over the face's vertices (v1, v2, ..., v0 order),
    n = N / |N|, d = <v_first, n>,
    p = q + ((d - <q, n>) / <r - q, n>) (r - q).

The normalisation cancels in the ratio, so the exact point is the rational

    p* = q + (<v_first - q, N> / <r - q, N>) (r - q)

with N summed exactly. For a face whose vertices are exactly coplanar this is
also the exact intersection of the line qr with the face's plane. This module
evaluates p* in rational arithmetic (fractions.Fraction over the recentred
fp64 coordinates the oracle hands out) for every record of every committed
fixture and of the full-size single-pair workload, and bounds |p - p*| (max over components) in ulps of the point's
largest coordinate by a small multiple of the conditioning

    kappa = |r - q| |N| / |<r - q, N>|   (1 / sine of the segment-plane angle).

The device writes every record's point with the same bits as the reference
(the GPU parity tests compare the raw fp64 bits), so the bound measured here
on the fixtures is the device's error too.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

import golden_cases as G
import oracle

CASES = {k: c for k, c in G.all_cases().items() if len(c["rec_ids"])}

# Largest |p - p*| / (kappa * ulp) seen is 4.2 over the fixtures (crack4) and
# 4.5 over the full-size workload's 10,974 records;
# the fp64 formula takes about a dozen roundings, each worth at most half an
# ulp of its operand, so 8 leaves room without hiding a lost digit.
KAPPA_ULPS = 8.0


def _faces(m):
    f = np.asarray(m["f"], dtype=np.int64)
    fs = m.get("fs")
    if fs is None:
        return [list(f[3 * i:3 * i + 3]) for i in range(len(f) // 3)]
    out, o = [], 0
    for s in np.asarray(fs, dtype=np.int64):
        out.append(list(f[o:o + s]))
        o += s
    return out


def point_errors(c):
    """Per record: (|p - p*| in ulps of max|p*_k|, kappa)."""
    r = oracle.front_end(c["src"], c["cut"], float_input=bool(c["float_input"]))
    assert G.same_bits(r["rec_pts"], c["rec_pts"])
    x = np.concatenate([r["src_xyz"], r["cut_xyz"]])
    nsv = len(r["src_xyz"])
    faces = _faces(c["src"]) + [[i + nsv for i in fv] for fv in _faces(c["cut"])]
    memo = {}

    def vx(i):
        if i not in memo:
            memo[i] = [Fraction(float(v)) for v in x[i]]
        return memo[i]

    out = []
    for (q, rr, g), p in zip(c["rec_ids"], c["rec_pts"]):
        fv = faces[int(g)]
        V = [vx(int(fv[(k + 1) % len(fv)])) for k in range(len(fv))]
        N = [Fraction(0)] * 3
        for k in range(len(V)):
            a, b = V[k], V[(k + 1) % len(V)]
            N[0] += (a[1] - b[1]) * (a[2] + b[2])
            N[1] += (a[2] - b[2]) * (a[0] + b[0])
            N[2] += (a[0] - b[0]) * (a[1] + b[1])
        Q, R = vx(int(q)), vx(int(rr))
        d = [R[k] - Q[k] for k in range(3)]
        den = sum(d[k] * N[k] for k in range(3))
        t = sum((V[0][k] - Q[k]) * N[k] for k in range(3)) / den
        pe = [Q[k] + t * d[k] for k in range(3)]
        err = max(abs(Fraction(float(p[k])) - pe[k]) for k in range(3))
        ulp = math.ulp(max(abs(float(v)) for v in pe))
        kappa = (math.sqrt(sum(float(v) ** 2 for v in d)) * math.sqrt(sum(float(v) ** 2 for v in N))
                 / abs(float(den)))
        out.append((float(err) / ulp, max(kappa, 1.0)))
    return out


@pytest.fixture(scope="module")
def errors():
    return {k: point_errors(c) for k, c in sorted(CASES.items())}


@pytest.mark.parametrize("name", sorted(CASES))
def test_point_error_within_conditioned_bound(errors, name):
    for i, (ulps, kappa) in enumerate(errors[name]):
        assert ulps <= KAPPA_ULPS * kappa, (name, i, ulps, kappa)


def test_point_error_report(errors):
    """Summary over all fixture records (6,327): the 5,820 with kappa < 16 stay
    within 22 ulps. Of the other 507, 482 are nearly parallel segments of the
    coplanar-cube fixture (kappa up to 1.2e11) and 12 of two benchmark cases
    (kappa 6.3e6); the conditioned bound covers them all."""
    allr = [e for v in errors.values() for e in v]
    assert len(allr) > 6000
    well = [u for u, k in allr if k < 16]
    assert len(well) > 0.9 * len(allr)
    assert max(well) <= 64
    assert max(u / k for u, k in allr) <= KAPPA_ULPS
    assert float(np.median([u for u, _ in allr])) <= 2


def test_point_error_at_the_headline_size():
    """The single-large-pair workload at full size (327,680 vs 2,093,058
    triangles, coordinates x16): all 10,974 records within the conditioned
    bound, median under one ulp. The device's points at this size carry the
    oracle's bits (the full-size GPU parity test), so these are its errors."""
    from mcut_gb300 import meshgen
    s, c = meshgen.sphere_heightfield(16.0)
    r = oracle.front_end(s, c)
    errs = point_errors(dict(src=s, cut=c, float_input=0, rec_ids=r["rec_ids"], rec_pts=r["rec_pts"]))
    assert len(errs) == 10974
    assert max(u / k for u, k in errs) <= KAPPA_ULPS
    assert float(np.median([u for u, _ in errs])) <= 1
