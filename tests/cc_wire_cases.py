"""The reference's connected components as mcGetConnectedComponentData hands
them out (tests/golden/cc_wire.npz, made by tests/golden/make_cc_wire.py)."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    """[(case, k, dict(type, vd, vf, face, fsize, adj, adjsize, edge))]"""
    d = np.load(os.path.join(HERE, "golden", "cc_wire.npz"))
    names = sorted({k.split("/")[0] for k in d.files})
    out = []
    for n in names:
        for k in range(int(d[f"{n}/n"])):
            out.append((n, k, {key: d[f"{n}/{k}/{key}"] for key in
                               ("type", "vd", "vf", "face", "fsize", "adj", "adjsize", "edge")}))
    return out
