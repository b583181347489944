"""Helpers shared by the GPU parity tests."""
import numpy as np


def sort_rows(a, key_cols):
    a = np.asarray(a)
    if len(a) == 0:
        return a
    order = np.lexsort(tuple(a[:, k] for k in reversed(key_cols)))
    return a[order]


def canonical_tests(tests, info):
    order = np.lexsort((tests[:, 2], tests[:, 1], tests[:, 0]))
    return tests[order], info[order]


def canonical_records(ids, pts):
    order = np.lexsort((ids[:, 2], ids[:, 1], ids[:, 0]))
    return ids[order][:, :3], pts[order]
