"""Shared inputs and comparisons for the tests."""
from __future__ import annotations

import numpy as np

from dawgs_gb300 import mesh

TYPES = [np.float32, np.float64, np.int32, np.int64]
OPS = ["add", "mul", "max", "min"]
TRANS = ["sym", "notrans", "trans"]


def values(n, dtype, op, seed):
    """Field values by op: U[0.5,2] for Mul and U[-1,1] otherwise (floats),
    U[-2^30, 2^30) for integer Add/Max/Min and small integers for Mul."""
    dt = np.dtype(dtype)
    if dt.kind == "f":
        return mesh.uniform_values(n, dt, 0.5, 2.0, seed) if op == "mul" else \
            mesh.uniform_values(n, dt, -1.0, 1.0, seed)
    if op == "mul":
        return mesh.uniform_values(n, dt, -3, 4, seed)
    return mesh.uniform_values(n, dt, -(2 ** 30), 2 ** 30, seed)


def signed_ids(ids, seed, frac4=1):
    """Flag (negate) about frac4/4 of the ids."""
    r = mesh.uniform_values(ids.size, np.int64, 0, 4, seed)
    return np.where(r < frac4, -ids, ids).astype(np.int64)


def random_ids(n, ngroups, seed, zero_frac=0.0):
    """n ids drawn from 1..ngroups (arbitrary multiplicities), some zeroed."""
    ids = mesh.uniform_values(n, np.int64, 1, ngroups + 1, seed)
    if zero_frac > 0:
        z = mesh.uniform_values(n, np.float64, 0.0, 1.0, seed + 1) < zero_frac
        ids[z] = 0
    return ids


def same_bits(a: np.ndarray, b: np.ndarray) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and a.tobytes() == b.tobytes()


def first_diff(a, b):
    av = np.ascontiguousarray(a).view(np.uint8)
    bv = np.ascontiguousarray(b).view(np.uint8)
    d = np.nonzero(av != bv)[0]
    if d.size == 0:
        return None
    i = d[0] // a.dtype.itemsize
    return int(i), a.reshape(-1)[i], b.reshape(-1)[i], int(d.size)
