"""Synthetic inputs for the gather-scatter path: box-mesh global ids and seeded
field values.

``box_ids`` restates dawgs' ``MakeIds`` (dawgsMain.cpp:49-143) for one rank:
an NX x NY x NZ box of hexahedral elements of degree p, element-major, each
element's (p+1)^3 nodes with ``i`` fastest, and global ids lexicographic on the
(NX*p+1)(NY*p+1)(NZ*p+1) node lattice, 1-based so that no id is 0.  Nodes on
shared faces, edges and corners of neighbouring elements get the same id.

Values come from a counter-based splitmix64 stream, so a (seed, index) pair
gives the same number on every machine and numpy version.
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "box_ids", "box_counts", "permute_elements", "uniform_values",
    "splitmix64", "mesh_mix",
]

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def box_ids(nx: int, ny: int, nz: int, p: int) -> np.ndarray:
    """Global ids of a one-rank nx*ny*nz box of degree-p hexes (int64[nx*ny*nz*(p+1)^3]).

    Element (I,J,K) has baseId = I*p + J*p*(p*nx+1) + K*p*(p*nx+1)*(p*ny+1) + 1
    and node (i,j,k) of it the id i + j*(p*nx+1) + k*(p*nx+1)*(p*ny+1) + baseId
    (dawgsMain.cpp:117-140); local index (I + J*nx + K*nx*ny)*Np + i + j*Nq + k*Nq^2.
    """
    if min(nx, ny, nz) < 0 or p < 1:
        raise ValueError("box sizes must be >= 0 and p >= 1")
    nq = p + 1
    sx = p * nx + 1
    sxy = sx * (p * ny + 1)
    I = np.arange(nx, dtype=np.int64)
    J = np.arange(ny, dtype=np.int64)
    K = np.arange(nz, dtype=np.int64)
    # element base ids, ordered K (slowest), J, I (fastest)
    base = (K[:, None, None] * p * sxy + J[None, :, None] * p * sx
            + I[None, None, :] * p + 1).reshape(-1)
    q = np.arange(nq, dtype=np.int64)
    node = (q[:, None, None] * sxy + q[None, :, None] * sx
            + q[None, None, :]).reshape(-1)  # k slowest, i fastest
    return (base[:, None] + node[None, :]).reshape(-1)


def box_counts(nx: int, ny: int, nz: int, p: int) -> dict:
    """Closed-form local/global node counts and row-degree histogram of a box mesh."""
    def axis(n):
        # lattice points along one axis: n-1 interior element boundaries have
        # multiplicity 2, the other n*(p-1)+2 multiplicity 1
        return {1: n * (p - 1) + 2, 2: max(n - 1, 0)}
    ax, ay, az = axis(nx), axis(ny), axis(nz)
    hist = {}
    for mx, cx in ax.items():
        for my, cy in ay.items():
            for mz, cz in az.items():
                d = mx * my * mz
                hist[d] = hist.get(d, 0) + cx * cy * cz
    nlocal = nx * ny * nz * (p + 1) ** 3
    nglobal = (nx * p + 1) * (ny * p + 1) * (nz * p + 1) if nlocal else 0
    return {"local": nlocal, "global": nglobal,
            "rows_by_degree": {d: c for d, c in sorted(hist.items()) if c}}


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser of uint64 counters (Steele, Lea, Flood 2014)."""
    z = (x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def _stream(seed: int, n: int, salt: int = 0) -> np.ndarray:
    with np.errstate(over="ignore"):
        ctr = (np.arange(n, dtype=np.uint64)
               + np.uint64((seed * 0x100000001B3 + salt * 0x9E3779B1) & 0xFFFFFFFFFFFFFFFF))
        return splitmix64(ctr)


def uniform_values(n: int, dtype, lo, hi, seed: int, salt: int = 0) -> np.ndarray:
    """n seeded values, uniform in [lo, hi) (floats) or [lo, hi) integers."""
    bits = _stream(seed, n, salt)
    dt = np.dtype(dtype)
    if dt.kind == "f":
        u = (bits >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return (lo + (hi - lo) * u).astype(dt)
    span = int(hi) - int(lo)
    if span <= 0:
        raise ValueError("empty integer range")
    r = (bits % np.uint64(span)).astype(np.int64) + int(lo)
    return r.astype(dt)


def permute_elements(ids: np.ndarray, p: int, seed: int) -> np.ndarray:
    """Reorder whole elements by a seeded Fisher-Yates permutation."""
    npe = (p + 1) ** 3
    ne = ids.size // npe
    perm = np.arange(ne, dtype=np.int64)
    r = _stream(seed, max(ne, 1), salt=77)
    for i in range(ne - 1, 0, -1):
        j = int(r[i] % np.uint64(i + 1))
        perm[i], perm[j] = perm[j], perm[i]
    return ids.reshape(ne, npe)[perm].reshape(-1).copy()


def mesh_mix(count: int, seed: int, lo: int = 2, hi: int = 16, pmax: int = 7):
    """(nx, ny, nz, p) for `count` meshes: sides uniform in [lo, hi], p in [1, pmax]."""
    r = _stream(seed, 4 * count, salt=991)
    out = []
    for m in range(count):
        nx = lo + int(r[4 * m] % np.uint64(hi - lo + 1))
        ny = lo + int(r[4 * m + 1] % np.uint64(hi - lo + 1))
        nz = lo + int(r[4 * m + 2] % np.uint64(hi - lo + 1))
        p = 1 + int(r[4 * m + 3] % np.uint64(pmax))
        out.append((nx, ny, nz, p))
    return out
