"""Pin the CPU oracle's operator to the reference's own code.

oracle/_ref/libogsref.so is libs/ogs/ogsOperator.cpp of the reference,
compiled unmodified against the OCCA and MPI stand-ins in oracle/refstub
(`make -C oracle refop`; only where the reference tree is present).  Over the
oracle's maps it runs the reference's GatherScatter, Gather and Scatter
(ogsOperator.cpp:60-97, 206-238, 311-360 with the Op functors of 36-55), so
the oracle's fold -- and with it every GPU parity test that compares against
the oracle -- is checked against the reference's arithmetic itself: the ogs
identities (Max from -max, which gslib does not share), -0.0, NaN, integer
extremes, every transpose on Signed maps, interleaved k, rows above degree 8.
Both run on this host, so results agree bit for bit, NaN payloads included.
"""
import numpy as np
import pytest

from dawgs_gb300 import mesh
from helpers import OPS, TYPES, first_diff, random_ids, same_bits, signed_ids, values

TRANS = ("sym", "notrans", "trans")


@pytest.fixture(scope="module")
def refop(oracle_mod):
    if not oracle_mod.ogsref_available():
        pytest.skip("the reference's host operator is not built here (no reference tree)")
    return oracle_mod


MESHES = {
    "box_permuted_p3": lambda: mesh.permute_elements(mesh.box_ids(5, 4, 3, 3), 3, seed=1),
    "random_deg1_to_30_zeros": lambda: random_ids(6000, 900, seed=3, zero_frac=0.1),
    "degree_above_8": lambda: np.concatenate([random_ids(3000, 2000, seed=4),
                                              random_ids(1500, 20, seed=5) + 10 ** 6]),
}


@pytest.mark.parametrize("mname", list(MESHES))
@pytest.mark.parametrize("kind", ["unsigned", "signed"])
@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: np.dtype(t).name)
def test_oracle_gather_scatter_is_the_reference_operator(refop, mname, kind, dtype):
    base = MESHES[mname]()
    ids = base if kind == "unsigned" else signed_ids(base, seed=6)
    o = refop.OracleOgs(ids.copy(), kind)
    r = refop.RefOperator(o)
    for op in OPS:
        for trans in TRANS:
            for k in (1, 3):
                v = values(k * ids.size, dtype, op, seed=11 + k)
                a = o.gather_scatter(v.copy(), k, op, trans)
                b = r.gather_scatter(v.copy(), k, op, trans)
                assert same_bits(a, b), (op, trans, k, first_diff(a, b))


@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: np.dtype(t).name)
def test_oracle_gather_and_scatter_are_the_reference_operator(refop, dtype):
    """Signed unique handle, as dawgs' PerformanceTest uses for Gather/Scatter."""
    base = mesh.permute_elements(mesh.box_ids(4, 4, 3, 3), 3, seed=2)
    ids = base.copy()
    o = refop.OracleOgs(ids, "signed", unique=True)
    r = refop.RefOperator(o)
    for op in OPS:
        for trans in TRANS:
            for k in (1, 2):
                v = values(k * ids.size, dtype, op, seed=21)
                a = o.gather(np.zeros(k * o.Ngather, dtype), v, k, op, trans)
                b = r.gather(np.zeros(k * o.Ngather, dtype), v, k, op, trans)
                assert same_bits(a, b), ("gather", op, trans, k, first_diff(a, b))
                v0 = values(k * ids.size, dtype, "add", seed=22)
                sa = o.scatter(v0.copy(), a, k, trans)
                sb = r.scatter(v0.copy(), a, k, trans)
                assert same_bits(sa, sb), ("scatter", op, trans, k, first_diff(sa, sb))


def test_special_values_follow_the_reference_operator(refop):
    """-0.0 in lone and all-(-0.0) rows under Add, NaN and +-inf under every op,
    -DBL_MAX and INT_MIN under Max (whose identity is -max, not INT_MIN)."""
    ids = np.array([1, 2, 2, 3, 3, 3, 4, 5, 5, 6, 6, 7], np.int64)
    o = refop.OracleOgs(ids.copy(), "unsigned")
    r = refop.RefOperator(o)
    nan, inf = np.nan, np.inf
    fv = np.array([-0.0, -0.0, -0.0, nan, 1.0, -inf, -inf, nan, 2.0, -np.finfo(np.float64).max, -0.0, inf])
    for dt in (np.float64, np.float32):
        with np.errstate(over="ignore"):
            x = fv.astype(dt)
        for op in OPS:
            assert same_bits(o.gather_scatter(x.copy(), 1, op), r.gather_scatter(x.copy(), 1, op)), (dt, op)
    for dt in (np.int32, np.int64):
        info = np.iinfo(dt)
        xi = np.array([info.min, info.min, info.max, info.max, 1, info.min, 0, info.max, info.max, -1,
                       info.min, 5], dt)
        for op in OPS:
            assert same_bits(o.gather_scatter(xi.copy(), 1, op), r.gather_scatter(xi.copy(), 1, op)), (dt, op)
