"""Property tests of the host setup against the oracle on random id lists:
duplicates, zeros, flagged (negative) ids and extreme values in any order.
The library's hash-grouping setup must give the oracle's maps, counts and
rewritten ids exactly (ogsSetup.cpp:69-190, 333-433, 569-776), and setup must
refuse what the reference refuses (Unsigned with unique, ogsSetup.cpp:98-100)."""
import numpy as np
import pytest

hyp = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

from dawgs_gb300 import ogs  # noqa: E402

SMALL = st.integers(min_value=-12, max_value=12)
WIDE = st.sampled_from([2 ** 62, -(2 ** 62), 2 ** 31, -(2 ** 31), 2 ** 31 - 1, 2 ** 63 - 1, -(2 ** 63 - 1)])
IDS = st.lists(st.one_of(SMALL, SMALL, SMALL, WIDE), min_size=0, max_size=300).map(
    lambda xs: np.array(xs, dtype=np.int64))


def _same(oracle_mod, ids, kind, unique):
    a, b = ids.copy(), ids.copy()
    ref = oracle_mod.OracleOgs(a, kind, unique)
    g = ogs.ogs_t().Setup(b.size, b, None, ogs.Signed if kind == "signed" else ogs.Unsigned,
                          ogs.Auto, unique, False, None, host_only=True)
    assert (g.N, g.NlocalP, g.NlocalT, g.Ngather, g.NgatherGlobal, g.nnzT, g.nnzN, g.gather_defined) == \
        (ref.N, ref.NlocalP, ref.NlocalT, ref.Ngather, ref.NgatherGlobal, ref.nnzT, ref.nnzN, ref.gather_defined)
    for x, y in zip(g.maps(), ref.maps()):
        assert np.array_equal(x, y)
    assert np.array_equal(a, b)
    # every row lands in exactly one degree bucket
    stats = g.layout_stats()
    deg = np.diff(ref.maps()[0])
    assert sum(stats["rows_by_degree"].values()) + stats["rows_general"] == deg.size
    for d, n in stats["rows_by_degree"].items():
        assert n == int((deg == d).sum())


@settings(max_examples=300, deadline=None, derandomize=True)
@given(IDS)
def test_unsigned_setup_matches_oracle(oracle_mod, ids):
    _same(oracle_mod, ids, "unsigned", False)


@settings(max_examples=300, deadline=None, derandomize=True)
@given(IDS, st.booleans())
def test_signed_setup_matches_oracle(oracle_mod, ids, unique):
    _same(oracle_mod, ids, "signed", unique)


@settings(max_examples=50, deadline=None, derandomize=True)
@given(IDS)
def test_unsigned_unique_is_refused(ids):
    with pytest.raises(ogs.OgsError):
        ogs.ogs_t().Setup(ids.size, ids.copy(), None, ogs.Unsigned, ogs.Auto, True, False, None, host_only=True)


@settings(max_examples=50, deadline=None, derandomize=True)
@given(IDS, st.integers(min_value=0, max_value=300), st.booleans())
def test_int64_min_id_is_refused(ids, where, signed):
    """|INT64_MIN| has no int64 value: setup reports a range error."""
    ids = np.insert(ids, min(where, ids.size), np.iinfo(np.int64).min)
    with pytest.raises(ogs.OgsError):
        ogs.ogs_t().Setup(ids.size, ids.copy(), None, ogs.Signed if signed else ogs.Unsigned, ogs.Auto, False,
                          False, None, host_only=True)


def _check_phases(ph, n):
    """Every slice finds its nodes copied in; no later slice touches nodes
    already copied out; the last chunks cover every node."""
    assert ph[-1][2] == n and ph[-1][3] == n
    prev_d = 0
    for p, (lo, hi, h1, d1) in enumerate(ph):
        assert hi < h1
        assert d1 <= h1
        assert d1 >= prev_d
        for q in range(p + 1, len(ph)):
            assert ph[q][0] >= d1
        prev_d = d1


@settings(max_examples=25, deadline=None, derandomize=True)
@given(st.integers(4, 12), st.integers(4, 12), st.integers(4, 10), st.integers(2, 5), st.integers(0, 2 ** 31),
       st.booleans())
def test_host_pipeline_slices_are_safe_on_random_boxes(nx, ny, nz, p, seed, permute):
    """The host-buffer pipeline's slices on random box meshes, natural or
    element-permuted, keep the copy-in / copy-out invariants."""
    from dawgs_gb300 import mesh
    ids = mesh.box_ids(nx, ny, nz, p)
    if permute:
        ids = mesh.permute_elements(ids, p, seed=seed)
    g = ogs.ogs_t().Setup(ids.size, ids.copy(), host_only=True)
    ph = g.layout_stats()["phases"]
    assert 1 <= len(ph) <= 32
    _check_phases(ph, ids.size)


@st.composite
def _caller_maps(draw):
    """A T map over N local nodes (rows of distinct members, ascending) and an
    N map whose rows are subsequences of the first NrowsN T rows."""
    N = draw(st.integers(1, 40))
    nrows = draw(st.integers(0, 12))
    rows = [sorted(draw(st.sets(st.integers(0, N - 1), max_size=6))) for _ in range(nrows)]
    nrowsN = draw(st.integers(0, nrows))
    rowsN = [sorted(draw(st.sets(st.sampled_from(r), max_size=len(r)))) if (i < nrowsN and r) else []
             for i, r in enumerate(rows)]
    return N, rows, nrowsN, rowsN


def _csr(rows):
    rs = np.zeros(len(rows) + 1, np.int32)
    rs[1:] = np.cumsum([len(r) for r in rows])
    ci = np.array([c for r in rows for c in r], np.int32)
    return rs, ci


@settings(max_examples=200, deadline=None, derandomize=True)
@given(_caller_maps())
def test_setup_maps_round_trip(m):
    """Operators from caller maps (ogsOperator_t-style CSR, as the reference's
    setup builds gatherLocal / gatherHalo / postmpi) keep the maps exactly."""
    N, rows, nrowsN, rowsN = m
    rsT, ciT = _csr(rows)
    rsN, ciN = _csr(rowsN)
    g = ogs.ogs_t().SetupMaps(N, rsT, ciT, rsN, ciN, NrowsN=nrowsN, host_only=True)
    assert (g.N, g.NlocalT, g.NlocalP, g.nnzT, g.nnzN) == (N, len(rows), nrowsN, ciT.size, ciN.size)
    got = g.maps()
    assert np.array_equal(got[0], rsT) and np.array_equal(got[1], ciT)
    assert np.array_equal(got[2], rsN) and np.array_equal(got[3], ciN)
    stats = g.layout_stats()
    deg = np.diff(rsT)
    assert sum(stats["rows_by_degree"].values()) + stats["rows_general"] == len(rows)
    for d, n in stats["rows_by_degree"].items():
        assert n == int((deg == d).sum())


@settings(max_examples=100, deadline=None, derandomize=True)
@given(_caller_maps(), st.integers(0, 2))
def test_setup_maps_refuses_broken_maps(m, how):
    """A column outside [0, N), an N member missing from its T row, or an N
    row at or above NrowsN is refused."""
    N, rows, nrowsN, rowsN = m
    rsT, ciT = _csr(rows)
    rsN, ciN = _csr(rowsN)
    if how == 0:
        if ciT.size == 0:
            return
        ciT = ciT.copy()
        ciT[-1] = N  # outside [0, N)
    elif how == 1:
        cand = [i for i in range(nrowsN) if len(rows[i]) < N]
        if not cand:
            return
        i = cand[0]
        missing = next(c for c in range(N) if c not in rows[i])
        rowsN = [list(r) for r in rowsN]
        rowsN[i] = sorted(set(rowsN[i]) | {missing})
        rsN, ciN = _csr(rowsN)
    else:
        j = next((i for i in range(nrowsN, len(rows)) if rows[i]), None)
        if j is None:
            return
        rowsN = [list(r) for r in rowsN]
        rowsN[j] = [rows[j][0]]
        rsN, ciN = _csr(rowsN)
    with pytest.raises(ogs.OgsError):
        ogs.ogs_t().SetupMaps(N, rsT, ciT, rsN, ciN, NrowsN=nrowsN, host_only=True)


@settings(max_examples=40, deadline=None, derandomize=True)
@given(st.integers(1, 7), st.integers(1, 7), st.integers(1, 7), st.integers(1, 6), st.booleans(), st.integers(0, 99))
def test_box_meshes_match_the_closed_form(nx, ny, nz, p, permute, seed):
    """MakeIds box meshes (dawgsMain.cpp:49-143), natural or element-permuted:
    local and global node counts and the row-degree histogram of the setup
    equal the closed form (lattice points per axis with multiplicity 1 or 2)."""
    from dawgs_gb300 import mesh
    ids = mesh.box_ids(nx, ny, nz, p)
    if permute:
        ids = mesh.permute_elements(ids, p, seed=seed)
    cf = mesh.box_counts(nx, ny, nz, p)
    g = ogs.ogs_t().Setup(ids.size, ids.copy(), host_only=True)
    assert (g.N, g.NgatherGlobal) == (cf["local"], cf["global"])
    assert g.layout_stats()["rows_by_degree"] == cf["rows_by_degree"]
