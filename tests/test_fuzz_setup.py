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


@settings(max_examples=300, deadline=None)
@given(IDS)
def test_unsigned_setup_matches_oracle(oracle_mod, ids):
    _same(oracle_mod, ids, "unsigned", False)


@settings(max_examples=300, deadline=None)
@given(IDS, st.booleans())
def test_signed_setup_matches_oracle(oracle_mod, ids, unique):
    _same(oracle_mod, ids, "signed", unique)


@settings(max_examples=50, deadline=None)
@given(IDS)
def test_unsigned_unique_is_refused(ids):
    with pytest.raises(ogs.OgsError):
        ogs.ogs_t().Setup(ids.size, ids.copy(), None, ogs.Unsigned, ogs.Auto, True, False, None, host_only=True)


@settings(max_examples=50, deadline=None)
@given(IDS, st.integers(min_value=0, max_value=300), st.booleans())
def test_int64_min_id_is_refused(ids, where, signed):
    """|INT64_MIN| has no int64 value: setup reports a range error."""
    ids = np.insert(ids, min(where, ids.size), np.iinfo(np.int64).min)
    with pytest.raises(ogs.OgsError):
        ogs.ogs_t().Setup(ids.size, ids.copy(), None, ogs.Signed if signed else ogs.Unsigned, ogs.Auto, False,
                          False, None, host_only=True)
