"""The library's host setup (ogs_setup_ex with OGS_SETUP_HOST_ONLY, no device
needed) builds exactly the oracle's N and T maps and counts: same rows in the
same first-appearance order, same ascending colIds, same NlocalP/NlocalT,
gather_defined and rewritten ids.  The library groups ids with a hash table in
one pass; the oracle sorts -- two algorithms for one contract
(ogsSetup.cpp:69-190, 333-433, 569-776)."""
import numpy as np
import pytest

from dawgs_gb300 import mesh, ogs
from helpers import random_ids, signed_ids

CASES = {
    "c1_box": lambda: mesh.box_ids(10, 10, 10, 3),
    "box_p1": lambda: mesh.box_ids(7, 5, 3, 1),
    "box_permuted": lambda: mesh.permute_elements(mesh.box_ids(6, 5, 4, 4), 4, seed=2),
    "random_multiplicity": lambda: random_ids(20000, 1500, seed=4, zero_frac=0.05),
    "high_degree": lambda: random_ids(5000, 7, seed=8),  # rows of ~700 members
    "all_zero": lambda: np.zeros(100, np.int64),
    "empty": lambda: np.zeros(0, np.int64),
    "single": lambda: np.array([42], np.int64),
    "huge_ids": lambda: np.array([2 ** 62, -(2 ** 62), 3, 2 ** 40, 3, -(2 ** 40)], np.int64),
}


def _compare(oracle_mod, ids, kind, unique):
    a = ids.copy()
    b = ids.copy()
    ref = oracle_mod.OracleOgs(a, kind, unique)
    g = ogs.ogs_t().Setup(b.size, b, None, ogs.Signed if kind == "signed" else ogs.Unsigned,
                          ogs.Auto, unique, False, None, host_only=True)
    assert (g.NlocalP, g.NlocalT, g.Ngather, g.NgatherGlobal, g.nnzT, g.nnzN, g.gather_defined) == \
        (ref.NlocalP, ref.NlocalT, ref.Ngather, ref.NgatherGlobal, ref.nnzT, ref.nnzN, ref.gather_defined)
    for x, y in zip(g.maps(), ref.maps()):
        assert np.array_equal(x, y)
    assert np.array_equal(a, b)  # ids rewritten identically when unique
    return g, ref


@pytest.mark.parametrize("name", list(CASES))
def test_unsigned_maps_match_oracle(oracle_mod, name):
    _compare(oracle_mod, CASES[name](), "unsigned", False)


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("unique", [False, True])
def test_signed_maps_match_oracle(oracle_mod, name, unique):
    ids = CASES[name]()
    _compare(oracle_mod, signed_ids(ids, seed=6) if ids.size else ids, "signed", unique)


def test_layout_covers_every_row(oracle_mod):
    ids = random_ids(30000, 2000, seed=12, zero_frac=0.02)
    g, ref = _compare(oracle_mod, ids, "unsigned", False)
    st = g.layout_stats()
    deg = np.diff(ref.maps()[0])
    hist = np.bincount(deg, minlength=9)
    for d in range(1, 9):
        assert st["rows_by_degree"].get(d, 0) == hist[d]
    assert st["rows_general"] == int((deg > 8).sum())
    assert st["nnz_general"] == int(deg[deg > 8].sum())
    assert st["device_bytes"] == 0  # host-only


def test_c2_box_counts_match_closed_form(oracle_mod):
    """24^3 p=7: 7,077,888 local / 4,826,809 global DOFs and the row-degree histogram."""
    ids = mesh.box_ids(24, 24, 24, 7)
    cf = mesh.box_counts(24, 24, 24, 7)
    g = ogs.ogs_t().Setup(ids.size, ids, host_only=True)
    assert g.N == cf["local"] == 7077888
    assert g.NgatherGlobal == cf["global"] == 4826809
    st = g.layout_stats()
    assert st["rows_by_degree"] == cf["rows_by_degree"] == {1: 3112136, 2: 1470804, 4: 231702, 8: 12167}
    # warp tiles: 32 lanes x 8 entries, i.e. 32 * (8 // d) rows of degree d, per bucket
    want = sum(-(-n // (32 * max(1, 8 // d))) for d, n in cf["rows_by_degree"].items())
    assert st["nwarp_tiles"] == want == 27650
    assert st["ngeneral_tiles"] == 0


def _box_with_zero_block():
    ids = mesh.box_ids(16, 14, 12, 4)
    a = int(ids.size * 0.3)
    ids[a:a + ids.size // 5] = 0  # a block of nodes in no row, inside a four-slice pipeline
    return ids


PIPE_CASES = dict(CASES, box_zero_block=_box_with_zero_block, box_multi_slice=lambda: mesh.box_ids(12, 10, 9, 4))


@pytest.mark.parametrize("name", ["c1_box", "box_permuted", "random_multiplicity", "high_degree", "box_zero_block",
                                  "box_multi_slice"])
def test_host_pipeline_phases_are_safe(oracle_mod, name):
    """The host-buffer pipeline copies node chunks in and out around slices of
    the tiles; every slice must find its nodes already copied in, and no later
    slice may touch nodes that were already copied out."""
    ids = PIPE_CASES[name]()
    g = ogs.ogs_t().Setup(ids.size, ids.copy(), host_only=True)
    st = g.layout_stats()
    ph = st["phases"]
    # gathered rows: the final rows grow to every row; the rows read reach every row by the last slice
    prev_r = 0
    for r1, rn in st["phase_rows"]:
        assert prev_r <= r1 <= g.NlocalT and rn <= g.NlocalT
        prev_r = r1
    assert st["phase_rows"][-1] == (g.NlocalT, g.NlocalT)
    assert 1 <= len(ph) <= 32
    assert ph[-1][2] == ids.size and ph[-1][3] == ids.size
    prev_d = 0
    for p, (lo, hi, h1, d1) in enumerate(ph):
        assert hi < h1  # touched nodes are in chunks 0..p
        assert d1 <= h1  # nothing goes out before it came in
        assert d1 >= prev_d
        for q in range(p + 1, len(ph)):
            assert ph[q][0] >= d1  # later slices stay above the nodes sent back
        prev_d = d1
