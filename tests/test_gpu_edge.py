"""Edge cases on the GPU, each against the oracle bit for bit: empty and
all-zero id lists, single nodes, rows above the exact-degree buckets (the
reference aborts above 512 members, ogsOperator.cpp:459-465; here they run),
-0.0 under Add, NaN under Max/Min, integer extremes, ill-defined Gather."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import _lib, mesh, ogs
from helpers import first_diff, random_ids, same_bits

pytestmark = pytest.mark.gpu


def gs(g, v, k, op, trans=ogs.Sym):
    d = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    g.GatherScatter(d, k, op, trans)
    torch.cuda.synchronize()
    return d.cpu().numpy()


def test_empty_and_zero_ids(cuda, oracle_mod):
    g = ogs.ogs_t().Setup(0, np.zeros(0, np.int64))
    assert (g.N, g.NlocalT, g.NgatherGlobal) == (0, 0, 0)
    g.GatherScatter(torch.zeros(0, dtype=torch.float64, device="cuda"), 1, ogs.Add, ogs.Sym)
    z = np.zeros(1000, np.int64)
    g = ogs.ogs_t().Setup(z.size, z.copy())
    v = np.linspace(-1, 1, 1000)
    assert same_bits(gs(g, v, 1, ogs.Add), v)  # nothing takes part
    ids = np.where(np.arange(5000) % 3 == 0, 0, mesh.box_ids(5, 5, 5, 3)[:5000]).astype(np.int64)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    v = np.linspace(-3, 3, ids.size)
    assert same_bits(gs(g, v, 1, ogs.Add), ref.gather_scatter(v.copy(), 1, "add", "sym"))


def test_single_node_and_gather_of_ill_defined(cuda):
    g = ogs.ogs_t().Setup(1, np.array([7], np.int64))
    assert same_bits(gs(g, np.array([2.5]), 1, ogs.Add), np.array([2.5]))
    ids = np.array([1, 1, 2], np.int64)
    g = ogs.ogs_t().Setup(3, ids.copy())  # Unsigned, group 1 has two positive members
    assert not g.gather_defined
    with pytest.raises(_lib.OgsError) as e:
        g.Gather(torch.zeros(2, dtype=torch.float64, device="cuda"),
                 torch.ones(3, dtype=torch.float64, device="cuda"), 1, ogs.Add, ogs.Trans)
    assert e.value.status == _lib.OGS_EUNDEFINED


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int64, np.int32], ids=lambda t: np.dtype(t).name)
def test_high_degree_rows(cuda, oracle_mod, dtype):
    """Rows of 9..2000 members (general bucket) beside rows of 1..8."""
    parts = [random_ids(2000, 2000, seed=1), random_ids(6000, 40, seed=2) + 10 ** 5,
             random_ids(4000, 2, seed=3) + 10 ** 6, np.arange(1, 4001, dtype=np.int64) % 500 + 10 ** 7]
    ids = np.concatenate(parts).astype(np.int64)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    assert g.max_degree >= 1500
    for op, name in ((ogs.Add, "add"), (ogs.Max, "max"), (ogs.Min, "min"), (ogs.Mul, "mul")):
        if np.dtype(dtype).kind == "f":
            v = np.sin(np.arange(ids.size, dtype=np.float64)).astype(dtype)
            if name == "mul":
                v = (1.0 + 0.001 * v).astype(dtype)
        else:
            v = (np.arange(ids.size) * 2654435761 % 1000003 - 500000).astype(dtype)
        for k in (1, 2):
            vk = np.repeat(v, k) if k > 1 else v
            got = gs(g, vk.copy(), k, op)
            want = ref.gather_scatter(vk.copy(), k, name, "sym")
            assert same_bits(got, want), (name, k, first_diff(got, want))


def test_signed_zero_nan_and_extremes(cuda, oracle_mod):
    ids = np.array([1, 2, 2, 3, 3, 3, 4, 5, 5, 6, 6], np.int64)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    nan, inf = np.nan, np.inf
    v = np.array([-0.0, -0.0, -0.0, nan, 1.0, -inf, -inf, nan, 2.0, -np.finfo(np.float64).max, -0.0])
    for op, name in ((ogs.Max, "max"), (ogs.Min, "min")):  # comparisons only: NaN handling is exact
        for dt in (np.float64, np.float32):
            with np.errstate(over="ignore"):  # -DBL_MAX becomes -inf in fp32, on purpose
                x = v.astype(dt)
            assert same_bits(gs(g, x.copy(), 1, op), ref.gather_scatter(x.copy(), 1, name, "sym"))
    # -0.0 under Add: the host computes 0.0 + (-0.0) = +0.0, also in degree-1 rows
    x = np.array([-0.0, -0.0, -0.0, 0.0, -0.0, -0.0, -0.0, 5.0, -5.0, 1e-310, -1e-310])
    for dt in (np.float64, np.float32):
        xx = x.astype(dt)
        assert same_bits(gs(g, xx.copy(), 1, ogs.Add), ref.gather_scatter(xx.copy(), 1, "add", "sym"))
    # fp32 subnormals are not flushed
    sub = np.full(ids.size, 1e-40, np.float32)
    assert same_bits(gs(g, sub.copy(), 1, ogs.Add), ref.gather_scatter(sub.copy(), 1, "add", "sym"))
    # integer extremes: Max identity is -max, so a lone INT_MIN becomes -INT_MAX
    for dt in (np.int32, np.int64):
        info = np.iinfo(dt)
        xi = np.array([info.min, info.min, info.max, info.max, 1, info.min, 0, info.max, info.max, -1, info.min], dt)
        for op, name in ((ogs.Max, "max"), (ogs.Min, "min"), (ogs.Add, "add"), (ogs.Mul, "mul")):
            assert same_bits(gs(g, xi.copy(), 1, op), ref.gather_scatter(xi.copy(), 1, name, "sym")), name


def test_bad_arguments_on_device_handle(cuda):
    ids = mesh.box_ids(2, 2, 2, 2)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    d = torch.zeros(ids.size, dtype=torch.float64, device="cuda")
    L = _lib.lib()
    assert L.ogs_gather_scatter(g.handle, d.data_ptr(), 0, 1, 0, 0, None) == _lib.OGS_EINVAL
    assert L.ogs_gather_scatter(g.handle, d.data_ptr(), 1, 9, 0, 0, None) == _lib.OGS_EINVAL
    assert L.ogs_gather_scatter(g.handle, d.data_ptr(), 1, 1, 9, 0, None) == _lib.OGS_EINVAL
    assert L.ogs_gather_scatter(g.handle, d.data_ptr(), 1, 1, 0, 5, None) == _lib.OGS_EINVAL
    assert L.ogs_gather_scatter(g.handle, None, 1, 1, 0, 0, None) == _lib.OGS_EINVAL



@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("op,name", [(ogs.Add, "add"), (ogs.Mul, "mul")])
def test_nan_results_are_nan_where_the_host_has_nan(cuda, oracle_mod, dtype, op, name):
    """Add and Mul with NaN operands or invalid steps (two different quiet
    NaNs, a quiet then a signalling NaN, inf - inf or 0 * inf) in
    exact-degree rows and in a row of 12 members: every entry the host makes
    NaN is NaN here and every other entry is bit-identical.  The NaN's own
    bits are the GPU's (fp32: 0x7fffffff; fp64: the first NaN operand, or a
    negative quiet NaN), not the host CPU's, which differ between x86 and
    Arm as well; following the host's rules costs the headline kernel a
    fifth of its speed (measured), so the payload is the documented
    deviation."""
    ut = np.uint64 if dtype == np.float64 else np.uint32
    qa, qb, sa = ((0x7ff8000000000123, 0xfff8000000000456, 0x7ff0000000000789) if dtype == np.float64
                  else (0x7fc00123, 0xffc00456, 0x7f800789))
    ids = np.array([1, 1, 2, 2, 3, 3, 4, 4, 4] + [5] * 12 + [6], np.int64)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    v = np.arange(1, ids.size + 1).astype(dtype)
    u = v.view(ut)
    u[0], u[1], u[2], u[3] = qa, qb, qa, sa
    if name == "add":
        v[4], v[5] = np.inf, -np.inf
    else:
        v[4], v[5] = 0, np.inf
    v[6], v[8] = -np.inf, np.inf
    u[12], u[15] = qb, sa
    got = gs(g, v.copy(), 1, op)
    want = oracle_mod.OracleOgs(ids.copy(), "unsigned").gather_scatter(v.copy(), 1, name, "sym")
    assert np.array_equal(np.isnan(got), np.isnan(want))
    keep = ~np.isnan(want)
    assert same_bits(got[keep], want[keep])
