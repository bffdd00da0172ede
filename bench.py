"""Benchmark of the single-rank ogs GatherScatter on GB300.

Default workload: the reference's headline call, ogs_t::GatherScatter(o_q, 1,
ogs::Add, ogs::Sym) on an Unsigned handle (dawgsMain.cpp:211-219), fp64, k=1,
over a 24x24x24-hex box mesh of degree p=7 (7,077,888 local / 4,826,809 global
nodes), values U[-1,1] from a fixed seed.  The metric is the reference's
DOFS/s = NgatherGlobal / seconds per call (dawgsMain.cpp:207).

One step = one GatherScatter launch over the whole mesh, inputs resident in
HBM.  Between steps the field is restored from a pristine device copy and L2
is flushed by writing a buffer of twice the L2 size and then reading it back
(the maps and field, about 0.1 GB, would otherwise stay in the 126 MB L2; the
read leaves L2 holding clean lines, so the timed kernel does not pay for
writing back the flush's dirty lines); only the GatherScatter is inside the
CUDA-event timing.  `e2e` is the same metric through the C ABI's
host-buffer entry point (ogs_gather_scatter_host: pinned host field copied in,
GatherScatter, copied back, stream synchronised) timed on the host clock.
`--impl reference` times the CPU oracle -- the C restatement of the
reference's host ogs (libs/ogs/ogsOperator.cpp:311-360) with its OpenMP row
loop -- on all host cores, on the same workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# e2e steps move the whole field both ways (113 MB at the default workload)
# and refill the pinned buffer from the CPU: they are capped apart from the
# kernel steps, which run long enough for several clock samples.
E2E_STEPS = 30
# the committed ncu summaries: each names the bench workload it captured
# ("bench_workload: ...") and its DRAM bytes per timed call
PROFILES = os.path.join(ROOT, "profiles")
FALLBACK_HBM_GBS = 6800.0
TYPE_CODE = {"float32": 0, "float64": 1, "int32": 2, "int64": 3}
OP_CODE = {"add": 0, "mul": 1, "max": 2, "min": 3}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nx", type=int, default=24)
    ap.add_argument("--ny", type=int, default=24)
    ap.add_argument("--nz", type=int, default=24)
    ap.add_argument("--p", type=int, default=7)
    ap.add_argument("--dtype", choices=list(TYPE_CODE), default="float64")
    ap.add_argument("--op", choices=list(OP_CODE), default="add")
    ap.add_argument("--k", type=int, default=1)
    ap.add_argument("--mode", choices=["gs", "gather", "scatter"], default="gs",
                    help="the timed call: GatherScatter (Sym, Unsigned handle; the headline), or Gather (Trans) / "
                         "Scatter (NoTrans) on a Signed unique handle, as dawgsMain.cpp:174-310 times them")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--permute", type=int, default=None, metavar="SEED",
                    help="permute the elements with this seed (the multi-field irregular-access workload "
                         "uses 32x32x16 p=5 with seed 2024)")
    ap.add_argument("--many", action="store_true",
                    help="k separate arrays (ogs_gather_scatter_many) instead of k interleaved components")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-meshes", type=int, default=256)
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-refdev", action="store_true")
    ap.add_argument("--no-partitioned", action="store_true")
    ap.add_argument("--served-requests", type=int, default=100000)
    ap.add_argument("--sweep", action="store_true",
                    help="print the results tables (one JSON line per case) instead of the bench line")
    ap.add_argument("--cases", default=None, metavar="REGEX",
                    help="with --sweep: only the cases whose name matches")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    if a.many and a.mode != "gs":
        ap.error("--many applies to GatherScatter only")
    if a.many:
        a.no_e2e = True  # no host-buffer form of the many layout
    return a


# ------------------------------------------------------------------ helpers
class Clocks:
    """nvidia-smi sampling the GPU every 50 ms (one streaming process, started
    before the region and stopped after it).  `summary()` gives the samples
    taken inside the region; `mark()` records a narrower timed region inside
    it, and `summary(marked=True)` reports that region's samples beside those
    of the whole window (a region shorter than the 50 ms period holds one
    sample at most)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.rows = []
        self._all = []
        self._proc = None
        self._t = None
        self._t0 = self._t1 = None
        self._m0 = self._m1 = None

    def _read(self):
        for line in self._proc.stdout:
            line = line.strip()
            if line:
                self._all.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                           "--format=csv,noheader,nounits", "-lms", "50"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            deadline = time.perf_counter() + 5.0
            while not self._all and time.perf_counter() < deadline:  # the sampler is running
                time.sleep(0.01)
        except OSError:
            self._proc = None
        self._t0 = time.perf_counter()
        return self

    def __exit__(self, *exc):
        self._t1 = time.perf_counter()
        if self._proc is not None:
            time.sleep(0.06)  # one more sample period
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
            if self._t:
                self._t.join(timeout=5)
        inside = [r for t, r in self._all if self._t0 <= t <= self._t1 + 0.06]
        self.rows = inside if inside else [r for _, r in self._all[-1:]]

    def mark(self, t0, t1):
        self._m0, self._m1 = t0, t1

    @staticmethod
    def _stats(rows):
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, val in zip(names, r[5:9]) if val.strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}

    def summary(self, marked=False):
        if not marked or self._m0 is None:
            return self._stats(self.rows)
        inside = [r for t, r in self._all if self._m0 <= t <= self._m1 + 0.06]
        out = self._stats(inside) or {"samples": 0}
        whole = self._stats(self.rows)
        out["timed_region_ms"] = 1e3 * (self._m1 - self._m0)
        out["sample_period_ms"] = 50
        if out["timed_region_ms"] < 10 * out["sample_period_ms"]:
            out["note"] = ("the timed region is shorter than ten sampling periods: its samples include the "
                           "ones just after it; whole_run covers every kernel leg of the run")
        if whole is not None:
            # the kernel legs of this run (cold and warm loops, the reference
            # device algorithm, e2e): the region above is too short for many
            # 50 ms samples
            out["whole_run"] = whole
        return out


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profiled_traffic(workload):
    """(dram bytes per timed call, summary file) from the committed ncu
    summary of this exact workload, or (None, None)."""
    try:
        names = sorted(os.listdir(PROFILES))
    except OSError:
        return None, None
    for fn in names:
        if not fn.endswith(".md"):
            continue
        got_w, got_b = None, None
        for line in open(os.path.join(PROFILES, fn)):
            t = line.strip()
            if t.startswith("bench_workload:"):
                got_w = t.split(":", 1)[1].strip()
            elif t.startswith("dram_bytes_per_launch:"):
                got_b = int(t.split(":")[1].strip().replace(",", ""))
        if got_w == workload and got_b is not None:
            return got_b, fn
    return None, None


MODE_NAME = {"gs": "GatherScatter", "gather": "Gather", "scatter": "Scatter"}
MODE_TRANS = {"gs": "Sym", "gather": "Trans", "scatter": "NoTrans"}


def workload_name(a):
    mode = getattr(a, "mode", "gs")
    op = "" if mode == "scatter" else f" {a.op.capitalize()}"
    handle = "" if mode == "gs" else " (Signed unique handle)"
    layout = " separate arrays" if getattr(a, "many", False) else (" interleaved" if a.k > 1 else "")
    perm = f", elements permuted (seed {a.permute})" if getattr(a, "permute", None) is not None else ""
    return (f"ogs {MODE_NAME[mode]} {a.dtype}{op} {MODE_TRANS[mode]} k={a.k}{layout}{handle}, "
            f"{a.nx}x{a.ny}x{a.nz} hex box p={a.p}{perm}")


def metric_name(a):
    lead = "fp64" if a.dtype == "float64" else a.dtype
    return f"{lead} {MODE_NAME[getattr(a, 'mode', 'gs')]} DOFS/s"


def alg_bytes(N, nnz, R, k, s, mode="gs", Nglobal=0):
    """GatherScatter (Sym): read and write every local value, read colIds and
    rowStarts.  Gather / Scatter: read (write) every local value once, write
    (read) every gathered value once, read colIds and rowStarts."""
    if mode == "gs":
        return 2 * k * s * N + 4 * nnz + 4 * (R + 1)
    return k * s * (N + Nglobal) + 4 * nnz + 4 * (R + 1)


def make_inputs(a):
    from dawgs_gb300 import mesh
    ids = mesh.box_ids(a.nx, a.ny, a.nz, a.p)
    if getattr(a, "permute", None) is not None:
        ids = mesh.permute_elements(ids, a.p, seed=a.permute)
    dt = np.dtype(a.dtype)
    n = a.k * ids.size
    if dt.kind == "f":
        v = mesh.uniform_values(n, dt, 0.5, 2.0, a.seed) if a.op == "mul" else \
            mesh.uniform_values(n, dt, -1.0, 1.0, a.seed)
    else:
        v = mesh.uniform_values(n, dt, -(2 ** 30), 2 ** 30, a.seed)
    return ids, v


def cpu_reference_run(a, ids, v, warmup, steps):
    """Oracle port of the host ogs operator of `a.mode` on all host cores:
    GatherScatter on an Unsigned handle, or Gather (Trans) / Scatter
    (NoTrans) on a Signed unique one (the scatter's input is the gather of v)."""
    import oracle
    oracle.build(ref=False)
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    mode = getattr(a, "mode", "gs")
    if mode == "gs" and getattr(a, "many", False):
        h = oracle.OracleOgs(ids.copy(), "unsigned")
        x = v.copy().reshape(a.k, -1)

        def call():
            for j in range(a.k):
                h.gather_scatter(x[j], 1, a.op, "sym")
        reset = lambda: np.copyto(x, v.reshape(a.k, -1))  # noqa: E731
    elif mode == "gs":
        h = oracle.OracleOgs(ids.copy(), "unsigned")
        x = v.copy()
        call = lambda: h.gather_scatter(x, a.k, a.op, "sym")  # noqa: E731
        reset = lambda: np.copyto(x, v)  # noqa: E731
    else:
        h = oracle.OracleOgs(ids.copy(), "signed", True)
        gv = np.zeros(a.k * h.Ngather, v.dtype)
        h.gather(gv, v.copy(), a.k, a.op, "trans")
        x = v.copy()
        if mode == "gather":
            out = np.zeros_like(gv)
            call = lambda: h.gather(out, x, a.k, a.op, "trans")  # noqa: E731
        else:
            call = lambda: h.scatter(x, gv, a.k, "notrans")  # noqa: E731
        reset = lambda: np.copyto(x, v)  # noqa: E731
    for _ in range(warmup):
        call()
    times = []
    for _ in range(steps):
        reset()
        t0 = time.perf_counter()
        call()
        times.append(time.perf_counter() - t0)
    return h, times, cores


def run_batched(a, dev, L, stream, log=None):
    """Uneven mesh mix: `batch_meshes` meshes with NX, NY, NZ uniform in [2,16]
    and p uniform in [1,7], each with an fp64 field of k in [1,4] components
    (U[-1,1]), Add GatherScatter.  Plain = one ogs_gather_scatter per mesh,
    back to back on one stream; batched = one tuned persistent launch replayed
    from a CUDA graph.  Aggregate DOFS/s counts NgatherGlobal * k per mesh."""
    import torch
    from dawgs_gb300 import mesh, ogs
    mix = mesh.mesh_mix(a.batch_meshes, seed=2024, lo=2, hi=16, pmax=7)
    ks = [1 + int(x % np.uint64(4)) for x in mesh.splitmix64(np.arange(len(mix), dtype=np.uint64) + np.uint64(77))]
    handles, fields, pristine, dofs, nlocal = [], [], [], 0, 0
    for (nx, ny, nz, p), k in zip(mix, ks):
        ids = mesh.box_ids(nx, ny, nz, p)
        g = ogs.ogs_t().Setup(ids.size, ids, None, ogs.Unsigned)
        v = torch.from_numpy(mesh.uniform_values(k * ids.size, np.float64, -1.0, 1.0, seed=nx * 1000 + p)).to(dev)
        handles.append(g)
        fields.append(v)
        pristine.append(v.clone())
        dofs += g.NgatherGlobal * k
        nlocal += ids.size * k
    batch = ogs.ogs_batch_t([(g, f, k, ogs.Add, ogs.Sym) for g, f, k in zip(handles, fields, ks)], graph=True)

    def restore():
        for f, p0 in zip(fields, pristine):
            f.copy_(p0)

    def time_it(fn, reps, chunk=50):
        # Repeated Add GatherScatter on one field multiplies a degree-d row by
        # d per call: within a few hundred calls the high-degree rows reach
        # +-inf and their stores turn silent.  The fields are restored every
        # `chunk` calls, outside the timed windows.
        restore()
        for _ in range(3):
            fn()
        total, done = 0.0, 0
        while done < reps:
            n = min(chunk, reps - done)
            restore()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(n):
                fn()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            total += e0.elapsed_time(e1) * 1e-3
            done += n
        return total / reps

    def plain():
        for g, f, k in zip(handles, fields, ks):
            L.ogs_gather_scatter(g.handle, f.data_ptr(), k, 1, 0, 0, stream.cuda_stream)

    t_plain = time_it(plain, max(a.steps // 2, 5))
    # every entry in the one persistent launch, as many CTAs as fit
    batch.set_config(stream=stream)
    t_persistent = time_it(lambda: batch.GatherScatter(stream), max(a.steps, 10))
    # the tuner times on scratch copies: the fields must come out untouched
    restore()
    tuned = batch.tune(stream, use_cache=False)
    untouched = all(torch.equal(f, p0) for f, p0 in zip(fields, pristine))
    again = batch.tune(stream)  # same key: taken from the cache
    t_batch = time_it(lambda: batch.GatherScatter(stream), max(a.steps, 10))
    # results: batched equals plain bit for bit (both from the pristine fields)
    restore()
    batch.GatherScatter(stream)
    got = [f.clone() for f in fields]
    restore()
    plain()
    torch.cuda.synchronize(dev)
    same = all(torch.equal(x, y) for x, y in zip(got, fields))
    return {"workload": f"{len(mix)} box meshes, NX,NY,NZ~U[2,16], p~U[1,7], fp64 k~U[1,4], Add Sym",
            "local_values": int(nlocal), "global_dofs_x_k": int(dofs), "items": batch.items,
            "tuned": tuned, "second_tune_from_cache": again["from_cache"], "tuner_left_fields_untouched": untouched,
            "plain_ms": t_plain * 1e3, "batched_ms": t_batch * 1e3, "persistent_only_ms": t_persistent * 1e3,
            "plain_dofs_per_s": dofs / t_plain, "batched_dofs_per_s": dofs / t_batch,
            "speedup": t_plain / t_batch, "speedup_persistent_only": t_plain / t_persistent,
            "identical_to_plain": bool(same),
            "l2": "working set larger than L2 (no flush)", "graph": True}


def run_served(a, dev, L, stream):
    """Served gather-scatter: 64 resident meshes drawn like the batched mix; a
    request picks a mesh uniformly, fp64 or fp32 (50/50), k uniform in [1,8],
    op Add 80% / Min 10% / Max 10% (integers are not used); fields are slices
    of one pinned host arena, initialised U[-1,1] and reused round-robin, so a
    later request finds what earlier ones left there (after many repeated Adds
    that includes +-inf and NaN bit patterns): this leg measures throughput and
    latency, the per-request results are checked by the served tests.
    Requests are admitted against a 16 GB device budget.  First a saturation
    run (all requests queued at once) gives the throughput; then Poisson
    arrivals at 25%, 50% and 80% of it give p50/p99 latency, counted from each
    request's scheduled arrival, after 0.5 s of the same arrival stream that
    is served but not counted (a GPU and host coming out of idle run the
    first tens of milliseconds slower).  The whole arrival schedule is handed to the
    server at once, which admits each request at its arrival time, so the
    client's own submission cost does not stand in for the server's.  Plain =
    the same requests one after another through ogs_gather_scatter_host."""
    import torch
    from dawgs_gb300 import mesh, ogs
    mix = mesh.mesh_mix(64, seed=77, lo=2, hi=16, pmax=7)
    handles = []
    for nx, ny, nz, p in mix:
        ids = mesh.box_ids(nx, ny, nz, p)
        handles.append(ogs.ogs_t().Setup(ids.size, ids, None, ogs.Unsigned))
    n = a.served_requests
    r = mesh.splitmix64(np.arange(4 * n, dtype=np.uint64) + np.uint64(4242))
    meshes = (r[0::4] % np.uint64(64)).astype(np.int64)
    dts = (r[1::4] % np.uint64(2)).astype(np.int64)            # 0: fp64, 1: fp32
    ks = 1 + (r[2::4] % np.uint64(8)).astype(np.int64)
    u = (r[3::4] % np.uint64(10)).astype(np.int64)
    ops = np.where(u < 8, 0, np.where(u == 8, 3, 2))           # Add / Min / Max
    nodes = np.array([handles[m].N for m in meshes], np.int64)
    nbytes = nodes * ks * np.where(dts == 0, 8, 4)
    dofs = float(sum(handles[m].NgatherGlobal * k for m, k in zip(meshes, ks)))
    # one pinned arena; request i works in place on its own slice, reused round-robin
    arena_bytes = int(max(256 << 20, 2 * nbytes.max()))
    arena = torch.empty(arena_bytes // 8, dtype=torch.float64).pin_memory()
    arena.uniform_(-1.0, 1.0)
    offs, off = np.zeros(n, np.int64), 0
    for i in range(n):
        b = int(nbytes[i])
        if off + b > arena_bytes:
            off = 0
        offs[i] = off
        off += (b + 255) // 256 * 256
    views = []
    for i in range(n):
        t = torch.float64 if dts[i] == 0 else torch.float32
        cnt = int(nodes[i] * ks[i])
        views.append(arena.view(torch.uint8)[offs[i]:offs[i] + nbytes[i]].view(t)[:cnt])

    import ctypes as C
    from dawgs_gb300 import _lib
    L = _lib.lib()
    req_table = (_lib.OgsServerRequest * n)()
    for i in range(n):
        req_table[i] = _lib.OgsServerRequest(int(meshes[i]), 1 if dts[i] == 0 else 0, int(ks[i]), int(ops[i]), 0,
                                             0, views[i].data_ptr())

    warm_s = 0.5

    def serve(rate):
        srv = ogs.ogs_server_t(field_budget_bytes=16 << 30, max_inflight=4096, max_batch=256)
        for g in handles:
            srv.add_mesh(g)
        # the first arrival comes after the whole schedule has been handed
        # over (queueing 100k requests takes some ms, under the server's lock)
        t0 = srv.clock() + 0.25
        nw = 0
        if rate is None:
            arr = np.full(n, t0)
            table = req_table
        else:
            # Poisson arrivals, led by warm_s seconds of the same stream that
            # are served but not counted: an idle GPU and host start slower
            # (clocks and power states ramp up), which a server under steady
            # load does not see
            nw = int(warm_s * rate)
            gaps = -np.log(1.0 - (mesh.splitmix64(np.arange(nw + n, dtype=np.uint64) + np.uint64(99))
                                  >> np.uint64(11)).astype(np.float64) / 9007199254740992.0) / rate
            arr = t0 + np.cumsum(gaps)
            # the warm-up requests repeat the table from its start (as often
            # as the warm-up needs), then the counted requests follow
            table = (_lib.OgsServerRequest * (nw + n))()
            rsz = C.sizeof(_lib.OgsServerRequest)
            done = 0
            while done < nw:
                m = min(n, nw - done)
                C.memmove(C.addressof(table) + rsz * done, req_table, rsz * m)
                done += m
            C.memmove(C.addressof(table) + rsz * nw, req_table, rsz * n)
        # the whole arrival schedule is handed over at once: the server admits
        # each request at its arrival time, and latency counts from there
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        first = C.c_int64()
        _lib.check(L.ogs_server_submit_many(srv._s, table, arr.ctypes.data, nw + n, C.byref(first)))
        srv.drain()
        ta, tl, td = srv.times(first.value + nw, n, launched=True)
        launches, _ = srv.counters()
        worker = srv.stats()
        srv.Free()
        lat = (td - ta) * 1e3
        span = td.max() - ta.min()
        out = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
               "p999_ms": float(np.percentile(lat, 99.9)),
               "dofs_per_s": dofs / span, "requests_per_s": n / span, "launches": int(launches)}
        if nw:
            out["warm_up"] = {"requests": nw, "seconds": warm_s, "counted": False}
        # when the slow requests arrived (50 ms bins from the first arrival)
        # and whether the worker itself stalled: a tail made of a few bins, at
        # a regular period, with long gaps between the worker's passes or
        # long CUDA calls, comes from outside the service (the host or the
        # driver), not from queueing in it
        slow = lat > 5.0
        bins = np.unique(np.floor((ta[slow] - ta.min()) / 0.05).astype(np.int64))
        out["over_5ms"] = {"share": float(slow.mean()), "bins_50ms": int(bins.size),
                           "first_bins": [int(b) for b in bins[:12]]}
        out["worker"] = {k: (round(v, 3) if isinstance(v, float) else v) for k, v in worker.items()}
        # where the time goes: waiting to be launched (admission, worker) and
        # from launch to completion (copies and kernels), small and large
        # fields apart (the server's two lanes split at 4 MiB)
        small = nbytes <= (4 << 20)
        for nm, sel in (("small", small), ("large", ~small)):
            if sel.any():
                out[nm] = {"share": float(sel.mean()),
                           "p99_ms": float(np.percentile(lat[sel], 99)),
                           "queue_p99_ms": float(np.percentile((tl - ta)[sel] * 1e3, 99)),
                           "service_p99_ms": float(np.percentile((td - tl)[sel] * 1e3, 99))}
        return out

    sat = serve(None)
    rates = {}
    for frac in (0.25, 0.5, 0.8):
        rates[f"{int(frac * 100)}%"] = dict(serve(frac * sat["requests_per_s"]),
                                             offered_per_s=frac * sat["requests_per_s"])
    # plain: one host-buffer call per request, back to back
    m_plain = min(n, 4000)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for i in range(m_plain):
        handles[meshes[i]].GatherScatter(views[i], int(ks[i]), int(ops[i]), 0, stream=stream)
    t_plain = time.perf_counter() - t0
    dofs_plain = float(sum(handles[meshes[i]].NgatherGlobal * ks[i] for i in range(m_plain)))
    return {"workload": "64 resident box meshes (NX,NY,NZ~U[2,16], p~U[1,7]); requests fp64/fp32 50/50, "
                        "k~U[1,8], Add 80%/Min 10%/Max 10%, pinned host fields, 16 GB device budget",
            "requests": n, "saturation": sat, "poisson": rates,
            "plain_dofs_per_s": dofs_plain / t_plain, "plain_requests": m_plain,
            "speedup_vs_plain": sat["dofs_per_s"] / (dofs_plain / t_plain)}


def run_partitioned(a, dev, stream, single_step_s, ranks_n=8):
    """The benchmark mesh split into `ranks_n` slabs of elements (z-major
    element order, like MakeIds' rank grid along z), run as emulated ranks on
    this GPU: per rank a halo Gather, send-buffer packing, the exchange as a
    device gather, the local GatherScatter, the postmpi Gather and the halo
    Scatter (dawgs_gb300/ranks.py).  The whole sequence of every rank is one
    CUDA graph; each step restores the fields and flushes L2 first."""
    import torch
    from dawgs_gb300 import mesh, ogs, ranks
    ids = mesh.box_ids(a.nx, a.ny, a.nz, a.p)
    ne, npe = a.nx * a.ny * a.nz, (a.p + 1) ** 3
    owner = (np.arange(ne) * ranks_n) // ne
    parts = [ids.reshape(ne, npe)[owner == r].reshape(-1).copy() for r in range(ranks_n)]
    t0 = time.perf_counter()
    rk = ranks.ranks_ogs_t(parts)
    setup_s = time.perf_counter() - t0
    pristine = [torch.from_numpy(mesh.uniform_values(p.size, np.float64, -1.0, 1.0, seed=100 + r)).to(dev)
                for r, p in enumerate(parts)]
    vs = [x.clone() for x in pristine]
    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        for _ in range(3):
            rk.GatherScatter(vs, 1, ogs.Add)
    torch.cuda.current_stream(dev).wait_stream(side)
    torch.cuda.synchronize(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        rk.GatherScatter(vs, 1, ogs.Add)
    l2 = torch.cuda.get_device_properties(dev).L2_cache_size
    flush = torch.empty(2 * l2 // 4 + 1, dtype=torch.float32, device=dev)
    sink = torch.empty((), dtype=torch.float32, device=dev)
    ts = []
    for it in range(a.warmup + a.steps):
        for v, p0 in zip(vs, pristine):
            v.copy_(p0)
        flush.zero_()
        torch.sum(flush, dim=0, out=sink)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        graph.replay()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        if it >= a.warmup:
            ts.append(e0.elapsed_time(e1) * 1e-3)
    t = sum(ts) / len(ts)
    nglobal = (a.nx * a.p + 1) * (a.ny * a.p + 1) * (a.nz * a.p + 1)
    halo_rows = sum(m["nhalo"] for m in rk.maps)
    sent = int(sum(m["send_T"].size for m in rk.maps))
    return {"workload": f"{workload_name(a)}, elements split into {ranks_n} z-slabs, emulated ranks on one GPU",
            "ranks": ranks_n, "ms_per_step": t * 1e3, "value": nglobal / t, "unit": "DOFS/s",
            "single_rank_ms_per_step": single_step_s * 1e3, "overhead_vs_single_rank": t / single_step_s,
            "halo_rows": int(halo_rows), "exchanged_entries": sent, "setup_s": setup_s,
            "graph": "all ranks' launches replayed from one CUDA graph",
            "l2": "flushed between steps"}


def aggregate_over_ranks(seconds, units, device=None):
    """Replicas: the job's time is the slowest rank's, its work the sum of all
    ranks' units.  Returns (seconds, units, throughput)."""
    import torch
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
        u = torch.tensor([float(units)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        seconds, units = float(t.item()), float(u.item())
    return seconds, units, units / seconds


# ------------------------------------------------------------------ arms
def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    ids, v = make_inputs(a)
    h, times, cores = cpu_reference_run(a, ids, v, a.warmup, a.steps)
    t = sum(times) / len(times)
    value = h.NgatherGlobal / t
    line = {
        "metric": metric_name(a),
        "value": value, "unit": "DOFS/s", "impl": "reference", "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"float64": "f64", "float32": "f32", "int32": "i32", "int64": "i64"}[a.dtype],
        "data": "synthetic (MakeIds box mesh, seeded U[-1,1])",
        "config": {"workload": workload_name(a), "local_dofs": int(ids.size),
                   "global_dofs": int(h.NgatherGlobal), "k": a.k, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "DOFS/s", "cores": cores, "kind": "port",
                         "sample": f"{a.steps} full {MODE_NAME[a.mode]} calls after {a.warmup} warm-up, "
                                   f"OpenMP over {cores} threads"},
        "e2e": {"value": value, "unit": "DOFS/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(a):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from dawgs_gb300 import _lib, ogs
    ids, v = make_inputs(a)
    # the headline's Unsigned handle, or the Signed unique handle dawgs times
    # Gather and Scatter on (dawgsMain.cpp:174-176)
    kind, unique = (ogs.Unsigned, False) if a.mode == "gs" else (ogs.Signed, True)
    g = ogs.ogs_t().Setup(ids.size, ids.copy(), None, kind, ogs.Auto, unique)
    # setup wall time, maps built on the GPU (the default at this size) and on the host
    setup_s = {"local_dofs": int(ids.size)}
    for how in ("device", "host"):
        idc = ids.copy()  # Setup may rewrite its ids (unique)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        h = ogs.ogs_t().Setup(ids.size, idc, None, kind, ogs.Auto, unique, maps=how)
        torch.cuda.synchronize(dev)
        setup_s[f"{how}_maps_s"] = time.perf_counter() - t0
        h.Free()
    tcode, ocode = TYPE_CODE[a.dtype], OP_CODE[a.op]
    s = np.dtype(a.dtype).itemsize
    pristine = torch.from_numpy(v).to(dev)
    work = pristine.clone()
    l2 = torch.cuda.get_device_properties(dev).L2_cache_size
    flush = torch.empty(2 * l2 // 4 + 1, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    L = _lib.lib()
    h = g.handle
    # gathered vector: Gather's output, Scatter's input (the gather of the field)
    gvd = torch.zeros(a.k * g.Ngather, dtype=pristine.dtype, device=dev)
    if a.mode == "scatter":
        _lib.check(L.ogs_gather(h, gvd.data_ptr(), pristine.data_ptr(), a.k, tcode, ocode, 2, stream.cuda_stream))

    import ctypes as C
    many_ptrs = (C.c_void_p * a.k)(*[work.data_ptr() + j * ids.size * s for j in range(a.k)])

    def call():
        if a.many:
            return L.ogs_gather_scatter_many(h, many_ptrs, a.k, tcode, ocode, 0, stream.cuda_stream)
        if a.mode == "gs":
            return L.ogs_gather_scatter(h, work.data_ptr(), a.k, tcode, ocode, 0, stream.cuda_stream)
        if a.mode == "gather":
            return L.ogs_gather(h, gvd.data_ptr(), work.data_ptr(), a.k, tcode, ocode, 2, stream.cuda_stream)
        return L.ogs_scatter(h, work.data_ptr(), gvd.data_ptr(), a.k, tcode, 1, stream.cuda_stream)

    def step(ev0=None, ev1=None):
        if ev0 is not None:
            ev0.record(stream)
        st = call()
        if ev1 is not None:
            ev1.record(stream)
        if st:
            _lib.check(st)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    sink = torch.empty((), dtype=torch.float32, device=dev)

    def flush_l2():
        flush.zero_()
        torch.sum(flush, dim=0, out=sink)

    # clocks are sampled over the kernel legs of the run (cold, warm, the
    # reference device algorithm, e2e); the cold timed loop is marked inside
    # that window
    clk = Clocks(local).__enter__()
    for _ in range(a.warmup):
        work.copy_(pristine)
        flush_l2()
        step()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    barrier()
    w0 = time.perf_counter()
    for e0, e1 in evs:
        work.copy_(pristine)
        flush_l2()
        step(e0, e1)
    barrier()
    w1 = time.perf_counter()
    clk.mark(w0, w1)
    kt = [e0.elapsed_time(e1) * 1e-3 for e0, e1 in evs]
    t_kernel, _, value = aggregate_over_ranks(sum(kt), g.NgatherGlobal * a.steps, dev)
    per_step = t_kernel / a.steps

    # warm: back-to-back calls on one field, no flush and no restore, so the
    # column ids and the field stay in L2 between calls (reported beside the
    # cold headline, not instead of it)
    # (the field is restored every 100 calls, outside the timed calls: repeated
    # Add multiplies a degree-d row by d per call, and rows that reached +-inf
    # would turn their stores silent)
    wev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    work.copy_(pristine)
    for _ in range(3):
        step()
    for j, (e0, e1) in enumerate(wev):
        if j % 100 == 0:
            work.copy_(pristine)
        step(e0, e1)
    torch.cuda.synchronize(dev)
    warm_per_step = sum(e0.elapsed_time(e1) * 1e-3 for e0, e1 in wev) / a.steps

    # the reference's device algorithm (OKL gatherScatter, 512-member row
    # blocks) restated in CUDA, timed the same way on the same GPU
    refdev_line = None
    if not a.no_refdev and rank == 0 and a.mode == "gs" and not a.many:
        import refdev
        refdev.build()
        rd = refdev.RefDevOgs(g)
        rts = []
        for it in range(a.warmup + a.steps):
            work.copy_(pristine)
            flush_l2()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rc = rd.gather_scatter(work.data_ptr(), a.k, tcode, ocode, stream.cuda_stream)
            e1.record(stream)
            if rc:
                raise SystemExit(f"bench: refdev launch failed ({rc})")
            torch.cuda.synchronize(dev)
            if it >= a.warmup:
                rts.append(e0.elapsed_time(e1) * 1e-3)
        ref_out = work.clone()
        work.copy_(pristine)
        step()
        torch.cuda.synchronize(dev)
        same = bool(torch.equal(ref_out.view(torch.uint8), work.view(torch.uint8)))
        rt = sum(rts) / len(rts)
        refdev_line = {"what": "reference device algorithm (ogsKernels.okl gatherScatter, 512-member row blocks, "
                               "256 threads, (blocks, k) grid) restated in CUDA, same GPU, same flush",
                       "value": g.NgatherGlobal / rt, "unit": "DOFS/s", "ms_per_step": rt * 1e3,
                       "row_blocks": rd.nblocks, "library_speedup": rt / per_step, "identical_results": same}
        rd.free()

    # e2e through the C ABI host-buffer entry point, pinned host memory
    e2e = None
    if not a.no_e2e:
        host = torch.from_numpy(v.copy()).pin_memory()
        host_gv = torch.zeros(a.k * g.Ngather, dtype=pristine.dtype).pin_memory()
        if a.mode == "scatter":
            host_gv.copy_(gvd.cpu())

        def host_call():
            if a.mode == "gs":
                return L.ogs_gather_scatter_host(h, host.data_ptr(), a.k, tcode, ocode, 0, stream.cuda_stream)
            if a.mode == "gather":
                return L.ogs_gather_host(h, host_gv.data_ptr(), host.data_ptr(), a.k, tcode, ocode, 2,
                                         stream.cuda_stream)
            return L.ogs_scatter_host(h, host.data_ptr(), host_gv.data_ptr(), a.k, tcode, 1, stream.cuda_stream)

        for _ in range(3):
            host.copy_(torch.from_numpy(v))
            _lib.check(host_call())
        et = []
        e2e_steps = min(a.steps, E2E_STEPS)
        for _ in range(e2e_steps):
            host.copy_(torch.from_numpy(v))
            flush_l2()
            barrier()
            t0 = time.perf_counter()
            _lib.check(host_call())
            et.append(time.perf_counter() - t0)
        t_e2e, _, e2e_value = aggregate_over_ranks(sum(et), g.NgatherGlobal * e2e_steps, dev)
        nbytes = a.k * ids.size * s
        gbytes = a.k * g.Ngather * s
        h2d, d2h = {"gs": (nbytes, nbytes), "gather": (nbytes, gbytes), "scatter": (gbytes, nbytes)}[a.mode]
        e2e = {"value": e2e_value, "unit": "DOFS/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": 1e3 * t_e2e / e2e_steps, "steps": e2e_steps,
               "api": {"gs": "ogs_gather_scatter_host", "gather": "ogs_gather_host",
                       "scatter": "ogs_scatter_host"}[a.mode] + " (C ABI)",
               "checked": "last step's host buffer equals the oracle bit for bit (with the CPU leg)"}

    # correctness of the timed configuration on this run's own output
    work.copy_(pristine)
    step()
    torch.cuda.synchronize(dev)
    # the sampler stops before the batched and served legs: its queries of the
    # driver every 50 ms stall the served requests' copies and launches now
    # and then, which would show in their latency tail
    clk.__exit__(None, None, None)

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        hc, times, cores = cpu_reference_run(a, ids, v, 2, 5)
        x = v.copy()
        if a.many:
            for j in range(a.k):
                hc.gather_scatter(x[j * ids.size:(j + 1) * ids.size], 1, a.op, "sym")
            got, host_got = work.cpu().numpy(), None
        elif a.mode == "gs":
            hc.gather_scatter(x, a.k, a.op, "sym")
            got, host_got = work.cpu().numpy(), (host.numpy() if e2e is not None else None)
        elif a.mode == "gather":
            x = np.zeros(a.k * hc.Ngather, v.dtype)
            hc.gather(x, v.copy(), a.k, a.op, "trans")
            got, host_got = gvd.cpu().numpy(), (host_gv.numpy() if e2e is not None else None)
        else:
            gx = np.zeros(a.k * hc.Ngather, v.dtype)
            hc.gather(gx, v.copy(), a.k, a.op, "trans")
            hc.scatter(x, gx, a.k, "notrans")
            got, host_got = work.cpu().numpy(), (host.numpy() if e2e is not None else None)
        if got.tobytes() != x.tobytes():
            raise SystemExit("bench: GPU result differs from the oracle on the timed workload")
        if host_got is not None and host_got.tobytes() != x.tobytes():
            raise SystemExit("bench: the host-buffer (e2e) result differs from the oracle")
        tc = sum(times) / len(times)
        cpu = {"value": hc.NgatherGlobal / tc, "unit": "DOFS/s", "cores": cores, "kind": "port",
               "sample": f"5 full {MODE_NAME[a.mode]} calls on this workload after 2 warm-up, OpenMP over "
                         f"{cores} threads; its output is also compared bit for bit with the GPU result"}

    # the batched and served legs use their own mesh mixes; they run beside
    # the fp64 Add k=1 GatherScatter of any box size
    headline_kind = (a.mode, a.dtype, a.op, a.k, a.many, a.permute) == ("gs", "float64", "add", 1, False, None)
    batched = None
    if rank == 0 and world == 1 and not a.no_batched and headline_kind:
        batched = run_batched(a, dev, L, stream)
    served = None
    if rank == 0 and world == 1 and not a.no_served and headline_kind:
        served = run_served(a, dev, L, stream)

    partitioned = None
    if rank == 0 and world == 1 and not a.no_partitioned and headline_kind:
        partitioned = run_partitioned(a, dev, stream, per_step)

    peak, peak_src = hbm_peak()
    nbytes_alg = alg_bytes(ids.size, g.nnzT, g.NlocalT, a.k, s, a.mode, g.Ngather)
    achieved = nbytes_alg / per_step / 1e9
    traffic, traffic_src = profiled_traffic(workload_name(a))
    stats = g.layout_stats()
    line = {
        "metric": metric_name(a),
        "value": value, "unit": "DOFS/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"float64": "f64", "float32": "f32", "int32": "i32", "int64": "i64"}[a.dtype],
        "data": "synthetic (MakeIds box mesh, seeded U[-1,1])",
        "config": {"workload": workload_name(a), "local_dofs": int(ids.size),
                   "global_dofs": int(g.NgatherGlobal), "k": a.k,
                   "l2": f"flushed between steps ({flush.numel() * 4 >> 20} MiB write then read)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "warp_tiles": stats["nwarp_tiles"], "general_tiles": stats["ngeneral_tiles"]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     # DRAM bytes one call really moves (ncu, committed summary of this workload),
                     # and that traffic over this run's time against the same peak: the
                     # algorithmic frac credits writes that silent stores skip and sectors
                     # that neighbouring rows share in L2
                     "traffic": traffic,
                     "dram_achieved": traffic / per_step / 1e9 if traffic else None,
                     "dram_frac": traffic / per_step / 1e9 / peak if traffic else None,
                     "traffic_source": f"profiles/{traffic_src}" if traffic_src else None,
                     "warm": {"ms_per_step": warm_per_step * 1e3, "achieved": nbytes_alg / warm_per_step / 1e9,
                              "frac": nbytes_alg / warm_per_step / 1e9 / peak},
                     "alg_bytes_per_launch": nbytes_alg, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"
                     if peak_src == "measured" else "fallback 6.8 TB/s"},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "batched": batched,
        "served": served,
        "setup": setup_s,
        "reference_device_equivalent": refdev_line,
        "partitioned": partitioned,
        "gpu_launches": a.steps,
        "clocks": clk.summary(marked=True),
        "wall_ms_per_step_incl_restore_and_flush": 1e3 * (w1 - w0) / a.steps,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_sweep(a):
    """The results tables: one JSON line per case, on cuda:0.

    24^3 box, fp64 Add GatherScatter for p = 1..15; at p = 7 also fp32 Add,
    int32/int64 Min/Max, Gather (Trans) and Scatter (NoTrans) on a Signed
    unique handle; the 32x32x16 p=5 mesh with a seeded element permutation,
    k = 1, k = 3 interleaved and k = 8 separate arrays, fp64/fp32 Add/Mul.
    cold: the field restored and L2 flushed (write then read 2x L2) before
    every timed call; warm (Add cases): back-to-back calls on one field."""
    import ctypes as C
    import torch
    from dawgs_gb300 import _lib, mesh, ogs
    L = _lib.lib()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    peak, _ = hbm_peak()
    l2 = torch.cuda.get_device_properties(dev).L2_cache_size
    flush = torch.empty(2 * l2 // 4 + 1, dtype=torch.float32, device=dev)
    sink = torch.empty((), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    tcode = {torch.float64: 1, torch.float32: 0, torch.int32: 2, torch.int64: 3}
    reps = max(a.steps, 5)

    def timeit(fn, restore=None, cold=True, restore_every=1):
        # restore_every > 1 (warm figures): the field goes back to its start
        # every few calls, untimed, so that repeated Add cannot drive rows to
        # +-inf (stores of rows already at inf are silent)
        # The calls are queued back to back and synchronised once at the end:
        # with a synchronisation between calls the GPU would sit idle from the
        # start event until the host's launch arrives, and the event pair
        # would time the host call too.
        evs = []
        for i in range(reps + 3):
            if restore is not None and i % restore_every == 0:
                restore()
            if cold:
                flush.zero_()
                torch.sum(flush, dim=0, out=sink)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            rc = fn()
            e1.record(st)
            if rc:
                raise SystemExit(f"bench --sweep: status {rc}: {L.ogs_last_error_string().decode()}")
            if i >= 3:
                evs.append((e0, e1))
        torch.cuda.synchronize(dev)
        ts = [e0.elapsed_time(e1) * 1e-3 for e0, e1 in evs]
        # CUDA event times come in steps of about 1 us on GB300: a median of
        # quantised samples is off by up to a step, the mean of the middle 80 %
        # of many samples is not
        ts = np.sort(np.asarray(ts))
        cut = len(ts) // 10
        return float(ts[cut:len(ts) - cut].mean())

    import re
    pick = re.compile(a.cases) if a.cases else None

    def wanted(case):
        return pick is None or pick.search(case) is not None

    def emit(case, g, k, t, ab, warm=None):
        r = {"case": case, "local_dofs": int(g.N), "global_dofs": int(g.NgatherGlobal), "k": k,
             "us_cold": t * 1e6, "dofs_per_s_cold": g.NgatherGlobal * k / t, "gbs_cold": ab / t / 1e9,
             "frac_cold": ab / t / 1e9 / peak, "alg_bytes": int(ab)}
        if warm is not None:
            r.update(us_warm=warm * 1e6, frac_warm=ab / warm / 1e9 / peak)
        print(json.dumps(r), flush=True)

    def gs(case, g, x, k, op, ab, many=None):
        if not wanted(case):
            return
        if many is None:
            x0 = x.clone()
            fn = lambda: L.ogs_gather_scatter(g.handle, x.data_ptr(), k, tcode[x.dtype], op, 0, st.cuda_stream)
            t = timeit(fn, restore=lambda: x.copy_(x0))
        else:
            arr = (C.c_void_p * len(many))(*[m.data_ptr() for m in many])
            m0 = [m.clone() for m in many]
            fn = lambda: L.ogs_gather_scatter_many(g.handle, arr, len(many), tcode[many[0].dtype], op, 0,
                                                   st.cuda_stream)

            def restore():
                for m, q in zip(many, m0):
                    m.copy_(q)
            t = timeit(fn, restore=restore)
        if op != 0:
            warm = None
        elif many is None:
            warm = timeit(fn, restore=lambda: x.copy_(x0), cold=False, restore_every=50)
        else:
            warm = timeit(fn, restore=restore, cold=False, restore_every=50)
        emit(case, g, k, t, ab, warm)

    def idx_bytes(g):
        return 4 * g.nnzT + 4 * (g.NlocalT + 1)

    # the floor of this harness: a one-element fill kernel between the same
    # events, after the same L2 flush
    one = torch.zeros(1, dtype=torch.float32, device=dev)
    t_empty = timeit(lambda: (one.fill_(1.0), 0)[1])
    print(json.dumps({"case": "empty launch (one-element fill kernel)", "us_cold": t_empty * 1e6}), flush=True)

    for p in range(1, 16):
        if pick is not None and not any(wanted(f"24^3 p={p} {c}") for c in
                                        ("f64 Add GS", "f32 Add GS", "int32 Min GS", "int32 Max GS", "int64 Min GS",
                                         "int64 Max GS", "f64 Gather Trans", "f64 Scatter NoTrans")):
            continue
        ids = mesh.box_ids(24, 24, 24, p)
        g = ogs.ogs_t().Setup(ids.size, ids.copy())
        x = torch.from_numpy(mesh.uniform_values(ids.size, np.float64, -1, 1, p)).to(dev)
        gs(f"24^3 p={p} f64 Add GS", g, x, 1, 0, 16 * ids.size + idx_bytes(g))
        if p == 7:
            # every case below starts from fresh seeded values, not from a field
            # that earlier timings have already folded
            xf = torch.from_numpy(mesh.uniform_values(ids.size, np.float32, -1, 1, p)).to(dev)
            gs("24^3 p=7 f32 Add GS", g, xf, 1, 0, 8 * ids.size + idx_bytes(g))
            for dt in (torch.int32, torch.int64):
                xi = torch.from_numpy(mesh.uniform_values(ids.size, np.int64, -(2 ** 30), 2 ** 30, 3)).to(dev).to(dt)
                for op, nm in ((3, "Min"), (2, "Max")):
                    # each op from the same pristine field: a field already folded by one op
                    # would leave the next with every store silent
                    gs(f"24^3 p=7 {str(dt)[6:]} {nm} GS", g, xi.clone(), 1, op,
                       2 * xi.element_size() * ids.size + idx_bytes(g))
            sa = ids.copy()
            sg = ogs.ogs_t().Setup(sa.size, sa, None, ogs.Signed, ogs.Auto, True)
            gv = torch.zeros(sg.Ngather, dtype=torch.float64, device=dev)
            x = torch.from_numpy(mesh.uniform_values(ids.size, np.float64, -1, 1, p)).to(dev)
            abg = 8 * (ids.size + sg.Ngather) + idx_bytes(sg)
            for nm, fn in (("Gather Trans", lambda: L.ogs_gather(sg.handle, gv.data_ptr(), x.data_ptr(), 1, 1, 0, 2,
                                                                 st.cuda_stream)),
                           ("Scatter NoTrans", lambda: L.ogs_scatter(sg.handle, x.data_ptr(), gv.data_ptr(), 1, 1, 1,
                                                                     st.cuda_stream))):
                if wanted(f"24^3 p=7 f64 {nm}"):
                    emit(f"24^3 p=7 f64 {nm}", sg, 1, timeit(fn), abg, timeit(fn, cold=False))
            del sg, gv
        del g, x
    ids = mesh.permute_elements(mesh.box_ids(32, 32, 16, 5), 5, seed=2024)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    x1 = torch.from_numpy(mesh.uniform_values(ids.size, np.float64, -1, 1, 1)).to(dev)
    gs("32x32x16 p=5 perm f64 Add k=1", g, x1, 1, 0, 16 * ids.size + idx_bytes(g))
    for dt, s in ((torch.float64, 8), (torch.float32, 4)):
        for op, nm, lo in ((0, "Add", -1.0), (1, "Mul", 0.5)):
            hi = 1.0 if op == 0 else 2.0
            x3 = torch.from_numpy(mesh.uniform_values(3 * ids.size, np.float64, lo, hi, 7)).to(dev).to(dt)
            gs(f"32x32x16 p=5 perm {str(dt)[6:]} {nm} k=3", g, x3, 3, op, 6 * s * ids.size + idx_bytes(g))
            vs = [torch.from_numpy(mesh.uniform_values(ids.size, np.float64, lo, hi, 70 + j)).to(dev).to(dt)
                  for j in range(8)]
            gs(f"32x32x16 p=5 perm {str(dt)[6:]} {nm} k=8 arrays", g, None, 8, op, 16 * s * ids.size + idx_bytes(g),
               many=vs)
    # Gather (Trans) and Scatter (NoTrans) of k = 3 interleaved components on
    # the Signed unique handle of the same mesh
    sa = ids.copy()
    sg = ogs.ogs_t().Setup(sa.size, sa, None, ogs.Signed, ogs.Auto, True)
    for dt, s in ((torch.float64, 8), (torch.float32, 4)):
        tc = tcode[dt]
        gv3 = torch.zeros(3 * sg.Ngather, dtype=dt, device=dev)
        x3 = torch.from_numpy(mesh.uniform_values(3 * ids.size, np.float64, -1.0, 1.0, 9)).to(dev).to(dt)
        ab3 = 3 * s * (ids.size + sg.Ngather) + idx_bytes(sg)
        for nm, fn in (("Gather Trans", lambda: L.ogs_gather(sg.handle, gv3.data_ptr(), x3.data_ptr(), 3, tc, 0, 2,
                                                             st.cuda_stream)),
                       ("Scatter NoTrans", lambda: L.ogs_scatter(sg.handle, x3.data_ptr(), gv3.data_ptr(), 3, tc, 1,
                                                                 st.cuda_stream))):
            case = f"32x32x16 p=5 perm {str(dt)[6:]} {nm} k=3"
            if wanted(case):
                emit(case, sg, 3, timeit(fn), ab3, timeit(fn, cold=False))
    return 0


def main():
    a = parse()
    if a.impl == "reference":
        return run_reference(a)
    if a.sweep:
        return run_sweep(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
