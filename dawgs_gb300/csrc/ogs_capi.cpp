// ogs_capi.cpp -- the C ABI (include/ogs_c.h): argument checks, the mapping of
// (kind, Transpose) to the members each operation reads and writes, and the
// host-buffer entry points.  No exception crosses this boundary.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"
#include "ogs_trace.hpp"

#ifndef OGS_KERNEL
#define OGS_KERNEL 0
#endif

namespace ogsgb {

static thread_local std::string g_last_error;

ogs_status set_error(ogs_status s, const std::string& msg) {
  g_last_error = msg;
  return s;
}

size_t type_size(int type) { return (type == OGS_DOUBLE || type == OGS_INT64) ? 8 : 4; }

ogs_status check_common(ogs_handle h, int k, int type, int trans, const char* fn) {
  if (!h) return set_error(OGS_EINVAL, std::string(fn) + ": handle is NULL");
  if (h->host_only) return set_error(OGS_EINVAL, std::string(fn) + ": handle was set up host-only");
  if (h->gslib) return set_error(OGS_EINVAL, std::string(fn) + ": handle was made by ogs_gslib_setup");
  if (k < 1) return set_error(OGS_EINVAL, std::string(fn) + ": k must be >= 1");
  if (type < OGS_FLOAT || type > OGS_INT64) return set_error(OGS_EINVAL, std::string(fn) + ": unknown type");
  if (trans < OGS_SYM || trans > OGS_TRANS) return set_error(OGS_EINVAL, std::string(fn) + ": unknown transpose");
  if (h->N > 0) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(OGS_EDEVICE, std::string(fn) + ": " + cudaGetErrorString(e));
    if (dev != h->device)
      return set_error(OGS_EINVAL, std::string(fn) + ": handle lives on device " + std::to_string(h->device) +
                                       ", current device is " + std::to_string(dev));
  }
  return OGS_OK;
}

// GatherScatter and Scatter write every member: refused when a local node
// sits in two rows of an operator built from caller maps.
ogs_status check_writes(ogs_handle h, const char* fn) {
  if (!h->distinct_cols)
    return set_error(OGS_EINVAL, std::string(fn) + ": a local node appears in two rows of this operator's map");
  return OGS_OK;
}

ogs_status check_op(int op, const char* fn) {
  if (op < OGS_ADD || op > OGS_MIN) return set_error(OGS_EINVAL, std::string(fn) + ": unknown op");
  return OGS_OK;
}

// Members read and written, ogsOperator.cpp:71-79 (Gather), 214-222 (Scatter),
// 321-339 (GatherScatter).  Unsigned handles alias N to T, so every transpose
// acts as Sym there.
Pattern pattern_for(const ogs_handle_s* h, int mode, int trans) {
  Pattern p{0, 0, 0};
  if (h->kind != OGS_SIGNED) return p;
  if (mode == kModeGS) {
    if (trans == OGS_TRANS) p = Pattern{0, 1, 1};
    else if (trans == OGS_NOTRANS) p = Pattern{1, 0, 0};
  } else if (mode == kModeGather) {
    if (trans == OGS_NOTRANS) p = Pattern{1, 0, 1};
  } else {
    if (trans == OGS_TRANS) p = Pattern{0, 1, 1};
  }
  return p;
}

namespace {

ogs_status launch_maps(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, int type,
                       void* stream, const char* fn) {
  int e = 0;
  switch (type) {
    case OGS_FLOAT: e = launch_f32(m, f, mode, op, pat, stream); break;
    case OGS_DOUBLE: e = launch_f64(m, f, mode, op, pat, stream); break;
    case OGS_INT32: e = launch_i32(m, f, mode, op, pat, stream); break;
    default: e = launch_i64(m, f, mode, op, pat, stream); break;
  }
  if (e != 0)
    return set_error(OGS_EDEVICE, std::string(fn) + ": kernel launch failed: " +
                                      cudaGetErrorString(static_cast<cudaError_t>(e)));
  return OGS_OK;
}

ogs_status launch(const ogs_handle_s* h, const FieldArgs& f, int mode, int op, Pattern pat, int type,
                  void* stream, const char* fn) {
  return launch_maps(h->dmaps, f, mode, op, pat, type, stream, fn);
}

ogs_status ensure_stage(ogs_handle_s* h, size_t bytes, const char* fn) {
  if (bytes <= h->stage_bytes) return OGS_OK;
  if (h->stage) dev_free(h->stage);
  h->stage = nullptr;
  h->stage_bytes = 0;
  cudaError_t e = dev_malloc(&h->stage, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    h->stage = nullptr;
    return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                     std::string(fn) + ": staging allocation: " + cudaGetErrorString(e));
  }
  h->stage_bytes = bytes;
  return OGS_OK;
}

ogs_status cuda_status(cudaError_t e, const char* fn, const char* what) {
  if (e == cudaSuccess) return OGS_OK;
  return set_error(OGS_EDEVICE, std::string(fn) + ": " + what + ": " + cudaGetErrorString(e));
}

// Copy streams, capture stream and events of the host-buffer pipeline, made
// on first use.
ogs_status ensure_pipeline(ogs_handle_s* h, const char* fn) {
  const size_t need = 3 + 2 * h->lay.phases.size();
  if (h->copy_in && h->events.size() >= need) return OGS_OK;
  ogs_status s;
  if (!h->copy_in) {
    cudaStream_t a = nullptr, b = nullptr, c = nullptr;
    if ((s = cuda_status(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking), fn, "stream")) != OGS_OK) return s;
    if ((s = cuda_status(cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking), fn, "stream")) != OGS_OK) {
      cudaStreamDestroy(a);
      return s;
    }
    if ((s = cuda_status(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking), fn, "stream")) != OGS_OK) {
      cudaStreamDestroy(a);
      cudaStreamDestroy(b);
      return s;
    }
    h->copy_in = a;
    h->copy_out = b;
    h->capture = c;
  }
  while (h->events.size() < need) {
    cudaEvent_t e = nullptr;
    if ((s = cuda_status(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), fn, "event")) != OGS_OK) return s;
    h->events.push_back(e);
  }
  return OGS_OK;
}

// The same pipeline captured once per (host buffer, k, type, op, transpose)
// into a CUDA graph and replayed on `st`, so a repeated call costs one graph
// launch (built when OGS_HOST_GRAPH is set).
ogs_status host_pipeline_graph(ogs_handle_s* h, void* v, int k, int type, int op, int trans, const FieldArgs& f,
                               const Pattern& pat, size_t node_bytes, cudaStream_t st, const char* fn) {
  ogs_status s;
  const size_t P = h->lay.phases.size();
  ogs_handle_s::HostGraph* hit = nullptr;
  for (auto& g : h->host_graphs)
    if (g.host == v && g.k == k && g.type == type && g.op == op && g.trans == trans) hit = &g;
  if (!hit) {
    cudaStream_t cap = static_cast<cudaStream_t>(h->capture);
    cudaStream_t sin = static_cast<cudaStream_t>(h->copy_in);
    cudaStream_t sout = static_cast<cudaStream_t>(h->copy_out);
    auto ev = [&](size_t i) { return static_cast<cudaEvent_t>(h->events[i]); };
    char* dv = static_cast<char*>(h->stage);
    char* hv = static_cast<char*>(v);
    const std::vector<Phase>& ph = h->lay.phases;
    if ((s = cuda_status(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), fn, "capture")) != OGS_OK)
      return s;
    cudaError_t ce = cudaEventRecord(ev(0), cap);
    if (!ce) ce = cudaStreamWaitEvent(sin, ev(0), 0);
    if (!ce) ce = cudaStreamWaitEvent(sout, ev(0), 0);
    for (size_t p = 0; !ce && p < P; ++p) {
      const size_t off = static_cast<size_t>(ph[p].h0) * node_bytes;
      const size_t len = static_cast<size_t>(ph[p].h1 - ph[p].h0) * node_bytes;
      if (len) ce = cudaMemcpyAsync(dv + off, hv + off, len, cudaMemcpyHostToDevice, sin);
      if (!ce) ce = cudaEventRecord(ev(1 + 2 * p), sin);
    }
    ogs_status ls = OGS_OK;
    for (size_t p = 0; !ce && ls == OGS_OK && p < P; ++p) {
      ce = cudaStreamWaitEvent(cap, ev(1 + 2 * p), 0);
      if (!ce) ls = launch_maps(phase_maps(h->dmaps, ph[p]), f, kModeGS, op, pat, type, cap, fn);
      if (!ce && ls == OGS_OK) ce = cudaEventRecord(ev(2 + 2 * p), cap);
    }
    for (size_t p = 0; !ce && ls == OGS_OK && p < P; ++p) {
      const size_t off = static_cast<size_t>(ph[p].d0) * node_bytes;
      const size_t len = static_cast<size_t>(ph[p].d1 - ph[p].d0) * node_bytes;
      if (!len) continue;
      ce = cudaStreamWaitEvent(sout, ev(2 + 2 * p), 0);
      if (!ce) ce = cudaMemcpyAsync(hv + off, dv + off, len, cudaMemcpyDeviceToHost, sout);
    }
    // join the copy streams back into the capture stream
    if (!ce && ls == OGS_OK) ce = cudaEventRecord(ev(1 + 2 * P), sin);
    if (!ce && ls == OGS_OK) ce = cudaEventRecord(ev(2 + 2 * P), sout);
    if (!ce && ls == OGS_OK) ce = cudaStreamWaitEvent(cap, ev(1 + 2 * P), 0);
    if (!ce && ls == OGS_OK) ce = cudaStreamWaitEvent(cap, ev(2 + 2 * P), 0);
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(cap, &graph);
    if (ls != OGS_OK) {
      if (graph) cudaGraphDestroy(graph);
      return ls;
    }
    if (ce || ee) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return cuda_status(ce ? ce : ee, fn, "capture of the host pipeline");
    }
    cudaGraphExec_t exec = nullptr;
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if ((s = cuda_status(ce, fn, "instantiate")) != OGS_OK) return s;
    if (h->host_graphs.size() >= 4) {  // keep the four most recent
      cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(h->host_graphs.back().exec));
      h->host_graphs.pop_back();
    }
    h->host_graphs.insert(h->host_graphs.begin(), ogs_handle_s::HostGraph{v, k, type, op, trans, exec});
    hit = &h->host_graphs.front();
  }
  if ((s = cuda_status(cudaGraphLaunch(static_cast<cudaGraphExec_t>(hit->exec), st), fn, "graph launch")) != OGS_OK)
    return s;
  return cuda_status(cudaStreamSynchronize(st), fn, "synchronize");
}

}  // namespace
}  // namespace ogsgb

using namespace ogsgb;

extern "C" {

const char* ogs_last_error_string(void) { return g_last_error.c_str(); }

int ogs_version(void) { return 10000; }

ogs_status ogs_setup_ex(ogs_handle* out, int64_t N, int64_t* ids, int kind, int unique, unsigned flags) {
  if (!out) return set_error(OGS_EINVAL, "ogs_setup: out is NULL");
  TraceRange trace("ogs_setup");
  *out = nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  ogs_handle_s* h = new (std::nothrow) ogs_handle_s();
  if (!h) return set_error(OGS_ENOMEM, "ogs_setup: out of host memory");
  const bool host_only = (flags & OGS_SETUP_HOST_ONLY) != 0;
  if ((flags & OGS_SETUP_DEVICE_MAPS) && (host_only || (flags & OGS_SETUP_HOST_MAPS))) {
    delete h;
    return set_error(OGS_EINVAL, "ogs_setup: OGS_SETUP_DEVICE_MAPS excludes HOST_ONLY and HOST_MAPS");
  }
  const bool device_maps =
      (flags & OGS_SETUP_DEVICE_MAPS) ||
      (!host_only && !(flags & OGS_SETUP_HOST_MAPS) && N >= OGS_DEVICE_MAPS_MIN_N);
  try {
    ogs_status s = device_maps ? build_device_maps(h, N, ids, kind, unique, true)
                               : build_host_maps(h, N, ids, kind, unique);
    if (s != OGS_OK) { release_device(h); delete h; return s; }
    h->host_only = host_only;
    if (!h->arena) build_layout(h);  // the device path built it already (unless the maps are empty)
    if (!h->host_only && !h->arena) {
      s = upload_layout(h);
      if (s != OGS_OK) { release_device(h); delete h; return s; }
      cudaError_t e = cudaDeviceSynchronize();
      if (e != cudaSuccess) {
        release_device(h);
        delete h;
        return cuda_status(e, "ogs_setup", "synchronize");
      }
    }
  } catch (const std::bad_alloc&) {
    release_device(h);  // the device setup may have made the arena already
    delete h;
    return set_error(OGS_ENOMEM, "ogs_setup: out of host memory");
  }
  if (flags & OGS_SETUP_VERBOSE) {  // ogsSetup.cpp:184-189
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("ogs Setup Time: %g seconds.\n", dt);
  }
  *out = h;
  return OGS_OK;
}

ogs_status ogs_setup(ogs_handle* out, int64_t N, int64_t* ids, int kind, int method, int unique,
                     int verbose) {
  if (method < OGS_AUTO || method > OGS_ALLTOALL) return set_error(OGS_EINVAL, "ogs_setup: unknown method");
  return ogs_setup_ex(out, N, ids, kind, unique, verbose ? OGS_SETUP_VERBOSE : 0u);
}

ogs_status ogs_free(ogs_handle h) {
  if (!h) return OGS_OK;
  release_device(h);
  delete h;
  return OGS_OK;
}

ogs_status ogs_gather_scatter(ogs_handle h, void* d_v, int k, int type, int op, int trans, void* stream) {
  const char* fn = "ogs_gather_scatter";
  ogs_status s = check_common(h, k, type, trans, fn);
  if (s == OGS_OK) s = check_writes(h, fn);
  if (s == OGS_OK) s = check_op(op, fn);
  if (s != OGS_OK) return s;
  if (h->N == 0) return OGS_OK;
  if (!d_v) return set_error(OGS_EINVAL, "ogs_gather_scatter: d_v is NULL");
  FieldArgs f{};
  f.v = d_v;
  f.K = k;
  return launch(h, f, kModeGS, op, pattern_for(h, kModeGS, trans), type, stream, fn);
}

ogs_status ogs_gather_scatter_many(ogs_handle h, void* const* d_vs, int k, int type, int op, int trans,
                                   void* stream) {
  const char* fn = "ogs_gather_scatter_many";
  ogs_status s = check_common(h, k, type, trans, fn);
  if (s == OGS_OK) s = check_writes(h, fn);
  if (s == OGS_OK) s = check_op(op, fn);
  if (s != OGS_OK) return s;
  if (h->N == 0) return OGS_OK;
  if (!d_vs) return set_error(OGS_EINVAL, "ogs_gather_scatter_many: d_vs is NULL");
  const Pattern pat = pattern_for(h, kModeGS, trans);
  for (int k0 = 0; k0 < k; k0 += kMaxMany) {
    FieldArgs f{};
    f.is_many = 1;
    f.K = (k - k0 < kMaxMany) ? (k - k0) : kMaxMany;
    for (int j = 0; j < f.K; ++j) {
      if (!d_vs[k0 + j]) return set_error(OGS_EINVAL, "ogs_gather_scatter_many: a field pointer is NULL");
      f.many[j] = d_vs[k0 + j];
    }
    s = launch(h, f, kModeGS, op, pat, type, stream, fn);
    if (s != OGS_OK) return s;
  }
  return OGS_OK;
}

ogs_status ogs_gather(ogs_handle h, void* d_gv, const void* d_v, int k, int type, int op, int trans,
                      void* stream) {
  const char* fn = "ogs_gather";
  ogs_status s = check_common(h, k, type, trans, fn);
  if (s == OGS_OK) s = check_op(op, fn);
  if (s != OGS_OK) return s;
  if (!h->gather_defined)  // ogsSetup.cpp:861-864
    return set_error(OGS_EUNDEFINED, "Gather operation not well-defined.");
  if (h->N == 0 || h->NlocalT == 0) return OGS_OK;
  if (!d_gv || !d_v) return set_error(OGS_EINVAL, "ogs_gather: NULL buffer");
  FieldArgs f{};
  f.v = const_cast<void*>(d_v);
  f.gv = d_gv;
  f.K = k;
  return launch(h, f, kModeGather, op, pattern_for(h, kModeGather, trans), type, stream, fn);
}

ogs_status ogs_scatter(ogs_handle h, void* d_v, const void* d_gv, int k, int type, int trans, void* stream) {
  const char* fn = "ogs_scatter";
  ogs_status s = check_common(h, k, type, trans, fn);
  if (s == OGS_OK) s = check_writes(h, fn);
  if (s != OGS_OK) return s;
  if (!h->gather_defined)  // AssertGatherDefined in ScatterStart, ogs.cpp:398
    return set_error(OGS_EUNDEFINED, "Gather operation not well-defined.");
  if (h->N == 0 || h->NlocalT == 0) return OGS_OK;
  if (!d_gv || !d_v) return set_error(OGS_EINVAL, "ogs_scatter: NULL buffer");
  FieldArgs f{};
  f.v = d_v;
  f.gv = const_cast<void*>(d_gv);
  f.K = k;
  return launch(h, f, kModeScatter, OGS_ADD, pattern_for(h, kModeScatter, trans), type, stream, fn);
}

ogs_status ogs_gather_scatter_host(ogs_handle h, void* v, int k, int type, int op, int trans, void* stream) {
  const char* fn = "ogs_gather_scatter_host";
  TraceRange trace(fn);
  ogs_status s = check_common(h, k, type, trans, fn);
  if (s == OGS_OK) s = check_writes(h, fn);
  if (s == OGS_OK) s = check_op(op, fn);
  if (s != OGS_OK) return s;
  if (h->N == 0) return OGS_OK;
  if (!v) return set_error(OGS_EINVAL, "ogs_gather_scatter_host: v is NULL");
  std::lock_guard<std::mutex> host_lock(h->host_mu);
  const size_t node_bytes = static_cast<size_t>(k) * type_size(type);
  const size_t bytes = static_cast<size_t>(h->N) * node_bytes;
  if ((s = ensure_stage(h, bytes, fn)) != OGS_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  FieldArgs f{};
  f.v = h->stage;
  f.K = k;
  const Pattern pat = pattern_for(h, kModeGS, trans);
  // The pipelined, graph-captured path needs page-locked host memory (copies
  // from pageable memory cannot be captured and are staged by the driver
  // anyway); pageable buffers take one copy in, the kernels, one copy out.
  cudaPointerAttributes attr{};
  const bool pinned = cudaPointerGetAttributes(&attr, v) == cudaSuccess && attr.type == cudaMemoryTypeHost;
  cudaGetLastError();
  if (OGS_KERNEL != 0 || h->lay.phases.size() < 2 || !pinned) {
    if ((s = cuda_status(cudaMemcpyAsync(h->stage, v, bytes, cudaMemcpyHostToDevice, st), fn, "copy in")) != OGS_OK)
      return s;
    if ((s = launch(h, f, kModeGS, op, pat, type, stream, fn)) != OGS_OK) return s;
    if ((s = cuda_status(cudaMemcpyAsync(v, h->stage, bytes, cudaMemcpyDeviceToHost, st), fn, "copy out")) !=
        OGS_OK)
      return s;
    return cuda_status(cudaStreamSynchronize(st), fn, "synchronize");
  }
  // Pipelined: chunk p goes in on copy_in while phase p-1 runs on `stream`
  // and the nodes that phase p-2 finished go out on copy_out.
  if ((s = ensure_pipeline(h, fn)) != OGS_OK) return s;
  if (OGS_HOST_GRAPH) return host_pipeline_graph(h, v, k, type, op, trans, f, pat, node_bytes, st, fn);
  cudaStream_t sin = static_cast<cudaStream_t>(h->copy_in);
  cudaStream_t sout = static_cast<cudaStream_t>(h->copy_out);
  auto ev = [&](size_t i) { return static_cast<cudaEvent_t>(h->events[i]); };
  char* dv = static_cast<char*>(h->stage);
  char* hv = static_cast<char*>(v);
  const std::vector<Phase>& ph = h->lay.phases;
  const size_t P = ph.size();
  // work already queued on the caller's stream comes first
  if ((s = cuda_status(cudaEventRecord(ev(0), st), fn, "event")) != OGS_OK) return s;
  if ((s = cuda_status(cudaStreamWaitEvent(sin, ev(0), 0), fn, "wait")) != OGS_OK) return s;
  for (size_t p = 0; p < P; ++p) {
    const size_t off = static_cast<size_t>(ph[p].h0) * node_bytes, len = static_cast<size_t>(ph[p].h1 - ph[p].h0) * node_bytes;
    if (len && (s = cuda_status(cudaMemcpyAsync(dv + off, hv + off, len, cudaMemcpyHostToDevice, sin), fn,
                                "copy in")) != OGS_OK)
      return s;
    if ((s = cuda_status(cudaEventRecord(ev(1 + 2 * p), sin), fn, "event")) != OGS_OK) return s;
  }
  for (size_t p = 0; p < P; ++p) {
    if ((s = cuda_status(cudaStreamWaitEvent(st, ev(1 + 2 * p), 0), fn, "wait")) != OGS_OK) return s;
    if ((s = launch_maps(phase_maps(h->dmaps, ph[p]), f, kModeGS, op, pat, type, stream, fn)) != OGS_OK) return s;
    if ((s = cuda_status(cudaEventRecord(ev(2 + 2 * p), st), fn, "event")) != OGS_OK) return s;
  }
  for (size_t p = 0; p < P; ++p) {
    const size_t off = static_cast<size_t>(ph[p].d0) * node_bytes, len = static_cast<size_t>(ph[p].d1 - ph[p].d0) * node_bytes;
    if (!len) continue;
    if ((s = cuda_status(cudaStreamWaitEvent(sout, ev(2 + 2 * p), 0), fn, "wait")) != OGS_OK) return s;
    if ((s = cuda_status(cudaMemcpyAsync(hv + off, dv + off, len, cudaMemcpyDeviceToHost, sout), fn, "copy out")) !=
        OGS_OK)
      return s;
  }
  if ((s = cuda_status(cudaStreamSynchronize(sout), fn, "synchronize")) != OGS_OK) return s;
  if ((s = cuda_status(cudaStreamSynchronize(sin), fn, "synchronize")) != OGS_OK) return s;
  return cuda_status(cudaStreamSynchronize(st), fn, "synchronize");
}

// True when the host buffer is page-locked (the sliced pipelines need it:
// copies of pageable memory do not overlap).
bool host_pinned(const void* p) {
  cudaPointerAttributes attr{};
  const bool pinned = cudaPointerGetAttributes(&attr, p) == cudaSuccess && attr.type == cudaMemoryTypeHost;
  cudaGetLastError();
  return pinned;
}

// The sliced copy/compute pipeline of the host-buffer Gather and Scatter
// (the GatherScatter one is in ogs_gather_scatter_host).  Slice p:
//   in  (copy_in):  Gather -- the nodes it reads [h0, h1);
//                   Scatter -- the gathered rows it reads, up to rn, and, if
//                   the scatter leaves some entries alone, the nodes [h0, h1);
//   run (stream):   the slice's kernels, after its copies in;
//   out (copy_out): Gather -- the rows final after it [r0, r1) (below nout);
//                   Scatter -- the nodes final after it [d0, d1).
ogs_status host_pipeline_gs_rows(ogs_handle_s* h, int mode, char* dv, char* dgv, char* hv, char* hgv,
                                 size_t node_bytes, size_t row_bytes, int64_t nout, bool nodes_in,
                                 const FieldArgs& f, int op, Pattern pat, int type, cudaStream_t st, const char* fn) {
  ogs_status s;
  if ((s = ensure_pipeline(h, fn)) != OGS_OK) return s;
  cudaStream_t sin = static_cast<cudaStream_t>(h->copy_in);
  cudaStream_t sout = static_cast<cudaStream_t>(h->copy_out);
  auto ev = [&](size_t i) { return static_cast<cudaEvent_t>(h->events[i]); };
  const std::vector<Phase>& ph = h->lay.phases;
  const size_t P = ph.size();
  if ((s = cuda_status(cudaEventRecord(ev(0), st), fn, "event")) != OGS_OK) return s;
  if ((s = cuda_status(cudaStreamWaitEvent(sin, ev(0), 0), fn, "wait")) != OGS_OK) return s;
  int64_t rows_in = 0;
  for (size_t p = 0; p < P; ++p) {
    if (mode == kModeGather || nodes_in) {
      const size_t off = static_cast<size_t>(ph[p].h0) * node_bytes;
      const size_t len = static_cast<size_t>(ph[p].h1 - ph[p].h0) * node_bytes;
      if (len && (s = cuda_status(cudaMemcpyAsync(dv + off, hv + off, len, cudaMemcpyHostToDevice, sin), fn,
                                  "copy in")) != OGS_OK)
        return s;
    }
    if (mode == kModeScatter) {
      const int64_t upto = std::min<int64_t>(ph[p].rn, nout);
      if (upto > rows_in) {
        const size_t off = static_cast<size_t>(rows_in) * row_bytes;
        const size_t len = static_cast<size_t>(upto - rows_in) * row_bytes;
        if ((s = cuda_status(cudaMemcpyAsync(dgv + off, hgv + off, len, cudaMemcpyHostToDevice, sin), fn,
                             "copy in rows")) != OGS_OK)
          return s;
        rows_in = upto;
      }
    }
    if ((s = cuda_status(cudaEventRecord(ev(1 + 2 * p), sin), fn, "event")) != OGS_OK) return s;
  }
  for (size_t p = 0; p < P; ++p) {
    if ((s = cuda_status(cudaStreamWaitEvent(st, ev(1 + 2 * p), 0), fn, "wait")) != OGS_OK) return s;
    if ((s = launch_maps(phase_maps(h->dmaps, ph[p]), f, mode, op, pat, type, st, fn)) != OGS_OK) return s;
    if ((s = cuda_status(cudaEventRecord(ev(2 + 2 * p), st), fn, "event")) != OGS_OK) return s;
  }
  for (size_t p = 0; p < P; ++p) {
    size_t off, len;
    char *dst, *src;
    if (mode == kModeGather) {
      const int64_t a = std::min<int64_t>(ph[p].r0, nout), b = std::min<int64_t>(ph[p].r1, nout);
      off = static_cast<size_t>(a) * row_bytes;
      len = static_cast<size_t>(b - a) * row_bytes;
      dst = hgv + off;
      src = dgv + off;
    } else {
      off = static_cast<size_t>(ph[p].d0) * node_bytes;
      len = static_cast<size_t>(ph[p].d1 - ph[p].d0) * node_bytes;
      dst = hv + off;
      src = dv + off;
    }
    if (!len) continue;
    if ((s = cuda_status(cudaStreamWaitEvent(sout, ev(2 + 2 * p), 0), fn, "wait")) != OGS_OK) return s;
    if ((s = cuda_status(cudaMemcpyAsync(dst, src, len, cudaMemcpyDeviceToHost, sout), fn, "copy out")) != OGS_OK)
      return s;
  }
  if ((s = cuda_status(cudaStreamSynchronize(sout), fn, "synchronize")) != OGS_OK) return s;
  if ((s = cuda_status(cudaStreamSynchronize(sin), fn, "synchronize")) != OGS_OK) return s;
  return cuda_status(cudaStreamSynchronize(st), fn, "synchronize");
}

ogs_status ogs_gather_host(ogs_handle h, void* gv, const void* v, int k, int type, int op, int trans,
                           void* stream) {
  const char* fn = "ogs_gather_host";
  TraceRange trace(fn);
  ogs_status s = check_common(h, k, type, trans, fn);
  if (s == OGS_OK) s = check_op(op, fn);
  if (s != OGS_OK) return s;
  if (!h->gather_defined) return set_error(OGS_EUNDEFINED, "Gather operation not well-defined.");
  if (h->N == 0 || h->NlocalT == 0) return OGS_OK;
  if (!gv || !v) return set_error(OGS_EINVAL, "ogs_gather_host: NULL buffer");
  std::lock_guard<std::mutex> host_lock(h->host_mu);
  const size_t ts = type_size(type);
  const size_t vb = static_cast<size_t>(h->N) * k * ts;
  const size_t voff = (vb + 255) / 256 * 256;
  const size_t gb = static_cast<size_t>(h->NlocalT) * k * ts;
  if ((s = ensure_stage(h, voff + gb, fn)) != OGS_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(h->stage);
  FieldArgs f{};
  f.v = base;
  f.gv = base + voff;
  f.K = k;
  const int64_t nout = trans == OGS_NOTRANS ? h->NlocalP : h->NlocalT;
  if (OGS_KERNEL == 0 && h->lay.phases.size() >= 2 && host_pinned(v) && host_pinned(gv))
    return host_pipeline_gs_rows(h, kModeGather, base, base + voff, static_cast<char*>(const_cast<void*>(v)),
                                 static_cast<char*>(gv), static_cast<size_t>(k) * ts, static_cast<size_t>(k) * ts,
                                 nout, true, f, op, pattern_for(h, kModeGather, trans), type, st, fn);
  if ((s = cuda_status(cudaMemcpyAsync(base, v, vb, cudaMemcpyHostToDevice, st), fn, "copy in")) != OGS_OK)
    return s;
  if ((s = launch(h, f, kModeGather, op, pattern_for(h, kModeGather, trans), type, stream, fn)) != OGS_OK)
    return s;
  const size_t ob = static_cast<size_t>(nout) * k * ts;
  if ((s = cuda_status(cudaMemcpyAsync(gv, base + voff, ob, cudaMemcpyDeviceToHost, st), fn, "copy out")) != OGS_OK)
    return s;
  return cuda_status(cudaStreamSynchronize(st), fn, "synchronize");
}

ogs_status ogs_scatter_host(ogs_handle h, void* v, const void* gv, int k, int type, int trans, void* stream) {
  const char* fn = "ogs_scatter_host";
  TraceRange trace(fn);
  ogs_status s = check_common(h, k, type, trans, fn);
  if (s == OGS_OK) s = check_writes(h, fn);
  if (s != OGS_OK) return s;
  if (!h->gather_defined) return set_error(OGS_EUNDEFINED, "Gather operation not well-defined.");
  if (h->N == 0 || h->NlocalT == 0) return OGS_OK;
  if (!gv || !v) return set_error(OGS_EINVAL, "ogs_scatter_host: NULL buffer");
  std::lock_guard<std::mutex> host_lock(h->host_mu);
  const size_t ts = type_size(type);
  const size_t vb = static_cast<size_t>(h->N) * k * ts;
  const size_t voff = (vb + 255) / 256 * 256;
  const size_t gb = static_cast<size_t>(h->NlocalT) * k * ts;
  if ((s = ensure_stage(h, voff + gb, fn)) != OGS_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(h->stage);
  const Pattern pat = pattern_for(h, kModeScatter, trans);
  // Entries outside the map keep their values, so v goes in unless the
  // scatter overwrites every entry.
  const bool writes_all = h->covers_all && !pat.scatter_n;
  const int64_t nin = trans == OGS_TRANS ? h->NlocalP : h->NlocalT;
  if (OGS_KERNEL == 0 && h->lay.phases.size() >= 2 && host_pinned(v) && host_pinned(gv)) {
    FieldArgs f{};
    f.v = base;
    f.gv = base + voff;
    f.K = k;
    return host_pipeline_gs_rows(h, kModeScatter, base, base + voff, static_cast<char*>(v),
                                 static_cast<char*>(const_cast<void*>(gv)), static_cast<size_t>(k) * ts,
                                 static_cast<size_t>(k) * ts, nin, !writes_all, f, OGS_ADD, pat, type, st, fn);
  }
  if (!writes_all &&
      (s = cuda_status(cudaMemcpyAsync(base, v, vb, cudaMemcpyHostToDevice, st), fn, "copy in v")) != OGS_OK)
    return s;
  const size_t ib = static_cast<size_t>(trans == OGS_TRANS ? h->NlocalP : h->NlocalT) * k * ts;
  if ((s = cuda_status(cudaMemcpyAsync(base + voff, gv, ib, cudaMemcpyHostToDevice, st), fn, "copy in gv")) !=
      OGS_OK)
    return s;
  FieldArgs f{};
  f.v = base;
  f.gv = base + voff;
  f.K = k;
  if ((s = launch(h, f, kModeScatter, OGS_ADD, pat, type, stream, fn)) != OGS_OK) return s;
  if ((s = cuda_status(cudaMemcpyAsync(v, base, vb, cudaMemcpyDeviceToHost, st), fn, "copy out")) != OGS_OK)
    return s;
  return cuda_status(cudaStreamSynchronize(st), fn, "synchronize");
}

ogs_status ogs_reserve_host(ogs_handle h, int k, int type) {
  const char* fn = "ogs_reserve_host";
  ogs_status s = check_common(h, k, type, OGS_SYM, fn);
  if (s != OGS_OK) return s;
  if (h->N == 0) return OGS_OK;
  // the largest staging any _host call takes for this k and type: the field,
  // 256-byte aligned, then the gathered vector (Gather / Scatter)
  const size_t nb = static_cast<size_t>(k) * type_size(type);
  const size_t voff = (static_cast<size_t>(h->N) * nb + 255) / 256 * 256;
  const size_t bytes = voff + static_cast<size_t>(h->NlocalT) * nb;
  std::lock_guard<std::mutex> host_lock(h->host_mu);
  if ((s = ensure_stage(h, bytes, fn)) != OGS_OK) return s;
  if (h->lay.phases.size() >= 2) return ensure_pipeline(h, fn);
  return OGS_OK;
}

ogs_status ogs_get_counts(ogs_handle h, ogs_counts* out) {
  if (!h || !out) return set_error(OGS_EINVAL, "ogs_get_counts: NULL argument");
  out->N = h->N;
  out->Ngather = h->Ngather;
  out->NgatherGlobal = h->NgatherGlobal;
  out->NlocalP = h->NlocalP;
  out->NlocalT = h->NlocalT;
  out->nnzT = h->nnzT;
  out->nnzN = h->nnzN;
  out->gather_defined = h->gather_defined;
  out->kind = h->kind;
  out->unique = h->unique;
  out->max_degree = h->max_degree;
  return OGS_OK;
}

ogs_status ogs_get_maps(ogs_handle h, int32_t* rowStartsT, int32_t* colIdsT, int32_t* rowStartsN,
                        int32_t* colIdsN) {
  if (!h) return set_error(OGS_EINVAL, "ogs_get_maps: handle is NULL");
  const bool sgn = h->kind == OGS_SIGNED;
  const std::vector<int32_t>& rsN = sgn ? h->rowStartsN : h->rowStartsT;
  const std::vector<int32_t>& ciN = sgn ? h->colIdsN : h->colIdsT;
  if (rowStartsT) std::memcpy(rowStartsT, h->rowStartsT.data(), h->rowStartsT.size() * 4);
  if (colIdsT && !h->colIdsT.empty()) std::memcpy(colIdsT, h->colIdsT.data(), h->colIdsT.size() * 4);
  if (rowStartsN) std::memcpy(rowStartsN, rsN.data(), rsN.size() * 4);
  if (colIdsN && !ciN.empty()) std::memcpy(colIdsN, ciN.data(), ciN.size() * 4);
  return OGS_OK;
}

ogs_status ogs_checked_id_errors(ogs_handle h, uint64_t* count) {
  if (!h || !count) return set_error(OGS_EINVAL, "ogs_checked_id_errors: NULL argument");
  *count = 0;
  if (h->host_only || !h->arena || !h->dmaps.b[1].err) return OGS_OK;
  unsigned int v = 0;
  const cudaError_t e = cudaMemcpy(&v, h->dmaps.b[1].err, sizeof(v), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e, "ogs_checked_id_errors", "copy");
  *count = v;
  return OGS_OK;
}

ogs_status ogs_get_layout_stats(ogs_handle h, ogs_layout_stats* out) {
  if (!h || !out) return set_error(OGS_EINVAL, "ogs_get_layout_stats: NULL argument");
  std::memset(out, 0, sizeof(*out));
  for (int d = 1; d <= kDmax; ++d) out->rows_by_degree[d] = h->lay.n[d];
  out->rows_by_degree[0] = h->lay.g_n;
  out->nnz_general = h->lay.g_nnzT;
  out->ntiles = static_cast<int64_t>(h->lay.tiles.size());
  out->nwarp_tiles = static_cast<int64_t>(h->lay.wtiles.size());
  out->ngeneral_tiles = static_cast<int64_t>(h->lay.gtiles.size());
  out->device_bytes = static_cast<int64_t>(h->arena_bytes);
  out->nphases = static_cast<int64_t>(h->lay.phases.size());
  for (size_t p = 0; p < h->lay.phases.size() && p < 32; ++p) {
    const Phase& q = h->lay.phases[p];
    out->phases[p][0] = q.lo;
    out->phases[p][1] = q.hi;
    out->phases[p][2] = q.h1;
    out->phases[p][3] = q.d1;
    out->phase_rows[p][0] = q.r1;
    out->phase_rows[p][1] = q.rn;
  }
  return OGS_OK;
}

}  // extern "C"
