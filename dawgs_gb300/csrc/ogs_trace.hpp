// ogs_trace.hpp -- NVTX ranges on the host timeline: setup and its map and
// layout builds, the host-buffer calls, batch calls and tuning, server
// batches and the halo steps, for Nsight Systems and other NVTX tools.  With
// no tool attached a range costs a check of one pointer.  Build with
// -DOGS_NVTX=0 to leave them out.
#pragma once

#ifndef OGS_NVTX
#define OGS_NVTX 1
#endif
#if OGS_NVTX
#include <nvtx3/nvToolsExt.h>
#endif

namespace ogsgb {

class TraceRange {
 public:
  explicit TraceRange(const char* name) {
#if OGS_NVTX
    nvtxRangePushA(name);
#else
    (void)name;
#endif
  }
  ~TraceRange() {
#if OGS_NVTX
    nvtxRangePop();
#endif
  }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace ogsgb
