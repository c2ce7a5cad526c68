// NVTX ranges over the C-ABI calls, so a profiler's timeline (Nsight Systems)
// and ncu's --nvtx filters show which call issued which kernels.  NVTX3 is
// header-only: with no tool attached a range is one indirect call that
// returns at once.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace bmf {

struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace bmf

#define BMF_TRACE(name) ::bmf::TraceRange bmf_trace_range_(name)
