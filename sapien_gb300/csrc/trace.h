// NVTX ranges around the C-ABI compute entry points, so a timeline (Nsight Systems or
// Compute) shows which library call launched which kernels. NVTX v3 is header-only and
// only loads an injection library when a profiler provides one; otherwise a range costs a
// function-pointer check.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace sgdyn {
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};
}  // namespace sgdyn

#define SG_TRACE(name) ::sgdyn::TraceRange sg_trace_range_(name)
