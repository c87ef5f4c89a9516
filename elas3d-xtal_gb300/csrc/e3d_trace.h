// NVTX ranges around the library's public entry points, so that a profiler
// timeline shows femat / energy / PCG / stress / batch / serve phases by name.
// NVTX 3 is header-only and does nothing unless a tool is attached.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace e3d {

struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace e3d

#define E3D_TRACE(name) ::e3d::TraceRange e3d_trace_range_(name)
