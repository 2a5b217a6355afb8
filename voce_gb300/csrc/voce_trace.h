// NVTX ranges around the library's host-side phases: creating an RVE (and
// its tile timing), running increments, batch ticks, server polls, field
// downloads, snapshots.  A profiler that records NVTX (ncu --nvtx, Nsight
// Systems) shows them on the host timeline beside the kernels.  NVTX 3 is
// header-only: with no tool attached a range costs one check of a function
// pointer.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace voce {

struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace voce

#define VOCE_TRACE(name) ::voce::TraceRange voce_trace_range_(name)
