// trace.h -- NVTX ranges around the library's host phases (header-only NVTX 3; a no-op unless a
// profiler such as Nsight Systems is attached), so a timeline shows equilibration, tracer,
// Poisson-Nernst-Planck, batch and serving phases by name.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace lbg {

struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace lbg
