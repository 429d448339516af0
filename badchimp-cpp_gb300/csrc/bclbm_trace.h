// NVTX ranges around the library's entry points, so that a profiler's timeline
// shows create / step / download / reduce / batch / output calls.  Without a
// tool attached an NVTX call returns at once.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace bclbm {

struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace bclbm

#define BCLBM_TRACE(name) ::bclbm::TraceRange bclbm_trace_range_(name)
