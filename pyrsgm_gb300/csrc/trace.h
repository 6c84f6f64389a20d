// trace.h -- NVTX ranges around the library's host-side stages, so that a
// profiler timeline (Nsight Systems, or ncu's NVTX filters) shows the
// pyramid levels of a compute(), the rounds of a batch and the life of a
// served request.  NVTX v3 is header-only: without a tool attached every
// call is a cheap no-op.
#pragma once

#include <nvtx3/nvToolsExt.h>

#include <cstdio>

namespace pg {

// Push / pop on the calling thread.
class TraceRange {
public:
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    template <class... A>
    TraceRange(const char* fmt, A... args)
    {
        char buf[96];
        std::snprintf(buf, sizeof buf, fmt, args...);
        nvtxRangePushA(buf);
    }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// A range that may end on another thread (a served request: submitted on
// the caller's thread, completed on a lane's).
inline unsigned long long trace_start(const char* name) { return nvtxRangeStartA(name); }
inline void trace_end(unsigned long long id) { nvtxRangeEnd(id); }

}  // namespace pg
