// chaos_trace.h -- NVTX ranges around the library's calls.
//
// Every public call that renders (frames, reference-mode kernels, compose,
// renderer frames, batch launches, perturbation frames, orbits, served
// launches) opens a range in the NVTX domain "chaos_gb300", named after the
// call.  NVTX is header-only: without a profiler attached the calls cost a
// branch; under Nsight Compute a capture can be limited to one of them
// (ncu --nvtx --nvtx-include "chaos_gb300@chaos_render_frame/").  The ranges
// are host-side: an asynchronous call's range covers its enqueue.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace chaos {

inline nvtxDomainHandle_t trace_domain()
{
    static nvtxDomainHandle_t d = nvtxDomainCreateA("chaos_gb300");
    return d;
}

struct TraceRange {
    explicit TraceRange(const char *name)
    {
        nvtxEventAttributes_t a = {};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(trace_domain(), &a);
    }
    ~TraceRange() { nvtxDomainRangePop(trace_domain()); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace chaos
