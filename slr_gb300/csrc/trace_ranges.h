// NVTX ranges of the renderer's host-side stages (render call, wave,
// bounce, scene build and upload, server admission and waves), in the
// "slrgpu" domain, so that a profiler's timeline (ncu --nvtx, Nsight
// Systems) groups the kernels by what launched them.  NVTX v3 is
// header-only: without a profiler attached each range costs one call
// through a null function pointer.
#pragma once
#include <nvtx3/nvToolsExt.h>

#include <cstdarg>
#include <cstdio>

namespace slrgpu {

inline nvtxDomainHandle_t traceDomain() {
    static nvtxDomainHandle_t d = nvtxDomainCreateA("slrgpu");
    return d;
}

// A range from construction to destruction; the name may be printf-style.
class TraceRange {
public:
    explicit TraceRange(const char* fmt, ...) {
        char buf[96];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        nvtxEventAttributes_t a = {};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = buf;
        nvtxDomainRangePushEx(traceDomain(), &a);
    }
    ~TraceRange() { nvtxDomainRangePop(traceDomain()); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace slrgpu
