// NVTX ranges around the library's bulk entry points, so that a profiler
// (`ncu --clock-control none --nvtx --nvtx-include ...`, Nsight Systems) can
// attribute each kernel to the call that launched it.  NVTX v3 is header-only; with no tool attached
// a push or pop costs a pointer check.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace gh {
namespace trace {

struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

}  // namespace trace
}  // namespace gh
