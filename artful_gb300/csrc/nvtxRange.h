/* artful_cuda — named ranges on a profiler's timeline (NVTX, header-only): each entry point that
 * launches work opens one for its whole call, so a capture shows which call each kernel came from.
 * With no tool attached a range costs a test of a null pointer. */
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace artf {

struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

}  // namespace artf
