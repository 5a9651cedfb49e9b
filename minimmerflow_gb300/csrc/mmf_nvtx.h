// mmf_nvtx.h -- named ranges on the profiler timeline (NVTX, header-only) for
// the host entry points; without a profiler attached they cost nothing
// measurable.
#pragma once

#include <nvtx3/nvToolsExt.h>

struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
