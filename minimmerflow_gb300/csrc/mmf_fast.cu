// mmf_fast.cu -- fast-arithmetic instantiation of the stage kernels (FMA
// contraction on; one division and one square root per cell).
#include "mmf_launch.cuh"

namespace mmf {

cudaError_t launch_stage_fast(int stage, const GridParams &gp, const StageArgs &sa, cudaStream_t s)
{
    return launch_stage<FastArith>(stage, gp, sa, s);
}

} // namespace mmf
