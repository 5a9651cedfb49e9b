// mmf_fast.cu -- fast-arithmetic instantiation of the stage kernels (one
// reciprocal and one square root per cell).  Built without implicit FMA
// contraction: every fused multiply-add is written out, so a cell's bits do
// not depend on how the compiler unrolled the marching loop, and therefore
// not on the work decomposition either.
#include "mmf_batch.cuh"
#include "mmf_exact_occupancy.h"
#include "mmf_launch.cuh"

namespace mmf {

cudaError_t launch_stage_fast(int stage, const GridParams &gp, const StageArgs &sa, cudaStream_t s, bool w_zero)
{
    if (gp.dim == 2 && w_zero) return launch_stage<FastArith2DW0, false>(stage, gp, sa, s);
    return launch_stage<FastArith>(stage, gp, sa, s);
}

void prime_tile3d_fast() { prime_tile3d_slots<FastArith>(); }

cudaError_t launch_o2_fast(int op, int stage, const GridParams &gp, const StageArgs &sa, const O2Args &oa,
                           double *W1, cudaStream_t s, bool w_zero)
{
    if (gp.dim == 2 && w_zero) return launch_o2<FastArith2DW0, false>(op, stage, gp, sa, oa, W1, s);
    return launch_o2<FastArith>(op, stage, gp, sa, oa, W1, s);
}

cudaError_t launch_batch_fast(int stage, const CaseDesc *cases, const int *item_case, int nitems, Ctrl *cctrl,
                              const StageArgs &base, int blocks, cudaStream_t s, bool w_zero)
{
    if (w_zero) return launch_batch<FastArith2DW0>(stage, cases, item_case, nitems, cctrl, base, blocks, s);
    return launch_batch<FastArith>(stage, cases, item_case, nitems, cctrl, base, blocks, s);
}

cudaError_t launch_batch_o2_fast(int op, int stage, const CaseDesc *cases, const int *item_case, int nitems,
                                 Ctrl *cctrl, const StageArgs &base, const double *state, const O2Batch &ob,
                                 double *W1, int blocks, cudaStream_t s, bool w_zero)
{
    if (w_zero)
        return launch_batch_o2<FastArith2DW0>(op, stage, cases, item_case, nitems, cctrl, base, state, ob, W1, blocks, s);
    return launch_batch_o2<FastArith>(op, stage, cases, item_case, nitems, cctrl, base, state, ob, W1, blocks, s);
}

int batch_slope_blocks_per_sm(int arith, bool w_zero)
{
    if (arith == 0) return batch_slope_blocks_per_sm_exact();
    return w_zero ? batch_slopes_blocks_per_sm<FastArith2DW0>() : batch_slopes_blocks_per_sm<FastArith>();
}

int batch_max_blocks_per_sm(int arith, bool w_zero, int order)
{
    if (arith == 0) return batch_max_blocks_per_sm_exact(order);
    if (order == 2) return w_zero ? batch_o2_blocks_per_sm<FastArith2DW0>() : batch_o2_blocks_per_sm<FastArith>();
    return w_zero ? batch_blocks_per_sm<FastArith2DW0>() : batch_blocks_per_sm<FastArith>();
}

__global__ void newton_selftest_kernel(long long n, const double *x, double *r, double *q)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    r[i] = rcp_newton(x[i]);
    q[i] = sqrt_newton(x[i]);
}

cudaError_t launch_screen_selftest_fast(int nv, int dim, long long n, const double *uc, const double *sig, int *dec,
                                       unsigned char *ref, cudaStream_t s)
{
    if (nv == 4) return launch_screen_selftest<FastArith2DW0>(dim, n, uc, sig, dec, ref, s);
    return launch_screen_selftest<FastArith>(dim, n, uc, sig, dec, ref, s);
}

cudaError_t launch_newton_selftest(long long n, const double *x, double *r, double *q, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    newton_selftest_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n, x, r, q);
    return cudaPeekAtLastError();
}

} // namespace mmf
