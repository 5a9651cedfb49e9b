// mmf_launch.cuh -- host-side launch shapes of the stage kernels.  Included by
// the two arithmetic translation units (mmf_exact.cu, built with -fmad=false,
// and mmf_fast.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "mmf_cartesian.cuh"
#include "mmf_order2.cuh"

namespace mmf {

constexpr int BY3D = 16;        // warps per 3D block (14 output rows + 2 halo rows)
constexpr int WARPS_2D = 4;     // warps per 2D block
constexpr int BY3D_O2 = 16;     // warps per 3D order-2 block (14 output rows + 2 halo rows)
// order-1 3D kernel when nothing else is chosen: the tile kernel, one block
// per resident slot
constexpr int TILE3D_DEFAULT = 2;

// Fills the decomposition fields of gp for the given marching chunk; 'by' is
// the number of warps a 3D block stacks in y (two of them halo rows) in the
// row-block kernel; tile3d selects the 3D tile kernel (order 1 only: 1 = one
// block per tile and chunk, 2 = at most one block per resident slot, on
// units of 'chunk' planes that a band launch keeps); order 2 in 3D has rows
// of SEG3D_O2 output columns.
inline void plan_cartesian(GridParams &gp, int chunk, int by = 16, int wpb = 0, int tile3d = 0, int order = 1)
{
    const int seg = (gp.dim == 3 && order == 2) ? SEG3D_O2 : SEG;
    gp.nseg = (gp.n[0] + seg - 1) / seg;
    gp.wpb = (wpb >= 1 && wpb <= WARPS_2D) ? wpb : WARPS_2D;
    gp.tile3d = (gp.dim == 3 && tile3d >= 1 && tile3d <= 2) ? tile3d : 0;
    gp.chunk0 = 0;
    gp.bookkeep = 1;
    gp.unit = chunk > 0 ? chunk : 32;
    if (gp.dim == 2) {
        gp.chunk = chunk > 0 ? chunk : 32;
        gp.nchunk = (gp.n[1] + gp.chunk - 1) / gp.chunk;
        gp.nrowblk = 1;
    } else {
        gp.chunk = chunk > 0 ? chunk : 32;
        gp.nchunk = (gp.n[2] + gp.chunk - 1) / gp.chunk;
        gp.nrowblk = (gp.n[1] + by - 3) / (by - 2);
    }
    gp.plane = (long long)gp.n[0] * gp.n[1] * gp.n[2];
}

// Kernel launches this decomposition makes per stage (for launch counting).
inline long long cartesian_blocks(const GridParams &gp)
{
    if (gp.dim == 2) {
        long long warps = (long long)gp.nseg * gp.nchunk;
        return (warps + gp.wpb - 1) / gp.wpb;
    }
    if (gp.tile3d)
        return (long long)((gp.n[0] + TILE_X - 1) / TILE_X) * ((gp.n[1] + TILE_Y - 1) / TILE_Y) * gp.nchunk;
    return (long long)gp.nseg * gp.nrowblk * gp.nchunk;
}

// Blocks of the 3D tile kernel that are resident at once on the current
// device (SMs x blocks per SM), found once per kernel.
template <class A, int STAGE>
inline long long tile3d_slots()
{
    static const long long slots = [] {
        int dev = 0, sms = 0, per_sm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stage3d_tile_kernel<A, STAGE>, TILE_X * TILE_Y,
                                                          0) != cudaSuccess) {
            cudaGetLastError();
            return 152LL;
        }
        return (long long)std::max(sms, 1) * std::max(per_sm, 1);
    }();
    return slots;
}

// The slot counts of the four stage instantiations, found before a stream
// capture so that no occupancy query runs inside one.
template <class A>
inline void prime_tile3d_slots()
{
    tile3d_slots<A, STAGE_RHS>();
    tile3d_slots<A, STAGE_1>();
    tile3d_slots<A, STAGE_2>();
    tile3d_slots<A, STAGE_3>();
}

template <class A, int STAGE, bool HAS3D>
inline cudaError_t launch_stage_t(const GridParams &gp, const StageArgs &sa, cudaStream_t s)
{
    long long nb = cartesian_blocks(gp);
    if constexpr (HAS3D) {
        // at most one block per slot, and at least a plane per block
        if (gp.dim == 3 && gp.tile3d == 2) {
            const long long zlo = (long long)gp.chunk0 * gp.chunk;
            const long long nzr = std::min<long long>(gp.n[2], zlo + (long long)gp.nchunk * gp.chunk) - zlo;
            const long long ntiles =
                (long long)((gp.n[0] + TILE_X - 1) / TILE_X) * ((gp.n[1] + TILE_Y - 1) / TILE_Y);
            nb = std::min(ntiles * nzr, tile3d_slots<A, STAGE>());
        }
    }
    const unsigned blocks = (unsigned)nb;
    if (gp.dim == 2) {
        stage2d_kernel<A, STAGE><<<blocks, gp.wpb * 32, 0, s>>>(gp, sa);
    } else {
        if constexpr (HAS3D) {
            if (gp.tile3d) stage3d_tile_kernel<A, STAGE><<<blocks, TILE_X * TILE_Y, 0, s>>>(gp, sa);
            else stage3d_kernel<A, STAGE, BY3D><<<blocks, BY3D * 32, 0, s>>>(gp, sa);
        } else {
            return cudaErrorInvalidValue;
        }
    }
    return cudaPeekAtLastError();
}

template <class A, bool HAS3D = true>
inline cudaError_t launch_stage(int stage, const GridParams &gp, const StageArgs &sa, cudaStream_t s)
{
    switch (stage) {
    case STAGE_RHS: return launch_stage_t<A, STAGE_RHS, HAS3D>(gp, sa, s);
    case STAGE_1: return launch_stage_t<A, STAGE_1, HAS3D>(gp, sa, s);
    case STAGE_2: return launch_stage_t<A, STAGE_2, HAS3D>(gp, sa, s);
    case STAGE_3: return launch_stage_t<A, STAGE_3, HAS3D>(gp, sa, s);
    default: return cudaErrorInvalidValue;
    }
}

// ---- order 2 --------------------------------------------------------------
enum O2Op { O2_SLOPES = 0, O2_FORM_W1 = 1, O2_STAGE = 2 };

inline unsigned elementwise_blocks(long long n)
{
    long long b = (n + 255) / 256;
    return (unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}

template <class A, int STAGE, bool HAS3D>
inline cudaError_t launch_o2_stage_t(const GridParams &gp, const StageArgs &sa, const O2Args &oa, cudaStream_t s)
{
    const unsigned blocks = (unsigned)cartesian_blocks(gp);
    if (gp.dim == 2) {
        stage2d_o2_kernel<A, STAGE><<<blocks, gp.wpb * 32, 0, s>>>(gp, sa, oa.state, oa.S);
    } else {
        if constexpr (HAS3D) stage3d_o2_kernel<A, STAGE, BY3D_O2><<<blocks, BY3D_O2 * 32, 0, s>>>(gp, sa, oa.state, oa.S);
        else return cudaErrorInvalidValue;
    }
    return cudaPeekAtLastError();
}

template <class A, bool HAS3D = true>
inline cudaError_t launch_o2(int op, int stage, const GridParams &gp, const StageArgs &sa, const O2Args &oa,
                             double *W1, cudaStream_t s)
{
    switch (op) {
    case O2_SLOPES:
        if (gp.dim == 2) slopes_kernel<A, 2><<<elementwise_blocks(oa.cell1 - oa.cell0), 256, 0, s>>>(gp, oa);
        else {
            if constexpr (HAS3D) slopes_kernel<A, 3><<<elementwise_blocks(oa.cell1 - oa.cell0), 256, 0, s>>>(gp, oa);
            else return cudaErrorInvalidValue;
        }
        return cudaPeekAtLastError();
    case O2_FORM_W1:
        // four blocks per SM: each thread divides once for dt (an FP64 division
        // sequence), so fewer threads, each with more cells
        form_w1_kernel<A><<<std::min(elementwise_blocks(gp.plane), 4u * 152u), 256, 0, s>>>(gp, sa, W1);
        return cudaPeekAtLastError();
    case O2_STAGE:
        switch (stage) {
        case STAGE_RHS: return launch_o2_stage_t<A, STAGE_RHS, HAS3D>(gp, sa, oa, s);
        case STAGE_1: return launch_o2_stage_t<A, STAGE_1, HAS3D>(gp, sa, oa, s);
        case STAGE_2: return launch_o2_stage_t<A, STAGE_2, HAS3D>(gp, sa, oa, s);
        case STAGE_3: return launch_o2_stage_t<A, STAGE_3, HAS3D>(gp, sa, oa, s);
        default: return cudaErrorInvalidValue;
        }
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_o2_exact(int op, int stage, const GridParams &gp, const StageArgs &sa, const O2Args &oa,
                            double *W1, cudaStream_t s);
cudaError_t launch_o2_fast(int op, int stage, const GridParams &gp, const StageArgs &sa, const O2Args &oa,
                           double *W1, cudaStream_t s, bool w_zero);

// Entry points of the two arithmetic translation units.  w_zero selects the
// 2D kernels that skip the identically-zero z-momentum.
cudaError_t launch_stage_exact(int stage, const GridParams &gp, const StageArgs &sa, cudaStream_t s);
cudaError_t launch_stage_fast(int stage, const GridParams &gp, const StageArgs &sa, cudaStream_t s, bool w_zero);
void prime_tile3d_exact();
void prime_tile3d_fast();

// Self-test of the FP32 positivity screen of the order-2 slopes (nv 4: the 2D
// four-field layout of the fast arithmetic).
cudaError_t launch_screen_selftest_fast(int nv, int dim, long long n, const double *uc, const double *sig, int *dec,
                                       unsigned char *ref, cudaStream_t s);
cudaError_t launch_screen_selftest_exact(int dim, long long n, const double *uc, const double *sig, int *dec,
                                        unsigned char *ref, cudaStream_t s);

// Reciprocal and square root of the fast arithmetic, for the self-test.
cudaError_t launch_newton_selftest(long long n, const double *x, double *r, double *q, cudaStream_t s);

// Pointwise kernels of the reference's unit-level functions (exact arithmetic).
enum PointOp { OP_CONS2PRIM = 0, OP_PRIM2CONS = 1, OP_FLUXES = 2, OP_SPLITTING = 3, OP_BC = 4 };
cudaError_t launch_pointwise_exact(int op, long long n, const double *a, const double *b, const double *nrm,
                                   int bc, const double *dir_prim, double *out, double *out2, cudaStream_t s);

} // namespace mmf
