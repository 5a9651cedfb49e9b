// mmf_batch.cuh -- many independent 2D cases of uneven size in one persistent
// launch per Runge-Kutta stage.
//
// The cases' states are packed field-plane by field-plane: field k of case c
// is at base + k * total + offset_c, row-major inside the case.  The work of
// a stage is a flat list of items, one per (case, 30-column segment, row
// chunk), in case order; the persistent grid (a few blocks per SM) walks the
// list warp by warp.  Each case keeps its own control block (time, dt, maxEig,
// step, status), so dt is a per-case CFL reduction: a stage-1 item reduces its
// maxEig into its case's slot, stage-2 items derive their case's dt from it,
// and the first item of a case does that case's per-launch bookkeeping.  The
// arithmetic of an item is the single-grid march (march2d), so every case
// gets exactly the result it would get alone.
#pragma once

#include "mmf_cartesian.cuh"
#include "mmf_order2.cuh"

namespace mmf {

struct CaseDesc {
    GridParams gp;        // grid of the case (gp.plane = field stride of the packed planes)
    long long offset;     // first cell of the case in the packed planes
    int item0;            // first work item of the case
    int pad;
};

template <class A, int STAGE>
__global__ void __launch_bounds__(128) stage2d_batch_kernel(const CaseDesc *__restrict__ cases,
                                                            const int *__restrict__ item_case, int nitems,
                                                            Ctrl *cctrl, StageArgs base)
{
    const int warp0 = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    const int lane = threadIdx.x & 31;
    for (int item = warp0; item < nitems; item += nwarps) {
        const int c = item_case[item];
        const GridParams gp = cases[c].gp;
        const long long off = cases[c].offset;
        const int local = item - cases[c].item0;
        Ctrl *ctrl = cctrl + c;
        const StepScalars sc = step_scalars<A, STAGE>(gp, ctrl);
        if (local == 0 && lane == 0) step_bookkeeping<STAGE>(ctrl, sc);
        if (!sc.active) continue;
        StageArgs sa = base;
        sa.U = base.U + off;
        sa.R = base.R + off;
        sa.W = base.W + off;
        sa.out = base.out + off;
        sa.ctrl = ctrl;
        double lmax = 0.0;
        unsigned status = 0;
        march2d<A, STAGE>(gp, sa, sc, local % gp.nseg, local / gp.nseg, lmax, status);
        publish_reductions<STAGE>(lmax, status, ctrl, nullptr);
    }
}

template <class A>
inline cudaError_t launch_batch(int stage, const CaseDesc *cases, const int *item_case, int nitems, Ctrl *cctrl,
                                const StageArgs &base, int blocks, cudaStream_t s)
{
    switch (stage) {
    case STAGE_1: stage2d_batch_kernel<A, STAGE_1><<<blocks, 128, 0, s>>>(cases, item_case, nitems, cctrl, base); break;
    case STAGE_2: stage2d_batch_kernel<A, STAGE_2><<<blocks, 128, 0, s>>>(cases, item_case, nitems, cctrl, base); break;
    case STAGE_3: stage2d_batch_kernel<A, STAGE_3><<<blocks, 128, 0, s>>>(cases, item_case, nitems, cctrl, base); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaPeekAtLastError();
}

template <class A>
inline int batch_blocks_per_sm()
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stage2d_batch_kernel<A, STAGE_2>, 128, 0) != cudaSuccess)
        return 1;
    return nb > 0 ? nb : 1;
}

// ---- order 2 -----------------------------------------------------------------
struct O2Batch {
    double *S;                 // packed slopes: plane (d * NV + k) at S + (d * NV + k) * total
    unsigned char *flag;       // packed limiter flags
    unsigned char *active;     // packed limiter activity (nullable)
    int limit_mode;
    int *tick = nullptr;       // the indicator's step counter, advanced by a step's stage-1 slopes (nullable)
};

// Walks the item list; for each item of an active case calls body(gp, off, ctrl, seg, chunk).
template <class Body>
__device__ __forceinline__ void for_items(const CaseDesc *cases, const int *item_case, int nitems, Ctrl *cctrl,
                                          Body body)
{
    const int warp0 = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int item = warp0; item < nitems; item += nwarps) {
        const int c = item_case[item];
        const GridParams gp = cases[c].gp;
        const int local = item - cases[c].item0;
        body(gp, cases[c].offset, cctrl + c, local % gp.nseg, local / gp.nseg, local == 0);
    }
}

// Minimum resident blocks per SM the batch slope kernel is compiled for; it
// has its own grid (items are dealt to warps by for_items): five blocks of
// four warps (at most 102 registers) for the fast arithmetic, the most
// without spills (at six it spills 16-32 B, at eight 68-88 B).
template <class A> struct SlopesBatchMinBlocks { static constexpr int value = 1; };
template <int NV> struct SlopesBatchMinBlocks<FastArithT<NV>> { static constexpr int value = 5; };

// slopes (computePolynomials) of the output cells of every item
template <class A>
__global__ void __launch_bounds__(128, SlopesBatchMinBlocks<A>::value) slopes_batch_kernel(const CaseDesc *__restrict__ cases,
                                                           const int *__restrict__ item_case, int nitems, Ctrl *cctrl,
                                                           const double *state, O2Batch ob, int stage)
{
    const int lane = threadIdx.x & 31;
    // no block of this launch reads the counter
    if (ob.tick && blockIdx.x == 0 && threadIdx.x == 0) *ob.tick += 1;
    for_items(cases, item_case, nitems, cctrl, [&](const GridParams &gp, long long off, Ctrl *ctrl, int seg, int chunk,
                                                   bool) {
        if (!o2_step_active(ctrl, stage)) return;
        O2Args oa;
        oa.state = state + off;
        oa.S = ob.S + off;
        oa.flag = ob.flag + off;
        oa.active = ob.active ? ob.active + off : nullptr;
        oa.limit_mode = ob.limit_mode;
        oa.ctrl = ctrl;
        oa.stage = stage;
        const int x = seg * SEG - 1 + lane;
        if (lane < 1 || lane > SEG || x >= gp.n[0]) return;
        const int y1 = min((chunk + 1) * gp.chunk, gp.n[1]);
        for (int y = chunk * gp.chunk; y < y1; ++y) slopes_cell<A, 2>(gp, oa, (long long)x + (long long)gp.n[0] * y);
    });
}

// W1 = U + dt R1 / V of the output cells of every item (per-case dt)
template <class A>
__global__ void __launch_bounds__(128) form_w1_batch_kernel(const CaseDesc *__restrict__ cases,
                                                            const int *__restrict__ item_case, int nitems, Ctrl *cctrl,
                                                            StageArgs base, double *W1)
{
    const int lane = threadIdx.x & 31;
    for_items(cases, item_case, nitems, cctrl, [&](const GridParams &gp, long long off, Ctrl *ctrl, int seg, int chunk,
                                                   bool first) {
        const StepScalars sc = step_scalars<A, STAGE_2>(gp, ctrl);
        if (first && lane == 0 && sc.active) ctrl->dt = sc.dt;
        if (!sc.active) return;
        StageArgs sa = base;
        sa.U = base.U + off;
        sa.R = base.R + off;
        const int x = seg * SEG - 1 + lane;
        if (lane < 1 || lane > SEG || x >= gp.n[0]) return;
        const int y1 = min((chunk + 1) * gp.chunk, gp.n[1]);
        for (int y = chunk * gp.chunk; y < y1; ++y) {
            const long long g = (long long)x + (long long)gp.n[0] * y;
#pragma unroll
            for (int k = 0; k < A::NVAR; ++k) {
                const long long o = (long long)A::field(k) * gp.plane + g;
                W1[off + o] = form_w1_value<A>(sa, gp, sc, o);
            }
        }
    });
}

// Minimum resident blocks per SM the order-2 batch march is compiled for:
// the four-field fast variant (2D states with zero z-momentum, the batched
// sweep's) gets 128 registers, so that four persistent blocks of four warps
// fit on an SM (at five, 102 registers, it spills 200-260 B).
template <class A> struct O2BatchMinBlocks { static constexpr int value = 1; };
template <> struct O2BatchMinBlocks<FastArithT<4>> { static constexpr int value = 4; };

// order-2 stage march of every item
template <class A, int STAGE>
__global__ void __launch_bounds__(128, O2BatchMinBlocks<A>::value) stage2d_o2_batch_kernel(const CaseDesc *__restrict__ cases,
                                                               const int *__restrict__ item_case, int nitems,
                                                               Ctrl *cctrl, StageArgs base, const double *state,
                                                               const double *S)
{
    const int lane = threadIdx.x & 31;
    for_items(cases, item_case, nitems, cctrl, [&](const GridParams &gp, long long off, Ctrl *ctrl, int seg, int chunk,
                                                   bool first) {
        const StepScalars sc = step_scalars<A, STAGE>(gp, ctrl);
        if (first && lane == 0) step_bookkeeping<STAGE>(ctrl, sc);
        if (!sc.active) return;
        StageArgs sa = base;
        sa.U = base.U + off;
        sa.R = base.R + off;
        sa.W = base.W + off;
        sa.out = base.out + off;
        sa.ctrl = ctrl;
        double lmax = 0.0;
        unsigned status = 0;
        march2d_o2<A, STAGE>(gp, sa, state + off, S + off, sc, seg, chunk, lmax, status);
        publish_reductions<STAGE>(lmax, status, ctrl, nullptr);
    });
}

enum BatchO2Op { BO2_SLOPES = 0, BO2_FORM_W1 = 1, BO2_STAGE = 2 };

// Resident blocks per SM of the order-2 batch stage marches and W1 (the
// persistent grid they share).
template <class A>
inline int batch_o2_blocks_per_sm()
{
    int nb = 1 << 20, v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, stage2d_o2_batch_kernel<A, STAGE_1>, 128, 0) == cudaSuccess) nb = v < nb ? v : nb;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, stage2d_o2_batch_kernel<A, STAGE_2>, 128, 0) == cudaSuccess) nb = v < nb ? v : nb;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, stage2d_o2_batch_kernel<A, STAGE_3>, 128, 0) == cudaSuccess) nb = v < nb ? v : nb;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, form_w1_batch_kernel<A>, 128, 0) == cudaSuccess) nb = v < nb ? v : nb;
    return (nb > 0 && nb < (1 << 20)) ? nb : 1;
}

// ... of the batch slope kernel (its own grid)
template <class A>
inline int batch_slopes_blocks_per_sm()
{
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, slopes_batch_kernel<A>, 128, 0) != cudaSuccess || v < 1) return 1;
    return v;
}

template <class A>
inline cudaError_t launch_batch_o2(int op, int stage, const CaseDesc *cases, const int *item_case, int nitems,
                                   Ctrl *cctrl, const StageArgs &base, const double *state, const O2Batch &ob,
                                   double *W1, int blocks, cudaStream_t s)
{
    switch (op) {
    case BO2_SLOPES: slopes_batch_kernel<A><<<blocks, 128, 0, s>>>(cases, item_case, nitems, cctrl, state, ob, stage); break;
    case BO2_FORM_W1: form_w1_batch_kernel<A><<<blocks, 128, 0, s>>>(cases, item_case, nitems, cctrl, base, W1); break;
    case BO2_STAGE:
        switch (stage) {
        case STAGE_1: stage2d_o2_batch_kernel<A, STAGE_1><<<blocks, 128, 0, s>>>(cases, item_case, nitems, cctrl, base, state, ob.S); break;
        case STAGE_2: stage2d_o2_batch_kernel<A, STAGE_2><<<blocks, 128, 0, s>>>(cases, item_case, nitems, cctrl, base, state, ob.S); break;
        case STAGE_3: stage2d_o2_batch_kernel<A, STAGE_3><<<blocks, 128, 0, s>>>(cases, item_case, nitems, cctrl, base, state, ob.S); break;
        default: return cudaErrorInvalidValue;
        }
        break;
    default: return cudaErrorInvalidValue;
    }
    return cudaPeekAtLastError();
}

cudaError_t launch_batch_o2_exact(int op, int stage, const CaseDesc *cases, const int *item_case, int nitems,
                                  Ctrl *cctrl, const StageArgs &base, const double *state, const O2Batch &ob,
                                  double *W1, int blocks, cudaStream_t s);
cudaError_t launch_batch_o2_fast(int op, int stage, const CaseDesc *cases, const int *item_case, int nitems,
                                 Ctrl *cctrl, const StageArgs &base, const double *state, const O2Batch &ob,
                                 double *W1, int blocks, cudaStream_t s, bool w_zero);

// Entry points (arithmetic translation units).
cudaError_t launch_batch_exact(int stage, const CaseDesc *cases, const int *item_case, int nitems, Ctrl *cctrl,
                               const StageArgs &base, int blocks, cudaStream_t s);
cudaError_t launch_batch_fast(int stage, const CaseDesc *cases, const int *item_case, int nitems, Ctrl *cctrl,
                              const StageArgs &base, int blocks, cudaStream_t s, bool w_zero);
int batch_max_blocks_per_sm(int arith, bool w_zero, int order);
int batch_slope_blocks_per_sm(int arith, bool w_zero);

} // namespace mmf
