// mmf_mlp.cuh -- learned troubled-cell indicator: a 3-layer MLP over the
// normalised primitive variables of a cell's (3^dim)-cell stencil that
// predicts where the order-2 limiter would change a slope, so that cells
// predicted smooth take central slopes and skip the limiter.
//
//   features  x (dim 2: 9 x 5 = 45, padded to 48; dim 3: 27 x 5 = 135, padded
//             to 144): for each primitive q in (rho, u, v, w, p), FP32,
//             (q_j - q_c) / (max_j |q_j - q_c| + eps_q) over the stencil (c the
//             centre cell; eps = 1e-4 |q_c| for rho and p, 1e-4 a_c for the
//             velocities, a_c the centre sound speed); borders wrap (periodic)
//             or clamp (zero gradient)
//   network   h1 = GELU(W1 x + b1) (64), h2 = GELU(W2 h1 + b2) (64),
//             y = sigmoid(w3 . h2 + b3); BF16 operands, FP32 accumulation;
//             GELU in its tanh form (gelu below)
//
// Inference is two kernels.  mlp_prims_kernel converts every cell's state to
// FP32 primitives once.  mlp_infer_kernel is one fused, persistent tcgen05
// kernel per 128-cell tile, three CTAs per SM: the 128 threads of a CTA
// compute one cell's features each from the primitive planes and store them
// as BF16 in the shared-memory operand layout; one thread issues tcgen05.mma
// into a TMEM accumulator (layer 1: 9 MMAs of K 16 for 3D), the tile's h1
// comes back with tcgen05.ld and goes through GELU into the layer-2 operand,
// which reuses the layer-1 operand's shared memory once that MMA has
// completed; layer 2 accumulates into a second TMEM region, and each thread
// finishes its own row (GELU, dot with w3, sigmoid).  Weights are staged once
// per CTA with bulk asynchronous copies (cp.async.bulk).
//
// Shared operand layout (K-major, no swizzle): 8-row x 16-byte core matrices;
// core matrix (row block rb, k block kb) at byte (kb * ROWS/8 + rb) * 128, row
// r of it at r * 16.  Descriptor: leading byte offset = ROWS/8 * 128 (next
// core matrix along K), stride byte offset = 128 (next 8-row block).
//
// Training runs on the GPU as well (mlp_train.cuh): forward, backward and Adam
// kernels with mma.sync BF16 matmuls accumulated in FP32.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

#include "mmf_batch.cuh"

namespace mmf {

constexpr int MLP_H = 64;            // hidden width
constexpr int MLP_TILE = 128;        // cells per tcgen05 tile (M)
// inference CTAs per SM (shared memory, registers, 128 of the 512 TMEM
// columns each): four in 2D (48 features), three in 3D (144)
__host__ __device__ constexpr int mlp_ctas_per_sm(int dim) { return dim == 2 ? 4 : 3; }

__host__ __device__ constexpr int mlp_kin(int dim) { return dim == 3 ? 135 : 45; }
__host__ __device__ constexpr int mlp_kpad(int dim) { return dim == 3 ? 144 : 48; }
// elements of the inference kernel's first operand region: X (128 x KPAD),
// later H (128 x 64)
__host__ __device__ constexpr int mlp_operand_elems(int dim) { return 128 * (mlp_kpad(dim) > 64 ? mlp_kpad(dim) : 64); }

// Flat FP32 parameter vector: W1 [64][KPAD], b1 [64], W2 [64][64], b2 [64], w3 [64], b3 [1]
__host__ __device__ constexpr long long mlp_off_b1(int dim) { return (long long)MLP_H * mlp_kpad(dim); }
__host__ __device__ constexpr long long mlp_off_w2(int dim) { return mlp_off_b1(dim) + MLP_H; }
__host__ __device__ constexpr long long mlp_off_b2(int dim) { return mlp_off_w2(dim) + MLP_H * MLP_H; }
__host__ __device__ constexpr long long mlp_off_w3(int dim) { return mlp_off_b2(dim) + MLP_H; }
__host__ __device__ constexpr long long mlp_off_b3(int dim) { return mlp_off_w3(dim) + MLP_H; }
__host__ __device__ constexpr long long mlp_nparams(int dim) { return mlp_off_b3(dim) + 1; }

// element offset of (row, k) in the K-major no-swizzle operand layout
__host__ __device__ __forceinline__ int core_offset(int row, int k, int rows)
{
    return (((k >> 3) * (rows >> 3) + (row >> 3)) << 6) + ((row & 7) << 3) + (k & 7);
}

// Writes one row of a K-major BF16 operand (core-matrix layout) eight
// elements at a time: put(k, v) for k = 0, 1, 2, ... in order; every full
// group of eight (16 contiguous bytes of the row) goes out in one 16-byte
// shared-memory store.  With the k loops unrolled the packing stays in
// registers.
struct RowPacker {
    __nv_bfloat16 *base;
    int row, rows;
    uint32_t w[4];
    float pend = 0.0f;   // the even element of the pair being formed
    // Elements go in pairs through one two-way conversion (round to nearest
    // even, as the one-way conversion rounds).
    __device__ __forceinline__ void put(int k, float v)
    {
        if ((k & 1) == 0) {
            pend = v;
        } else {
            const __nv_bfloat162 h = __floats2bfloat162_rn(pend, v);   // .x = element k - 1
            w[(k & 7) >> 1] = *reinterpret_cast<const uint32_t *>(&h);
        }
        if ((k & 7) == 7)
            *reinterpret_cast<uint4 *>(base + core_offset(row, k - 7, rows)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
};

// GELU in its tanh form, 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))),
// written as x sigma(z) with z = 2 sqrt(2/pi) (x + 0.044715 x^3) and
// sigma(z) = 1 / (1 + 2^(-z log2 e)): the exponent -z log2 e as one
// polynomial in x with folded constants, then the hardware base-2
// exponential and reciprocal approximations (the network applies 128 per
// cell, so this is most of the inference's arithmetic).
constexpr float GELU_C = 1.5957691216057308f;   // 2 sqrt(2 / pi)
constexpr float GELU_E1 = -1.5957691216057308f * 1.4426950408889634f;   // -GELU_C log2 e
constexpr float GELU_E3 = GELU_E1 * 0.044715f;
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu(float x)
{
    const float t = x * fmaf(GELU_E3, x * x, GELU_E1);   // -z log2 e
    return x * rcp_approx(1.0f + ex2_approx(t));
}
__device__ __forceinline__ float gelu_grad(float x)
{
    const float x2 = x * x;
    const float z = GELU_C * fmaf(0.044715f * x, x2, x);
    const float s = __fdividef(1.0f, 1.0f + __expf(-z));
    return fmaf(x * s * (1.0f - s), GELU_C * fmaf(3.0f * 0.044715f, x2, 1.0f), s);
}
__device__ __forceinline__ float sigmoidf(float z) { return 1.0f / (1.0f + __expf(-z)); }

// Grid index of the stencil cell at (x, y, z): periodic borders wrap, the
// others clamp (zero gradient).
__device__ __forceinline__ long long stencil_index(const GridParams &gp, int x, int y, int z)
{
    const bool px = gp.bc_lo[0] == BC_PERIODIC, py = gp.bc_lo[1] == BC_PERIODIC, pz = gp.bc_lo[2] == BC_PERIODIC;
    const int nx = gp.n[0], ny = gp.n[1], nz = gp.n[2];
    x = x < 0 ? (px ? nx - 1 : 0) : (x >= nx ? (px ? 0 : nx - 1) : x);
    y = y < 0 ? (py ? ny - 1 : 0) : (y >= ny ? (py ? 0 : ny - 1) : y);
    z = z < 0 ? (pz ? nz - 1 : 0) : (z >= nz ? (pz ? 0 : nz - 1) : z);
    return (long long)x + (long long)nx * ((long long)y + (long long)ny * z);
}

// Primitive variables (rho, u, v, w, p) in FP32 of cell g of SoA FP64 planes
// n apart.  Every operation is an explicitly rounded intrinsic, so the bits do
// not depend on where the compiler inlines this (the indicator's primitive
// planes and the training features must agree).
__device__ __forceinline__ void prim_of(const double *U, long long n, long long g, float *q)
{
    const float rho = (float)__ldg(U + g);
    const float ri = __fdiv_rn(1.0f, rho);
    const float u = __fmul_rn((float)__ldg(U + n + g), ri), v = __fmul_rn((float)__ldg(U + 2 * n + g), ri),
                w = __fmul_rn((float)__ldg(U + 3 * n + g), ri);
    const float E = (float)__ldg(U + 4 * n + g);
    const float s2 = __fmaf_rn(w, w, __fmaf_rn(v, v, __fmul_rn(u, u)));
    q[0] = rho;
    q[1] = u;
    q[2] = v;
    q[3] = w;
    q[4] = __fmul_rn((float)(GAMMA - 1.0), __fsub_rn(E, __fmul_rn(__fmul_rn(0.5f, rho), s2)));
}

// Primitive variables of the stencil cell at (x, y, z), from the state.
__device__ __forceinline__ void prim_at(const double *U, const GridParams &gp, int x, int y, int z, float *q)
{
    prim_of(U, gp.plane, stencil_index(gp, x, y, z), q);
}

// ... and from the primitive planes of mlp_prims_kernel (the same values).
__device__ __forceinline__ void prim_q_at(const float *Q, const GridParams &gp, int x, int y, int z, float *q)
{
    const long long g = stencil_index(gp, x, y, z);
#pragma unroll
    for (int v = 0; v < 5; ++v) q[v] = __ldg(Q + v * gp.plane + g);
}

// The primitive variables of cells [0, n) of SoA FP64 planes n apart, as FP32
// SoA planes n apart: each cell converted once per indicator run, instead of
// once per stencil (or strip) that contains it.
__global__ void __launch_bounds__(256) mlp_prims_kernel(long long n, const double *__restrict__ U,
                                                        float *__restrict__ Q, IndicatorStep is)
{
    if (indicator_idle(is)) return;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        float q[5];
        prim_of(U, n, g, q);
#pragma unroll
        for (int v = 0; v < 5; ++v) Q[v * n + g] = q[v];
    }
}

template <int DIM, class Get, class Put>
__device__ __forceinline__ void stencil_features(Get get, Put put);

// The KPAD features of grid cell g (FP32), written through 'put(k, value)'.
// Stencil cell s is at (dx, dy, dz) = (s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1).
template <int DIM, class Put>
__device__ __forceinline__ void cell_features(const double *U, const GridParams &gp, long long g, Put put)
{
    constexpr int NS = DIM == 3 ? 27 : 9;
    int x, y, z;
    cell_coords(gp, g, x, y, z);
    if (DIM == 2) z = 0;
    float q[NS][5];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const int dx = s % 3 - 1, dy = (s / 3) % 3 - 1, dz = DIM == 3 ? s / 9 - 1 : 0;
        prim_at(U, gp, x + dx, y + dy, z + dz, q[s]);
    }
    stencil_features<DIM>([&](int s, int v) { return q[s][v]; }, put);
}

// The KPAD features of grid cell g from the primitive planes Q: the
// stencil's cell indices once, then one variable at a time (the loads hit L1
// and L2, where the neighbouring cells' stencils brought the same values).
template <int DIM, class Put>
__device__ __forceinline__ void cell_features_q(const float *Q, const GridParams &gp, long long g, Put put)
{
    constexpr int NS = DIM == 3 ? 27 : 9;
    int x, y, z;
    cell_coords(gp, g, x, y, z);
    if (DIM == 2) z = 0;
    // the neighbours' coordinates along each axis (wrapped or clamped as in
    // stencil_index), then the stencil's 3^DIM indices as row offsets + x
    const bool px = gp.bc_lo[0] == BC_PERIODIC, py = gp.bc_lo[1] == BC_PERIODIC, pz = gp.bc_lo[2] == BC_PERIODIC;
    const int nx = gp.n[0], ny = gp.n[1], nz = gp.n[2];
    int xs[3], ys[3], zs[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int xx = x + d - 1, yy = y + d - 1, zz = z + d - 1;
        xs[d] = xx < 0 ? (px ? nx - 1 : 0) : (xx >= nx ? (px ? 0 : nx - 1) : xx);
        ys[d] = yy < 0 ? (py ? ny - 1 : 0) : (yy >= ny ? (py ? 0 : ny - 1) : yy);
        zs[d] = DIM == 3 ? (zz < 0 ? (pz ? nz - 1 : 0) : (zz >= nz ? (pz ? 0 : nz - 1) : zz)) : 0;
    }
    long long row[NS / 3];
#pragma unroll
    for (int r = 0; r < NS / 3; ++r)
        row[r] = (long long)nx * ((long long)ys[r % 3] + (long long)ny * zs[DIM == 3 ? r / 3 : 1]);
    const float *Qv[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) Qv[v] = Q + v * gp.plane;
    stencil_features<DIM>([&](int s, int v) { return __ldg(Qv[v] + row[s / 3] + xs[s % 3]); }, put);
}

// Normalised stencil differences of the primitives get(s, v) (FP32), one
// variable at a time (the stencil's values of one variable are the only ones
// held at once).  Every operation is explicitly rounded: the features are the
// same bits wherever this is inlined (training data and inference).
template <int DIM, class Get, class Put>
__device__ __forceinline__ void stencil_features(Get get, Put put)
{
    constexpr int NS = DIM == 3 ? 27 : 9;
    constexpr int C = DIM == 3 ? 13 : 4;   // centre of the stencil
    const float a_c = sqrtf(fmaxf(__fdiv_rn(__fmul_rn((float)GAMMA, get(C, 4)), get(C, 0)), 0.0f));
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        float q[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) q[s] = get(s, v);
        const float c = q[C];
        float m = 0.0f;
#pragma unroll
        for (int s = 0; s < NS; ++s) m = fmaxf(m, fabsf(__fsub_rn(q[s], c)));
        const float eps = __fmul_rn(1e-4f, (v == 0 || v == 4) ? fabsf(c) : a_c);
        const float inv = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(m, eps), 1e-30f));
#pragma unroll
        for (int s = 0; s < NS; ++s) put(v * NS + s, __fmul_rn(__fsub_rn(q[s], c), inv));
    }
#pragma unroll
    for (int k = 5 * NS; k < mlp_kpad(DIM); ++k) put(k, 0.0f);
}

// ---- tcgen05 helpers ---------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory operand descriptor, K-major, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor: kind::f16, D f32, A and B bf16, both K-major, M x N
__host__ __device__ constexpr uint32_t umma_idesc(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, bool accumulate)
{
    const uint32_t acc = accumulate ? 1u : 0u;
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
                 "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar)));
}

// bounded wait on an mbarrier phase; false after the iteration limit
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, long long limit)
{
    uint32_t done = 0;
    for (long long it = 0; it < limit && !done; ++it) {
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done) : "r"(smem_addr(mbar)), "r"(parity));
    }
    return done != 0;
}

// 16 f32 accumulator columns of this thread's TMEM lane (row)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Cells of a packed batch of 2D grids: case c covers [offsets[c], offsets[c+1]).
struct BatchGeom {
    const CaseDesc *cases;
    const long long *offsets;
    int ncases;
};

__device__ __forceinline__ int case_of(const BatchGeom &bg, long long g)
{
    int lo = 0, hi = bg.ncases - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (bg.offsets[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

enum { MLP_SRC_GRID = 0, MLP_SRC_X = 1, MLP_SRC_BATCH = 2 };

struct MlpDev {
    const __nv_bfloat16 *w1c;   // W1 in the operand layout, 64 rows x KPAD
    const __nv_bfloat16 *w2c;   // W2 in the operand layout, 64 rows x 64
    const float *params;        // FP32 parameters (biases, w3, b3 are read from here)
};

// Iteration limits of the inference kernel's mbarrier waits.  'wait' bounds
// every wait on the weights' bulk copies and on the MMA completions.  'probe'
// > 0 makes each CTA first wait on a barrier that nothing completes, for that
// many iterations, before it issues any copy or MMA: the wait gives up with
// nothing in flight, so the kernel's give-up path (error flag, TMEM freed,
// early return) can be exercised on a GPU without leaving work behind.
struct WaitLimits {
    long long wait;
    long long probe;
};

// Fused features + MLP over the cells of a grid (persistent, one 128-cell tile
// per iteration).  prob (nullable) receives y, flags (nullable) y > threshold.
// Sets *err when a wait gave up: 1 an MMA completion, 2 the weights' copies,
// 3 the probe barrier (WaitLimits).
template <int DIM, int SRC>
__global__ void __launch_bounds__(128, mlp_ctas_per_sm(DIM)) mlp_infer_kernel(GridParams gp, const float *Q, const __nv_bfloat16 *X,
                                                           MlpDev w, float threshold, float *prob,
                                                           unsigned char *flags, int *err, BatchGeom bg,
                                                           WaitLimits lim, IndicatorStep is)
{
    if (indicator_idle(is)) return;   // uniform over the grid: before any barrier or allocation
    constexpr int KP = mlp_kpad(DIM);
    extern __shared__ __align__(1024) unsigned char dyn[];
    // the layer-1 operand X (128 x KP) and, once its MMA has completed, the
    // layer-2 operand H (128 x 64) share the first region
    __nv_bfloat16 *sX = reinterpret_cast<__nv_bfloat16 *>(dyn);
    __nv_bfloat16 *sH = sX;
    __nv_bfloat16 *sW1 = sX + mlp_operand_elems(DIM);                    // 64 x KP
    __nv_bfloat16 *sW2 = sW1 + MLP_H * KP;                               // 64 x 64
    __shared__ __align__(8) uint64_t mbar_mma;
    __shared__ __align__(8) uint64_t mbar_load;
    __shared__ __align__(8) uint64_t mbar_probe;
    __shared__ uint32_t tmem_base;
    __shared__ float s_b1[MLP_H], s_b2[MLP_H], s_w3[MLP_H];
    __shared__ int s_fail;
    __shared__ int s_case;
    const int tid = threadIdx.x;

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar_mma)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar_load)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar_probe)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        s_fail = 0;
    }
    if (tid < MLP_H) {
        s_b1[tid] = w.params[mlp_off_b1(DIM) + tid];
        s_b2[tid] = w.params[mlp_off_b2(DIM) + tid];
        s_w3[tid] = w.params[mlp_off_w3(DIM) + tid];
    }
    const float b3 = w.params[mlp_off_b3(DIM)];
    if (tid < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_addr(&tmem_base)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    if (lim.probe > 0) {
        // nothing arrives on mbar_probe and no copy or MMA has been issued yet
        const bool ok = __syncthreads_and(mbar_wait(&mbar_probe, 0, lim.probe));
        if (!ok && tid == 0) { atomicExch(err, 3); s_fail = 1; }
        __syncthreads();
    }
    // weights: two bulk asynchronous copies completing on mbar_load
    const uint32_t w1_bytes = MLP_H * KP * 2, w2_bytes = MLP_H * MLP_H * 2;
    if (tid == 0 && !s_fail) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&mbar_load)),
                     "r"(w1_bytes + w2_bytes));
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_addr(sW1)),
                     "l"(w.w1c), "r"(w1_bytes), "r"(smem_addr(&mbar_load)));
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_addr(sW2)),
                     "l"(w.w2c), "r"(w2_bytes), "r"(smem_addr(&mbar_load)));
    }
    const bool probe_failed = s_fail != 0;
    const bool loaded = probe_failed || __syncthreads_and(mbar_wait(&mbar_load, 0, lim.wait));
    if (!loaded && tid == 0) { atomicExch(err, 2); s_fail = 1; }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    const uint32_t tmem = tmem_base;
    const int warp = tid >> 5;
    const uint32_t lane_addr = (uint32_t)(warp * 32) << 16;
    const uint32_t idesc = umma_idesc(MLP_TILE, MLP_H);
    const long long ntiles = (gp.plane + MLP_TILE - 1) / MLP_TILE;
    uint32_t phase = 0;

    for (long long tile = blockIdx.x; tile < ntiles && !s_fail; tile += gridDim.x) {
        const long long g = tile * MLP_TILE + tid;
        RowPacker pk{sX, tid, MLP_TILE, {0u, 0u, 0u, 0u}};
        if (SRC == MLP_SRC_BATCH) {
            // the tile's first case, once per tile (a case has at least 32 x 32
            // cells, so a tile of 128 cells meets at most two)
            if (tid == 0) s_case = case_of(bg, tile * MLP_TILE < gp.plane ? tile * MLP_TILE : gp.plane - 1);
            __syncthreads();
        }
        // features of this thread's cell -> BF16 operand rows
        if (g < gp.plane && SRC == MLP_SRC_X) {
            for (int k = 0; k < KP; ++k) sX[core_offset(tid, k, MLP_TILE)] = X[g * KP + k];
        } else if (g < gp.plane && SRC == MLP_SRC_BATCH) {
            int c = s_case;
            while (c + 1 < bg.ncases && bg.offsets[c + 1] <= g) ++c;
            const long long off = bg.offsets[c];
            cell_features_q<DIM>(Q + off, bg.cases[c].gp, g - off,
                                 [&](int k, float v) { pk.put(k, v); });
        } else if (g < gp.plane) {
            cell_features_q<DIM>(Q, gp, g, [&](int k, float v) { pk.put(k, v); });
        } else {
#pragma unroll
            for (int k = 0; k < KP; ++k) pk.put(k, 0.0f);
        }
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        // layer 1: TMEM columns [0, 64)
        if (tid == 0) {
            for (int kk = 0; kk < KP / 16; ++kk) {
                const uint64_t da = umma_desc(smem_addr(sX) + kk * 2 * (MLP_TILE / 8) * 128, (MLP_TILE / 8) * 128, 128);
                const uint64_t db = umma_desc(smem_addr(sW1) + kk * 2 * (MLP_H / 8) * 128, (MLP_H / 8) * 128, 128);
                umma_bf16(tmem, da, db, idesc, kk > 0);
            }
            umma_commit(&mbar_mma);
        }
        bool ok = mbar_wait(&mbar_mma, phase, lim.wait);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (!__syncthreads_and(ok)) { if (tid == 0) { atomicExch(err, 1); s_fail = 1; } break; }
        // h1 = GELU(z1 + b1) -> BF16 operand of layer 2
        RowPacker ph{sH, tid, MLP_TILE, {0u, 0u, 0u, 0u}};
#pragma unroll
        for (int c0 = 0; c0 < MLP_H; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + lane_addr + (uint32_t)c0, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) ph.put(c0 + j, gelu(v[j] + s_b1[c0 + j]));
        }
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        // layer 2: TMEM columns [64, 128)
        if (tid == 0) {
            for (int kk = 0; kk < MLP_H / 16; ++kk) {
                const uint64_t da = umma_desc(smem_addr(sH) + kk * 2 * (MLP_TILE / 8) * 128, (MLP_TILE / 8) * 128, 128);
                const uint64_t db = umma_desc(smem_addr(sW2) + kk * 2 * (MLP_H / 8) * 128, (MLP_H / 8) * 128, 128);
                umma_bf16(tmem + MLP_H, da, db, idesc, kk > 0);
            }
            umma_commit(&mbar_mma);
        }
        ok = mbar_wait(&mbar_mma, phase, lim.wait);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (!__syncthreads_and(ok)) { if (tid == 0) { atomicExch(err, 1); s_fail = 1; } break; }
        float zz = b3;
#pragma unroll
        for (int c0 = 0; c0 < MLP_H; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + lane_addr + (uint32_t)(MLP_H + c0), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) zz = fmaf(gelu(v[j] + s_b2[c0 + j]), s_w3[c0 + j], zz);
        }
        if (g < gp.plane) {
            const float y = sigmoidf(zz);
            if (prob) prob[g] = y;
            if (flags) flags[g] = (y > threshold) ? 1 : 0;
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

template <int DIM>
constexpr int mlp_infer_smem()
{
    return (mlp_operand_elems(DIM) + MLP_H * mlp_kpad(DIM) + MLP_H * MLP_H) * 2;
}

// Dilation of the indicator's flags by one cell: flags[g] = 1 where a cell of
// g's 3^DIM neighbourhood (wrapped or clamped as in stencil_index) has raw = 1.
template <int DIM>
__global__ void __launch_bounds__(256) mlp_dilate_kernel(GridParams gp, const unsigned char *__restrict__ raw,
                                                         unsigned char *__restrict__ flags, IndicatorStep is)
{
    if (indicator_idle(is)) return;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < gp.plane;
         g += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        cell_coords(gp, g, x, y, z);
        if (DIM == 2) z = 0;
        unsigned m = 0;
#pragma unroll
        for (int dz = (DIM == 3 ? -1 : 0); dz <= (DIM == 3 ? 1 : 0); ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx) m |= raw[stencil_index(gp, x + dx, y + dy, z + dz)];
        flags[g] = m ? 1 : 0;
    }
}

// The same over a packed batch of 2D grids, one thread per cell; each block
// finds the case of its first cell once (a case has at least 32 x 32 cells,
// so a block of 256 cells meets at most two).
__global__ void __launch_bounds__(256) mlp_dilate_batch_kernel(BatchGeom bg, long long total,
                                                               const unsigned char *__restrict__ raw,
                                                               unsigned char *__restrict__ flags, IndicatorStep is)
{
    if (indicator_idle(is)) return;
    __shared__ int s_case;
    const long long g0 = blockIdx.x * 256LL;
    if (threadIdx.x == 0) s_case = case_of(bg, g0);
    __syncthreads();
    const long long g = g0 + threadIdx.x;
    if (g >= total) return;
    int c = s_case;
    while (c + 1 < bg.ncases && bg.offsets[c + 1] <= g) ++c;
    const long long off = bg.offsets[c];
    const GridParams &gp = bg.cases[c].gp;
    int x, y, z;
    cell_coords(gp, g - off, x, y, z);
    unsigned m = 0;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) m |= raw[off + stencil_index(gp, x + dx, y + dy, 0)];
    flags[g] = m ? 1 : 0;
}

} // namespace mmf
