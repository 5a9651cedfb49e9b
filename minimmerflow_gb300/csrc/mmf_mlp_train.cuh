// mmf_mlp_train.cuh -- training kernels of the troubled-cell MLP: forward,
// backward and Adam, with BF16 tensor-core matmuls (mma.sync m16n8k16,
// FP32 accumulation).  One warp owns 16 samples of a mini-batch:
//   forward   z1 = X W1^T + b1, a1 = GELU(z1), z2 = a1 W2^T + b2,
//             a2 = GELU(z2), z3 = a2 . w3 + b3, p = sigmoid(z3)
//   loss      mean binary cross-entropy; dz3 = (p - y) / B
//   backward  dz2 = (dz3 w3) GELU'(z2), da1 = dz2 W2, dz1 = da1 GELU'(z1)
//   gradients dW1 = dz1^T X, dW2 = dz2^T a1, dw3 = a2^T dz3, biases by sums
// (the accumulator fragments of one matmul are reused as the A operand of
// the next; the weight-gradient matmuls take their transposed operands from
// shared memory).  Per-warp partial gradients are added into an FP32 buffer.
#pragma once

#include <cuda_bf16.h>

#include "mmf_mlp.cuh"

namespace mmf {

__device__ __forceinline__ void mma16816(float *c, const uint32_t *a, const uint32_t *b)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    __nv_bfloat162 v;
    v.x = lo;
    v.y = hi;
    return *reinterpret_cast<uint32_t *>(&v);
}

// A fragment (16 x 16 tile, row-major) from an element function A(r, c)
template <class F>
__device__ __forceinline__ void load_a(uint32_t *a, F A)
{
    const int lane = threadIdx.x & 31, gid = lane >> 2, t2 = (lane & 3) * 2;
    a[0] = pack2(A(gid, t2), A(gid, t2 + 1));
    a[1] = pack2(A(gid + 8, t2), A(gid + 8, t2 + 1));
    a[2] = pack2(A(gid, t2 + 8), A(gid, t2 + 9));
    a[3] = pack2(A(gid + 8, t2 + 8), A(gid + 8, t2 + 9));
}

// B fragment (16 x 8 tile, k x n) from an element function B(k, n)
template <class F>
__device__ __forceinline__ void load_b(uint32_t *b, F B)
{
    const int lane = threadIdx.x & 31, gid = lane >> 2, t2 = (lane & 3) * 2;
    b[0] = pack2(B(t2, gid), B(t2 + 1, gid));
    b[1] = pack2(B(t2 + 8, gid), B(t2 + 9, gid));
}

// A fragment of the next matmul from the accumulators of two 8-column tiles
__device__ __forceinline__ void acc_to_a(uint32_t *a, const float *c0, const float *c1)
{
    a[0] = pack_bf16(c0[0], c0[1]);
    a[1] = pack_bf16(c0[2], c0[3]);
    a[2] = pack_bf16(c1[0], c1[1]);
    a[3] = pack_bf16(c1[2], c1[3]);
}

constexpr int TRAIN_WARPS = 4;

template <int DIM>
struct TrainSmem {
    __nv_bfloat16 x[TRAIN_WARPS][16][mlp_kpad(DIM)];
    __nv_bfloat16 dz1[TRAIN_WARPS][16][MLP_H];
    __nv_bfloat16 dz2[TRAIN_WARPS][16][MLP_H];
    __nv_bfloat16 a1[TRAIN_WARPS][16][MLP_H];
};

// One pass over a mini-batch of B samples (B a multiple of 16; warps beyond
// the batch exit).  w1, w2: BF16 [64][KPAD], [64][64]; w2t = W2^T.  grad has
// the layout of the FP32 parameter vector; loss accumulates the summed BCE.
template <int DIM>
__global__ void __launch_bounds__(TRAIN_WARPS * 32) mlp_train_kernel(const __nv_bfloat16 *X, const unsigned char *y,
                                                                     int B, const __nv_bfloat16 *w1,
                                                                     const __nv_bfloat16 *w2,
                                                                     const __nv_bfloat16 *w2t, const float *params,
                                                                     float *grad, float *loss)
{
    constexpr int KP = mlp_kpad(DIM);
    __shared__ TrainSmem<DIM> sm;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, gid = lane >> 2, t2 = (lane & 3) * 2;
    const int row0 = (blockIdx.x * TRAIN_WARPS + warp) * 16;
    if (row0 >= B) return;
    // stage the warp's 16 rows of X
    for (int i = lane; i < 16 * KP; i += 32) sm.x[warp][i / KP][i % KP] = X[(long long)(row0 + i / KP) * KP + i % KP];
    __syncwarp();
    const float *b1 = params + mlp_off_b1(DIM), *b2 = params + mlp_off_b2(DIM), *w3 = params + mlp_off_w3(DIM);
    const float b3 = params[mlp_off_b3(DIM)];
    // ---- layer 1: z1 [16 x 64]
    float z1[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) z1[j][0] = z1[j][1] = z1[j][2] = z1[j][3] = 0.0f;
    for (int ks = 0; ks < KP / 16; ++ks) {
        uint32_t a[4];
        load_a(a, [&](int r, int c) { return sm.x[warp][r][ks * 16 + c]; });
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            uint32_t bb[2];
            load_b(bb, [&](int k, int n) { return w1[(8 * j + n) * KP + ks * 16 + k]; });
            mma16816(z1[j], a, bb);
        }
    }
    float a1[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            z1[j][e] += b1[8 * j + t2 + (e & 1)];
            a1[j][e] = gelu(z1[j][e]);
        }
    // ---- layer 2
    float z2[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) z2[j][0] = z2[j][1] = z2[j][2] = z2[j][3] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        uint32_t a[4];
        acc_to_a(a, a1[2 * ks], a1[2 * ks + 1]);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            uint32_t bb[2];
            load_b(bb, [&](int k, int n) { return w2[(8 * j + n) * MLP_H + ks * 16 + k]; });
            mma16816(z2[j], a, bb);
        }
    }
    // ---- output: per row, z3 = a2 . w3 + b3 (rows gid and gid + 8)
    float a2[8][4];
    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            z2[j][e] += b2[8 * j + t2 + (e & 1)];
            a2[j][e] = gelu(z2[j][e]);
            const float contrib = a2[j][e] * w3[8 * j + t2 + (e & 1)];
            if (e < 2) s0 += contrib; else s1 += contrib;
        }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    const float p0 = sigmoidf(s0 + b3), p1 = sigmoidf(s1 + b3);
    const float y0 = y[row0 + gid] ? 1.0f : 0.0f, y1 = y[row0 + gid + 8] ? 1.0f : 0.0f;
    const float d0 = (p0 - y0) / (float)B, d1 = (p1 - y1) / (float)B;   // dL/dz3
    if ((lane & 3) == 0) {
        const float l0 = -(y0 * logf(fmaxf(p0, 1e-12f)) + (1.0f - y0) * logf(fmaxf(1.0f - p0, 1e-12f)));
        const float l1 = -(y1 * logf(fmaxf(p1, 1e-12f)) + (1.0f - y1) * logf(fmaxf(1.0f - p1, 1e-12f)));
        atomicAdd(loss, l0 + l1);
        atomicAdd(grad + mlp_off_b3(DIM), d0 + d1);
    }
    // dw3 = a2^T dz3 ; dz2 = dz3 w3 GELU'(z2)
    float dz2[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int col = 8 * j + t2 + (e & 1);
            const float d = (e < 2) ? d0 : d1;
            dz2[j][e] = d * w3[col] * gelu_grad(z2[j][e]);
        }
    // per-column partial sums over the warp's rows for dw3, db2
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int col = 8 * j + t2 + e;
            float gw3 = a2[j][e] * d0 + a2[j][e + 2] * d1;
            float gb2 = dz2[j][e] + dz2[j][e + 2];
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) {
                gw3 += __shfl_xor_sync(0xffffffffu, gw3, o);
                gb2 += __shfl_xor_sync(0xffffffffu, gb2, o);
            }
            if (gid == 0) {
                atomicAdd(grad + mlp_off_w3(DIM) + col, gw3);
                atomicAdd(grad + mlp_off_b2(DIM) + col, gb2);
            }
        }
    // da1 = dz2 W2 (B(k = i, n = j) = W2[i][j] = W2^T[j][i]); dz1 = da1 GELU'(z1)
    float dz1[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) dz1[j][0] = dz1[j][1] = dz1[j][2] = dz1[j][3] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        uint32_t a[4];
        acc_to_a(a, dz2[2 * ks], dz2[2 * ks + 1]);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            uint32_t bb[2];
            load_b(bb, [&](int k, int n) { return w2t[(8 * j + n) * MLP_H + ks * 16 + k]; });
            mma16816(dz1[j], a, bb);
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) dz1[j][e] *= gelu_grad(z1[j][e]);
    // db1
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            float gb1 = dz1[j][e] + dz1[j][e + 2];
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) gb1 += __shfl_xor_sync(0xffffffffu, gb1, o);
            if (gid == 0) atomicAdd(grad + mlp_off_b1(DIM) + 8 * j + t2 + e, gb1);
        }
    // stage dz1, dz2, a1 (BF16) for the weight-gradient matmuls
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int r = gid + ((e >> 1) << 3), c = 8 * j + t2 + (e & 1);
            sm.dz1[warp][r][c] = __float2bfloat16(dz1[j][e]);
            sm.dz2[warp][r][c] = __float2bfloat16(dz2[j][e]);
            sm.a1[warp][r][c] = __float2bfloat16(a1[j][e]);
        }
    __syncwarp();
    // dW1 [64 x KP] = dz1^T X : A(i, b) = dz1[b][i], B(b, k) = X[b][k]; K = the warp's 16 rows
    for (int mi = 0; mi < 4; ++mi) {
        uint32_t a[4];
        load_a(a, [&](int r, int c) { return sm.dz1[warp][c][16 * mi + r]; });
        for (int nk = 0; nk < KP / 8; ++nk) {
            uint32_t bb[2];
            load_b(bb, [&](int k, int n) { return sm.x[warp][k][8 * nk + n]; });
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma16816(c, a, bb);
            float *g = grad + (long long)(16 * mi + gid) * KP + 8 * nk + t2;
            atomicAdd(g, c[0]);
            atomicAdd(g + 1, c[1]);
            atomicAdd(g + 8 * KP, c[2]);
            atomicAdd(g + 8 * KP + 1, c[3]);
        }
    }
    // dW2 [64 x 64] = dz2^T a1
    for (int mi = 0; mi < 4; ++mi) {
        uint32_t a[4];
        load_a(a, [&](int r, int c) { return sm.dz2[warp][c][16 * mi + r]; });
        for (int nk = 0; nk < 8; ++nk) {
            uint32_t bb[2];
            load_b(bb, [&](int k, int n) { return sm.a1[warp][k][8 * nk + n]; });
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            mma16816(c, a, bb);
            float *g = grad + mlp_off_w2(DIM) + (long long)(16 * mi + gid) * MLP_H + 8 * nk + t2;
            atomicAdd(g, c[0]);
            atomicAdd(g + 1, c[1]);
            atomicAdd(g + 8 * MLP_H, c[2]);
            atomicAdd(g + 8 * MLP_H + 1, c[3]);
        }
    }
}

// Adam on the FP32 parameters (padding columns of W1 stay zero), then the BF16
// copies: row-major W1, W2, the transpose of W2, and the tcgen05 operand layouts.
template <int DIM>
__global__ void mlp_adam_kernel(float *params, const float *grad, float *m, float *v, float lr, float beta1,
                                float beta2, float eps, float bc1, float bc2)
{
    const long long n = mlp_nparams(DIM);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (i < mlp_off_b1(DIM) && (i % mlp_kpad(DIM)) >= mlp_kin(DIM)) continue;
        const float g = grad[i];
        const float mi = beta1 * m[i] + (1.0f - beta1) * g;
        const float vi = beta2 * v[i] + (1.0f - beta2) * g * g;
        m[i] = mi;
        v[i] = vi;
        params[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

template <int DIM>
__global__ void mlp_pack_kernel(const float *params, __nv_bfloat16 *w1, __nv_bfloat16 *w2, __nv_bfloat16 *w2t,
                                __nv_bfloat16 *w1c, __nv_bfloat16 *w2c)
{
    constexpr int KP = mlp_kpad(DIM);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    for (int i = tid; i < MLP_H * KP; i += stride) {
        const int r = i / KP, k = i % KP;
        const __nv_bfloat16 v = __float2bfloat16(params[i]);
        w1[i] = v;
        w1c[core_offset(r, k, MLP_H)] = v;
    }
    for (int i = tid; i < MLP_H * MLP_H; i += stride) {
        const int r = i / MLP_H, k = i % MLP_H;
        const __nv_bfloat16 v = __float2bfloat16(params[mlp_off_w2(DIM) + i]);
        w2[i] = v;
        w2t[k * MLP_H + r] = v;
        w2c[core_offset(r, k, MLP_H)] = v;
    }
}

// Stencil features of every cell of a grid, BF16 [n][KPAD] (training data).
template <int DIM>
__global__ void mlp_features_kernel(GridParams gp, const double *U, __nv_bfloat16 *X)
{
    constexpr int KP = mlp_kpad(DIM);
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < gp.plane;
         g += (long long)gridDim.x * blockDim.x)
        cell_features<DIM>(U, gp, g, [&](int k, float v) { X[g * KP + k] = __float2bfloat16(v); });
}

} // namespace mmf
