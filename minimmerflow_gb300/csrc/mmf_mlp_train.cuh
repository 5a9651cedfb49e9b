// mmf_mlp_train.cuh -- training kernels of the troubled-cell MLP: forward,
// backward and Adam.  Every matmul of a training step runs on the tcgen05
// tensor cores (BF16 operands in shared memory, FP32 accumulators in tensor
// memory), one CTA per tile of 128 samples:
//   forward   z1 = X W1^T + b1, a1 = GELU(z1), z2 = a1 W2^T + b2,
//             a2 = GELU(z2), z3 = a2 . w3 + b3, p = sigmoid(z3)
//   loss      mean binary cross-entropy; dz3 = (p - y) / B
//   backward  dz2 = (dz3 w3) GELU'(z2), da1 = dz2 W2, dz1 = da1 GELU'(z1)
//   gradients dW1 = dz1^T X, dW2 = dz2^T a1, dw3 = a2^T dz3, biases by sums
// Tiles add their gradients into an FP32 buffer; Adam updates the FP32
// parameters and repacks the BF16 operand copies.
#pragma once

#include <cuda_bf16.h>

#include "mmf_mlp.cuh"

namespace mmf {

// ---- tcgen05 training step ---------------------------------------------------
// One CTA of 128 threads per tile of 128 samples (thread = sample), every
// matmul a tcgen05.mma (M = 128, BF16 operands in shared memory, FP32
// accumulators in tensor memory), the same rounding points as the oracle:
//   Z1 = X W1^T        A = X [128 x KP],      B = W1 [64 x KP]      TMEM [0, 64)
//   Z2 = A1 W2^T       A = A1 [128 x 64],     B = W2 [64 x 64]      TMEM [64, 128)
//   dA1 = dZ2 W2       A = dZ2 [128 x 64],    B = W2^T [64 x 64]    TMEM [128, 192)
//   dW1 = dZ1^T X      A = dZ1^T [128 x 128] (rows 64..127 zero), B = X^T [KP x 128]   TMEM [192, 192 + KP)
//   dW2 = dZ2^T A1     A = dZ2^T [128 x 128] (rows 64..127 zero), B = A1^T [64 x 128]  TMEM [336, 400)
// Every operand is K-major in the core-matrix layout of the inference kernel;
// the transposed ones are written element by element by the threads.  The
// bias and w3 gradients are column sums over the tile (FP32, warp shuffles),
// the weight gradients leave tensor memory by rows (threads 0..63) and are
// added into the FP32 gradient buffer.
struct MlpTrainDev {
    const __nv_bfloat16 *w1c, *w2c, *w2tc;   // W1, W2, W2^T in the operand layout
    const float *params;
};

template <int DIM>
struct TrainTcLayout {
    static constexpr int KP = mlp_kpad(DIM);
    static constexpr int cmax(int a, int b) { return a > b ? a : b; }
    static constexpr int R0 = cmax(128 * KP * 2, 128 * 128 * 2);            // X, then dZ1^T
    static constexpr int R1 = cmax(64 * KP * 2 + 128 * 64 * 2, 128 * 128 * 2);   // W1 + A1, then dZ2^T
    static constexpr int oX = 0, oDZ1T = 0;
    static constexpr int oW1 = R0, oA1 = R0 + 64 * KP * 2, oDZ2T = R0;
    static constexpr int oW2 = R0 + R1;
    static constexpr int oDZ2 = oW2 + 64 * 64 * 2;
    static constexpr int oW2T = oDZ2 + 128 * 64 * 2;
    static constexpr int oXT = oW2T + 64 * 64 * 2;
    static constexpr int oA1T = oXT + KP * 128 * 2;
    static constexpr int bytes = oA1T + 64 * 128 * 2;
};

template <int DIM>
constexpr int mlp_train_tc_smem() { return TrainTcLayout<DIM>::bytes; }

// Column sums over the 32 rows of a warp; lane 0 adds them into dst[0..63].
__device__ __forceinline__ void warp_colsum_add(const float *v, float *dst)
{
#pragma unroll
    for (int j = 0; j < MLP_H; ++j) {
        float x = v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(dst + j, x);
    }
}

// MMA over K (16 per instruction) of a K-major A (arows rows) and B (brows rows)
__device__ __forceinline__ void umma_k(uint32_t tmem_d, uint32_t sa, int arows, uint32_t sb, int brows, int k,
                                       uint32_t idesc)
{
    for (int kk = 0; kk < k / 16; ++kk) {
        const uint64_t da = umma_desc(sa + kk * 2 * (arows / 8) * 128, (arows / 8) * 128, 128);
        const uint64_t db = umma_desc(sb + kk * 2 * (brows / 8) * 128, (brows / 8) * 128, 128);
        umma_bf16(tmem_d, da, db, idesc, kk > 0);
    }
}

template <int DIM>
__global__ void __launch_bounds__(128, 1) mlp_train_tc_kernel(const __nv_bfloat16 *X, const unsigned char *y, int B,
                                                              MlpTrainDev w, float *grad, float *loss, int *err,
                                                              WaitLimits lim)
{
    using L = TrainTcLayout<DIM>;
    constexpr int KP = mlp_kpad(DIM);
    extern __shared__ __align__(1024) unsigned char dyn[];
    __nv_bfloat16 *sX = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oX);
    __nv_bfloat16 *sDZ1T = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oDZ1T);
    __nv_bfloat16 *sW1 = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oW1);
    __nv_bfloat16 *sA1 = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oA1);
    __nv_bfloat16 *sDZ2T = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oDZ2T);
    __nv_bfloat16 *sW2 = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oW2);
    __nv_bfloat16 *sDZ2 = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oDZ2);
    __nv_bfloat16 *sW2T = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oW2T);
    __nv_bfloat16 *sXT = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oXT);
    __nv_bfloat16 *sA1T = reinterpret_cast<__nv_bfloat16 *>(dyn + L::oA1T);
    __shared__ __align__(8) uint64_t mbar_mma;
    __shared__ __align__(8) uint64_t mbar_load;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int s = blockIdx.x * 128 + tid;   // this thread's sample
    const bool live = s < B;

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar_mma)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar_load)));
        asm volatile("fence.mbarrier_init.release.cluster;");
        s_fail = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_addr(&tmem_base)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    const uint32_t w1_bytes = MLP_H * KP * 2, w2_bytes = MLP_H * MLP_H * 2;
    if (tid == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&mbar_load)),
                     "r"(w1_bytes + 2 * w2_bytes));
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_addr(sW1)), "l"(w.w1c), "r"(w1_bytes), "r"(smem_addr(&mbar_load)));
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_addr(sW2)), "l"(w.w2c), "r"(w2_bytes), "r"(smem_addr(&mbar_load)));
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_addr(sW2T)), "l"(w.w2tc), "r"(w2_bytes), "r"(smem_addr(&mbar_load)));
    }
    // this sample's features: the operand row (A of Z1) and the transposed copy (B of dW1)
    {
        RowPacker pk{sX, tid, 128, {0u, 0u, 0u, 0u}};
        const __nv_bfloat16 *xr = X + (long long)s * KP;
#pragma unroll 4
        for (int k = 0; k < KP; ++k) {
            const __nv_bfloat16 v = live ? xr[k] : __float2bfloat16(0.0f);
            pk.put(k, __bfloat162float(v));
            sXT[core_offset(k, tid, KP)] = v;   // row = feature (KP rows), K = sample
        }
    }
    const float *b1 = w.params + mlp_off_b1(DIM), *b2 = w.params + mlp_off_b2(DIM), *w3 = w.params + mlp_off_w3(DIM);
    const float b3 = w.params[mlp_off_b3(DIM)];
    const bool loaded = __syncthreads_and(mbar_wait(&mbar_load, 0, lim.wait));
    if (!loaded && tid == 0) { atomicExch(err, 2); s_fail = 1; }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_base;
    const uint32_t lane_addr = (uint32_t)(warp * 32) << 16;
    const uint32_t id64 = umma_idesc(128, 64), idKP = umma_idesc(128, KP);
    uint32_t phase = 0;
    // issue (one thread), commit, bounded wait, and the fences around the barrier
    auto mma_round = [&](auto issue) -> bool {
        if (s_fail) return false;
        if (tid == 0) {
            issue();
            umma_commit(&mbar_mma);
        }
        const bool ok = mbar_wait(&mbar_mma, phase, lim.wait);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;");
        if (!__syncthreads_and(ok)) {
            if (tid == 0) { atomicExch(err, 1); s_fail = 1; }
            __syncthreads();
            return false;
        }
        return true;
    };
    auto publish = [&]() {   // shared-memory operand writes visible to the tensor core
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
    };

    bool ok = mma_round([&] { umma_k(tmem, smem_addr(sX), 128, smem_addr(sW1), 64, KP, id64); });
    float z[MLP_H], a[MLP_H];
    if (ok) {
        // a1 = GELU(z1 + b1): operand row (A of Z2) and transposed copy (B of dW2)
#pragma unroll
        for (int c0 = 0; c0 < MLP_H; c0 += 16) tmem_ld16(tmem + lane_addr + (uint32_t)c0, z + c0);
        RowPacker pa{sA1, tid, 128, {0u, 0u, 0u, 0u}};
#pragma unroll
        for (int j = 0; j < MLP_H; ++j) {
            const float v = gelu(z[j] + b1[j]);
            const __nv_bfloat16 h = __float2bfloat16(v);
            pa.put(j, v);
            sA1T[core_offset(j, tid, 64)] = h;
        }
        publish();
        ok = mma_round([&] { umma_k(tmem + 64, smem_addr(sA1), 128, smem_addr(sW2), 64, MLP_H, id64); });
    }
    if (ok) {
        // output, loss, dz3, dz2 = dz3 w3 GELU'(z2); w3 and b2 gradients by column sums
#pragma unroll
        for (int c0 = 0; c0 < MLP_H; c0 += 16) tmem_ld16(tmem + lane_addr + (uint32_t)(64 + c0), z + c0);
        float z3 = b3;
#pragma unroll
        for (int j = 0; j < MLP_H; ++j) {
            z[j] += b2[j];
            a[j] = gelu(z[j]);
            z3 = fmaf(a[j], w3[j], z3);
        }
        const float p = sigmoidf(z3);
        const float yy = (live && y[s]) ? 1.0f : 0.0f;
        const float d3 = live ? (p - yy) / (float)B : 0.0f;
        float l = live ? -(yy * logf(fmaxf(p, 1e-12f)) + (1.0f - yy) * logf(fmaxf(1.0f - p, 1e-12f))) : 0.0f;
        float dsum = d3;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            l += __shfl_xor_sync(0xffffffffu, l, o);
            dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        }
        if ((tid & 31) == 0) {
            atomicAdd(loss, l);
            atomicAdd(grad + mlp_off_b3(DIM), dsum);
        }
#pragma unroll
        for (int j = 0; j < MLP_H; ++j) a[j] *= d3;                  // dw3 terms
        warp_colsum_add(a, grad + mlp_off_w3(DIM));
        RowPacker pd{sDZ2, tid, 128, {0u, 0u, 0u, 0u}};
#pragma unroll
        for (int j = 0; j < MLP_H; ++j) {
            z[j] = d3 * w3[j] * gelu_grad(z[j]);                     // dz2
            const __nv_bfloat16 h = __float2bfloat16(z[j]);
            pd.put(j, z[j]);
            sDZ2T[core_offset(j, tid, 128)] = h;
            sDZ2T[core_offset(j + 64, tid, 128)] = __float2bfloat16(0.0f);
        }
        warp_colsum_add(z, grad + mlp_off_b2(DIM));
        publish();
        ok = mma_round([&] { umma_k(tmem + 128, smem_addr(sDZ2), 128, smem_addr(sW2T), 64, MLP_H, id64); });
    }
    if (ok) {
        // dz1 = dA1 GELU'(z1): transposed copy (A of dW1); b1 gradient by column sums
        float da[MLP_H];
#pragma unroll
        for (int c0 = 0; c0 < MLP_H; c0 += 16) {
            tmem_ld16(tmem + lane_addr + (uint32_t)(128 + c0), da + c0);
            tmem_ld16(tmem + lane_addr + (uint32_t)c0, z + c0);
        }
#pragma unroll
        for (int j = 0; j < MLP_H; ++j) {
            z[j] = da[j] * gelu_grad(z[j] + b1[j]);
            sDZ1T[core_offset(j, tid, 128)] = __float2bfloat16(z[j]);
            sDZ1T[core_offset(j + 64, tid, 128)] = __float2bfloat16(0.0f);
        }
        warp_colsum_add(z, grad + mlp_off_b1(DIM));
        publish();
        ok = mma_round([&] {
            umma_k(tmem + 192, smem_addr(sDZ1T), 128, smem_addr(sXT), KP, 128, idKP);
            umma_k(tmem + 336, smem_addr(sDZ2T), 128, smem_addr(sA1T), 64, 128, id64);
        });
    }
    if (ok && warp < 2) {
        // weight gradients: TMEM lane i = hidden unit i (threads 0..63)
        float *g1 = grad + (long long)tid * KP;
#pragma unroll 1
        for (int c0 = 0; c0 < KP; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + lane_addr + (uint32_t)(192 + c0), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) atomicAdd(g1 + c0 + j, v[j]);
        }
        float *g2 = grad + mlp_off_w2(DIM) + (long long)tid * MLP_H;
#pragma unroll 1
        for (int c0 = 0; c0 < MLP_H; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + lane_addr + (uint32_t)(336 + c0), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) atomicAdd(g2 + c0 + j, v[j]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
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
                                __nv_bfloat16 *w1c, __nv_bfloat16 *w2c, __nv_bfloat16 *w2tc)
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
        w2tc[core_offset(k, r, MLP_H)] = v;
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
