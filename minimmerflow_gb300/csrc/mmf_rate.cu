// mmf_rate.cu -- measured FP64 instruction rate of the current GPU, the
// roofline denominator of the stage kernels (they are bound by FP64 issue,
// not by HBM).  Two streams of independent FP64 instructions per thread,
// eight accumulators, every SM filled (2048 threads each):
//   mode 0  DFMA whose multiplier and addend stay in the same registers
//           (the best case of the FP64 pipe);
//   mode 1  DADD, DMUL and DFMA in turn, each reading accumulators that
//           the previous instructions wrote (operands change from one
//           instruction to the next, as in the stage kernels).
// Built with -fmad=false so that every written operation is one instruction.
#include <cuda_runtime.h>

#include "../../include/mmf_gb300.h"

namespace mmf {
int set_last_error(int code, const char *msg);   // mmf_capi.cu
}

namespace {

constexpr int kAcc = 8;

template <int MODE>
__global__ void __launch_bounds__(256) fp64_rate_kernel(double seed, int iters, double *sink)
{
    double a[kAcc];
#pragma unroll
    for (int j = 0; j < kAcc; ++j) a[j] = seed + 1e-3 * (double)(threadIdx.x + j);
    const double m = 1.0 - 1e-12 * seed, c = 1e-7 * seed;
    for (int i = 0; i < iters; ++i) {
        if (MODE == 0) {
#pragma unroll
            for (int j = 0; j < kAcc; ++j) a[j] = fma(a[j], m, c);
        } else {
            a[0] = a[0] + a[1];
            a[1] = a[1] * a[2];
            a[2] = fma(a[2], a[3], a[4]);
            a[3] = a[3] + a[4];
            a[4] = a[4] * a[5];
            a[5] = fma(a[5], a[6], a[7]);
            a[6] = a[6] + a[7];
            a[7] = a[7] * a[0];
        }
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < kAcc; ++j) s += a[j];
    if (s == 1.2345e300) *sink = s;   // keeps the loop; never true for these inputs
}

template <int MODE>
cudaError_t time_mode(int blocks, int iters, double *sink, cudaEvent_t e0, cudaEvent_t e1, double *best)
{
    *best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {   // the first launch is a warm-up
        cudaEventRecord(e0, 0);
        fp64_rate_kernel<MODE><<<blocks, 256>>>(1.0 + rep, iters, sink);
        cudaEventRecord(e1, 0);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) return e;
        float ms = 0.f;
        if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) return e;
        const double ops = (double)blocks * 256.0 * iters * kAcc;
        if (rep > 0 && ms > 0.f) *best = fmax(*best, ops / (1e-3 * ms));
    }
    return cudaGetLastError();
}

} // namespace

extern "C" int mmf_fp64_rate(int device, double *out)
{
    if (!out) return mmf::set_last_error(MMF_ERR_ARG, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
        return mmf::set_last_error(MMF_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev) return mmf::set_last_error(MMF_ERR_ARG, "device index out of range");
    cudaError_t e = cudaSetDevice(device);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    double *sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int blocks = sms * 8, iters = 4096;   // 8 blocks of 256 threads fill an SM
    if (e == cudaSuccess) e = time_mode<0>(blocks, iters, sink, e0, e1, &out[0]);
    if (e == cudaSuccess) e = time_mode<1>(blocks, iters, sink, e0, e1, &out[1]);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) return mmf::set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}
