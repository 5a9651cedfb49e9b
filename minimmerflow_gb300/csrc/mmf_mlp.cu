// mmf_mlp.cu -- C ABI of the troubled-cell MLP: parameters, GPU training
// (forward/backward/Adam), inference on stored features, and the launchers
// the solver context uses for the fused indicator.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/mmf_gb300.h"
#include "mmf_mlp.cuh"
#include "mmf_mlp_train.cuh"
#include "mmf_nvtx.h"

namespace mmf {
int set_last_error(int code, const char *msg);
}
using namespace mmf;

#define MLP_CUDA(call)                                                                                   \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return set_last_error(MMF_ERR_CUDA, (std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
    } while (0)

struct mmf_mlp {
    int dim = 3;
    int device = 0;
    cudaStream_t stream = nullptr;
    float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr, *loss = nullptr;
    __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w2t = nullptr, *w1c = nullptr, *w2c = nullptr, *w2tc = nullptr;
    int *err = nullptr;
    long long adam_t = 0;
    long long n = 0;
    WaitLimits lim{1ll << 22, 0};   // inference kernel: mbarrier wait limit, probe wait (0 = none)
};

namespace mmf {

static int mlp_pack(mmf_mlp *p)
{
    if (p->dim == 3) mlp_pack_kernel<3><<<64, 256, 0, p->stream>>>(p->params, p->w1, p->w2, p->w2t, p->w1c, p->w2c, p->w2tc);
    else mlp_pack_kernel<2><<<64, 256, 0, p->stream>>>(p->params, p->w1, p->w2, p->w2t, p->w1c, p->w2c, p->w2tc);
    MLP_CUDA(cudaPeekAtLastError());
    return MMF_OK;
}

template <int DIM, int SRC>
static cudaError_t launch_infer(mmf_mlp *p, const GridParams &gp, const float *Q, const __nv_bfloat16 *X, float thr,
                                float *prob, unsigned char *flags, cudaStream_t s, BatchGeom bg = BatchGeom{nullptr, nullptr, 0},
                                IndicatorStep is = IndicatorStep{1, nullptr})
{
    const int smem = mlp_infer_smem<DIM>();
    cudaError_t e = cudaFuncSetAttribute(mlp_infer_kernel<DIM, SRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long ntiles = (gp.plane + MLP_TILE - 1) / MLP_TILE;
    const long long slots = (long long)mlp_ctas_per_sm(DIM) * sms;
    const int blocks = (int)(ntiles < slots ? ntiles : slots);
    MlpDev w;
    w.w1c = p->w1c;
    w.w2c = p->w2c;
    w.params = p->params;
    mlp_infer_kernel<DIM, SRC><<<blocks, 128, smem, s>>>(gp, Q, X, w, thr, prob, flags, p->err, bg, p->lim, is);
    return cudaPeekAtLastError();
}

// The primitive planes Q (5 x n FP32) of SoA FP64 planes U n apart.
static cudaError_t launch_prims(long long n, const double *U, float *Q, cudaStream_t s, IndicatorStep is)
{
    const long long b = (n + 255) / 256;
    mlp_prims_kernel<<<(unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16), 256, 0, s>>>(n, U, Q, is);
    return cudaPeekAtLastError();
}

// Features + MLP over a grid state (used by the solver context): the
// primitive planes of U into Q (scratch of 5 x gp.plane floats), then the
// fused kernel.  With 'raw' (one byte per cell) the network's flags go there
// and 'flags' receives them dilated by one cell.  'is' makes the launches of
// the steps between two indicator runs do nothing.
cudaError_t mlp_indicator(mmf_mlp *p, const GridParams &gp, const double *U, float thr, float *prob,
                          unsigned char *flags, cudaStream_t s, float *Q, unsigned char *raw, IndicatorStep is)
{
    if (p->dim != gp.dim || !Q) return cudaErrorInvalidValue;
    cudaError_t e = launch_prims(gp.plane, U, Q, s, is);
    if (e != cudaSuccess) return e;
    unsigned char *out = raw ? raw : flags;
    e = p->dim == 3 ? launch_infer<3, MLP_SRC_GRID>(p, gp, Q, nullptr, thr, prob, out, s, BatchGeom{nullptr, nullptr, 0}, is)
                    : launch_infer<2, MLP_SRC_GRID>(p, gp, Q, nullptr, thr, prob, out, s, BatchGeom{nullptr, nullptr, 0}, is);
    if (e != cudaSuccess || !raw || !flags) return e;
    const long long b = (gp.plane + 255) / 256;
    const unsigned blocks = (unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
    if (p->dim == 3) mlp_dilate_kernel<3><<<blocks, 256, 0, s>>>(gp, raw, flags, is);
    else mlp_dilate_kernel<2><<<blocks, 256, 0, s>>>(gp, raw, flags, is);
    return cudaPeekAtLastError();
}

// Indicator over a packed batch of 2D grids (total cells; Q: 5 x total floats;
// raw and is as for mlp_indicator).
cudaError_t mlp_indicator_batch(mmf_mlp *p, const CaseDesc *cases, const long long *offsets, int ncases,
                                long long total, const double *U, float thr, unsigned char *flags, cudaStream_t s,
                                float *Q, unsigned char *raw, IndicatorStep is)
{
    if (p->dim != 2 || !Q) return cudaErrorInvalidValue;
    GridParams gp;
    memset(&gp, 0, sizeof(gp));
    gp.dim = 2;
    gp.plane = total;
    cudaError_t e = launch_prims(total, U, Q, s, is);
    if (e != cudaSuccess) return e;
    const BatchGeom bg{cases, offsets, ncases};
    e = launch_infer<2, MLP_SRC_BATCH>(p, gp, Q, nullptr, thr, nullptr, raw ? raw : flags, s, bg, is);
    if (e != cudaSuccess || !raw) return e;
    mlp_dilate_batch_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(bg, total, raw, flags, is);
    return cudaPeekAtLastError();
}

cudaError_t mlp_features(int dim, const GridParams &gp, const double *U, void *X, cudaStream_t s)
{
    const long long blocks = (gp.plane + 255) / 256 < 4096 ? (gp.plane + 255) / 256 : 4096;
    if (dim == 3) mlp_features_kernel<3><<<(unsigned)blocks, 256, 0, s>>>(gp, U, (__nv_bfloat16 *)X);
    else mlp_features_kernel<2><<<(unsigned)blocks, 256, 0, s>>>(gp, U, (__nv_bfloat16 *)X);
    return cudaPeekAtLastError();
}

int mlp_dim(const mmf_mlp *p) { return p ? p->dim : 0; }
int mlp_error(mmf_mlp *p)
{
    int h = 0;
    if (cudaMemcpy(&h, p->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h;
}

} // namespace mmf

extern "C" {

int mmf_mlp_create(int dim, uint64_t seed, int device, mmf_mlp **out)
{
    if (!out || (dim != 2 && dim != 3)) return set_last_error(MMF_ERR_ARG, "dim must be 2 or 3");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return set_last_error(MMF_ERR_CUDA, "no CUDA device available");
    MLP_CUDA(cudaSetDevice(device));
    mmf_mlp *p = new mmf_mlp();
    p->dim = dim;
    p->device = device;
    p->n = mlp_nparams(dim);
    const int KP = mlp_kpad(dim), KIN = mlp_kin(dim);
    const size_t pb = sizeof(float) * (size_t)p->n;
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&p->params, pb);
    if (e == cudaSuccess) e = cudaMalloc(&p->grad, pb);
    if (e == cudaSuccess) e = cudaMalloc(&p->m, pb);
    if (e == cudaSuccess) e = cudaMalloc(&p->v, pb);
    if (e == cudaSuccess) e = cudaMalloc(&p->loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&p->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&p->w1, sizeof(__nv_bfloat16) * MLP_H * KP);
    if (e == cudaSuccess) e = cudaMalloc(&p->w1c, sizeof(__nv_bfloat16) * MLP_H * KP);
    if (e == cudaSuccess) e = cudaMalloc(&p->w2, sizeof(__nv_bfloat16) * MLP_H * MLP_H);
    if (e == cudaSuccess) e = cudaMalloc(&p->w2t, sizeof(__nv_bfloat16) * MLP_H * MLP_H);
    if (e == cudaSuccess) e = cudaMalloc(&p->w2c, sizeof(__nv_bfloat16) * MLP_H * MLP_H);
    if (e == cudaSuccess) e = cudaMalloc(&p->w2tc, sizeof(__nv_bfloat16) * MLP_H * MLP_H);
    if (e == cudaSuccess) e = cudaMemset(p->m, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(p->v, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(p->err, 0, sizeof(int));
    if (e != cudaSuccess) {
        std::string msg = cudaGetErrorString(e);
        mmf_mlp_destroy(p);
        return set_last_error(MMF_ERR_CUDA, msg.c_str());
    }
    // Glorot-uniform weights from the seed, zero biases, zero padding columns
    std::vector<float> h((size_t)p->n, 0.0f);
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<float> u01(-1.0f, 1.0f);
    const float a1 = std::sqrt(6.0f / (KIN + MLP_H)), a2 = std::sqrt(6.0f / (2 * MLP_H)), a3 = std::sqrt(6.0f / (MLP_H + 1));
    for (int r = 0; r < MLP_H; ++r)
        for (int k = 0; k < KIN; ++k) h[(size_t)r * KP + k] = a1 * u01(rng);
    for (int i = 0; i < MLP_H * MLP_H; ++i) h[(size_t)mlp_off_w2(dim) + i] = a2 * u01(rng);
    for (int i = 0; i < MLP_H; ++i) h[(size_t)mlp_off_w3(dim) + i] = a3 * u01(rng);
    int rc = mmf_mlp_set_params(p, h.data(), p->n);
    if (rc) { mmf_mlp_destroy(p); return rc; }
    *out = p;
    return MMF_OK;
}

int mmf_mlp_destroy(mmf_mlp *p)
{
    if (!p) return MMF_OK;
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    cudaFree(p->params); cudaFree(p->grad); cudaFree(p->m); cudaFree(p->v); cudaFree(p->loss); cudaFree(p->err);
    cudaFree(p->w1); cudaFree(p->w1c); cudaFree(p->w2); cudaFree(p->w2t); cudaFree(p->w2c); cudaFree(p->w2tc);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return MMF_OK;
}

int64_t mmf_mlp_num_params(const mmf_mlp *p) { return p ? p->n : 0; }
int mmf_mlp_input_width(const mmf_mlp *p) { return p ? mlp_kpad(p->dim) : 0; }

int mmf_mlp_get_params(mmf_mlp *p, float *out, int64_t n)
{
    if (!p || !out || n != p->n) return set_last_error(MMF_ERR_ARG, "bad parameter buffer");
    MLP_CUDA(cudaSetDevice(p->device));
    MLP_CUDA(cudaMemcpyAsync(out, p->params, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, p->stream));
    MLP_CUDA(cudaStreamSynchronize(p->stream));
    return MMF_OK;
}

int mmf_mlp_set_params(mmf_mlp *p, const float *in, int64_t n)
{
    if (!p || !in || n != p->n) return set_last_error(MMF_ERR_ARG, "bad parameter buffer");
    MLP_CUDA(cudaSetDevice(p->device));
    MLP_CUDA(cudaMemcpyAsync(p->params, in, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, p->stream));
    int rc = mlp_pack(p);
    if (rc) return rc;
    MLP_CUDA(cudaStreamSynchronize(p->stream));
    return MMF_OK;
}

static int run_train(mmf_mlp *p, const void *d_X, const unsigned char *d_y, int64_t B)
{
    if (B < 16 || B % 16) return set_last_error(MMF_ERR_ARG, "batch must be a positive multiple of 16");
    MLP_CUDA(cudaMemsetAsync(p->grad, 0, sizeof(float) * (size_t)p->n, p->stream));
    MLP_CUDA(cudaMemsetAsync(p->loss, 0, sizeof(float), p->stream));
    MLP_CUDA(cudaMemsetAsync(p->err, 0, sizeof(int), p->stream));
    const unsigned blocks = (unsigned)((B + 127) / 128);
    MlpTrainDev w;
    w.w1c = p->w1c;
    w.w2c = p->w2c;
    w.w2tc = p->w2tc;
    w.params = p->params;
    if (p->dim == 3) {
        MLP_CUDA(cudaFuncSetAttribute(mlp_train_tc_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      mlp_train_tc_smem<3>()));
        mlp_train_tc_kernel<3><<<blocks, 128, mlp_train_tc_smem<3>(), p->stream>>>(
            (const __nv_bfloat16 *)d_X, d_y, (int)B, w, p->grad, p->loss, p->err, p->lim);
    } else {
        MLP_CUDA(cudaFuncSetAttribute(mlp_train_tc_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      mlp_train_tc_smem<2>()));
        mlp_train_tc_kernel<2><<<blocks, 128, mlp_train_tc_smem<2>(), p->stream>>>(
            (const __nv_bfloat16 *)d_X, d_y, (int)B, w, p->grad, p->loss, p->err, p->lim);
    }
    MLP_CUDA(cudaPeekAtLastError());
    return MMF_OK;
}

int mmf_mlp_gradients(mmf_mlp *p, const void *d_X, const unsigned char *d_y, int64_t B, float *grad_out,
                      float *loss_out)
{
    if (!p || !d_X || !d_y) return set_last_error(MMF_ERR_ARG, "null argument");
    MLP_CUDA(cudaSetDevice(p->device));
    int rc = run_train(p, d_X, d_y, B);
    if (rc) return rc;
    float l = 0.0f;
    if (grad_out) MLP_CUDA(cudaMemcpyAsync(grad_out, p->grad, sizeof(float) * (size_t)p->n, cudaMemcpyDeviceToHost, p->stream));
    MLP_CUDA(cudaMemcpyAsync(&l, p->loss, sizeof(float), cudaMemcpyDeviceToHost, p->stream));
    MLP_CUDA(cudaStreamSynchronize(p->stream));
    if (mlp_error(p)) return set_last_error(MMF_ERR_CUDA, "MLP training kernel: an asynchronous-copy or MMA wait gave up");
    if (loss_out) *loss_out = l / (float)B;
    return MMF_OK;
}

int mmf_mlp_train_batch(mmf_mlp *p, const void *d_X, const unsigned char *d_y, int64_t B, float lr, float *loss_out)
{
    NvtxRange range_("mmf_mlp_train_batch");
    if (!p || !d_X || !d_y || !(lr > 0.0f)) return set_last_error(MMF_ERR_ARG, "bad argument");
    MLP_CUDA(cudaSetDevice(p->device));
    int rc = run_train(p, d_X, d_y, B);
    if (rc) return rc;
    p->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - std::pow(b1, (float)p->adam_t), bc2 = 1.0f - std::pow(b2, (float)p->adam_t);
    if (p->dim == 3) mlp_adam_kernel<3><<<64, 256, 0, p->stream>>>(p->params, p->grad, p->m, p->v, lr, b1, b2, 1e-8f, bc1, bc2);
    else mlp_adam_kernel<2><<<64, 256, 0, p->stream>>>(p->params, p->grad, p->m, p->v, lr, b1, b2, 1e-8f, bc1, bc2);
    MLP_CUDA(cudaPeekAtLastError());
    if ((rc = mlp_pack(p))) return rc;
    if (loss_out) {
        float l = 0.0f;
        MLP_CUDA(cudaMemcpyAsync(&l, p->loss, sizeof(float), cudaMemcpyDeviceToHost, p->stream));
        MLP_CUDA(cudaStreamSynchronize(p->stream));
        if (mlp_error(p)) return set_last_error(MMF_ERR_CUDA, "MLP training kernel: an asynchronous-copy or MMA wait gave up");
        *loss_out = l / (float)B;
    }
    return MMF_OK;
}

int mmf_mlp_set_wait_limits(mmf_mlp *p, int64_t wait_limit, int64_t probe_limit)
{
    if (!p || wait_limit < 1 || probe_limit < 0) return set_last_error(MMF_ERR_ARG, "bad argument");
    p->lim.wait = wait_limit;
    p->lim.probe = probe_limit;
    return MMF_OK;
}

int mmf_mlp_predict(mmf_mlp *p, const void *d_X, int64_t n, float *d_prob)
{
    if (!p || !d_X || !d_prob || n < 1) return set_last_error(MMF_ERR_ARG, "bad argument");
    MLP_CUDA(cudaSetDevice(p->device));
    GridParams gp;
    memset(&gp, 0, sizeof(gp));
    gp.dim = p->dim;
    gp.plane = n;
    MLP_CUDA(cudaMemsetAsync(p->err, 0, sizeof(int), p->stream));
    cudaError_t e = (p->dim == 3) ? launch_infer<3, MLP_SRC_X>(p, gp, nullptr, (const __nv_bfloat16 *)d_X, 0.5f, d_prob, nullptr, p->stream)
                                  : launch_infer<2, MLP_SRC_X>(p, gp, nullptr, (const __nv_bfloat16 *)d_X, 0.5f, d_prob, nullptr, p->stream);
    MLP_CUDA(e);
    MLP_CUDA(cudaStreamSynchronize(p->stream));
    if (const int we = mlp_error(p))
        return set_last_error(MMF_ERR_CUDA, we == 3 ? "MLP kernel: the probe wait gave up (nothing in flight)"
                                                    : "MLP kernel: an asynchronous-copy or MMA wait gave up");
    return MMF_OK;
}

} // extern "C"
