// mmf_capi.cu -- the C ABI (include/mmf_gb300.h): context, state transfer
// between the reference's AoS raw layout and the device SoA planes, the
// reference entry points, and the CUDA-graph time loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mmf_gb300.h"
#include "mmf_launch.cuh"

using namespace mmf;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

#define MMF_CUDA(call)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(MMF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

constexpr int GRAPH_STEPS = 16;

// AoS [n_raw][5] (raw order) -> SoA planes (grid order)
__global__ void aos_to_soa_kernel(const double *__restrict__ aos, double *__restrict__ soa, long long n_raw,
                                  long long plane, const long long *__restrict__ raw_to_cell)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n_raw) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    if (g < 0 || g >= plane) return;
#pragma unroll
    for (int k = 0; k < NF; ++k) soa[k * plane + g] = aos[NF * r + k];
}

// flag := 1 if any value of the plane is not +0.0 / -0.0
__global__ void nonzero_plane_kernel(const double *__restrict__ v, long long n, int *flag)
{
    bool nz = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        nz |= (mmf::dbits(v[i]) << 1) != 0;
    if (__any_sync(0xffffffffu, nz) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

__global__ void soa_to_aos_kernel(const double *__restrict__ soa, double *__restrict__ aos, long long n_raw,
                                  long long plane, const long long *__restrict__ raw_to_cell)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n_raw) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    if (g < 0 || g >= plane) return;
#pragma unroll
    for (int k = 0; k < NF; ++k) aos[NF * r + k] = soa[k * plane + g];
}

// Band [base, base + count) of a state in grid order: AoS -> SoA, and
// wflag := 1 when a z-momentum value of the band is not +0 / -0.
__global__ void aos_to_soa_band_kernel(const double *__restrict__ aos, double *__restrict__ soa, long long base,
                                       long long count, long long plane, int *wflag)
{
    bool nz = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const long long g = base + i;
#pragma unroll
        for (int k = 0; k < NF; ++k) soa[k * plane + g] = aos[NF * g + k];
        nz |= (mmf::dbits(aos[NF * g + 3]) << 1) != 0;
    }
    if (wflag && __any_sync(0xffffffffu, nz) && (threadIdx.x & 31) == 0) atomicOr(wflag, 1);
}

__global__ void soa_to_aos_band_kernel(const double *__restrict__ soa, double *__restrict__ aos, long long base,
                                       long long count, long long plane)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const long long g = base + i;
#pragma unroll
        for (int k = 0; k < NF; ++k) aos[NF * g + k] = soa[k * plane + g];
    }
}

} // namespace

namespace mmf {
// Records an error for mmf_last_error() from another translation unit.
int set_last_error(int code, const char *msg) { return fail(code, msg); }

// Checks of a Cartesian grid description, shared by every entry point that
// takes one: dimension, cells per direction, border codes (periodic sides
// paired), cell size, reconstruction order and arithmetic.
int check_grid(const mmf_grid *grid)
{
    if (grid->dim != 2 && grid->dim != 3) return fail(MMF_ERR_ARG, "dim must be 2 or 3");
    for (int d = 0; d < grid->dim; ++d) {
        if (grid->n[d] < 1) return fail(MMF_ERR_ARG, "cells per direction must be >= 1");
        const bool plo = grid->bc_lo[d] == MMF_BC_PERIODIC, phi = grid->bc_hi[d] == MMF_BC_PERIODIC;
        if (plo != phi) return fail(MMF_ERR_ARG, "periodic borders must be paired");
        for (int s = 0; s < 2; ++s) {
            const int bc = s ? grid->bc_hi[d] : grid->bc_lo[d];
            if (bc != MMF_BC_FREE_FLOW && bc != MMF_BC_REFLECTING && bc != MMF_BC_WALL && bc != MMF_BC_DIRICHLET &&
                bc != MMF_BC_PERIODIC)
                return fail(MMF_ERR_ARG, "unknown border condition");
        }
    }
    if (!(grid->h > 0.0)) return fail(MMF_ERR_ARG, "h must be > 0");
    if (grid->order != 1 && grid->order != 2)   // src/reconstruction.cpp:75-76 exits on any other order
        return fail(MMF_ERR_UNSUPPORTED, "reconstruction order must be 1 or 2");
    if (grid->arith != MMF_ARITH_REFERENCE && grid->arith != MMF_ARITH_FAST)
        return fail(MMF_ERR_ARG, "unknown arithmetic");
    return MMF_OK;
}
// mmf_mlp.cu
cudaError_t mlp_indicator(mmf_mlp *p, const GridParams &gp, const double *U, float thr, float *prob,
                          unsigned char *flags, cudaStream_t s, float *Q, unsigned char *raw, IndicatorStep is);
cudaError_t mlp_features(int dim, const GridParams &gp, const double *U, void *X, cudaStream_t s);
int mlp_dim(const mmf_mlp *p);
int mlp_error(mmf_mlp *p);
}

#include "mmf_context.cuh"

static int check_ctx(mmf_ctx *ctx)
{
    if (!ctx) return fail(MMF_ERR_ARG, "null context");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return fail(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}

extern "C" {

const char *mmf_last_error(void) { return g_last_error.c_str(); }
int mmf_abi_version(void) { return MMF_ABI_VERSION; }
int64_t mmf_launch_count(const mmf_ctx *ctx) { return ctx ? ctx->launches : 0; }

int mmf_create(const mmf_grid *grid, int device, mmf_ctx **out)
{
    if (!grid || !out) return fail(MMF_ERR_ARG, "null argument");
    *out = nullptr;
    int rc = mmf::check_grid(grid);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
        return fail(MMF_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev) return fail(MMF_ERR_ARG, "device index out of range");
    MMF_CUDA(cudaSetDevice(device));

    mmf_ctx *c = new mmf_ctx();
    c->device = device;
    c->grid = *grid;
    if (grid->dim == 2) c->grid.n[2] = 1;
    GridParams &gp = c->gp;
    memset(&gp, 0, sizeof(gp));
    gp.dim = grid->dim;
    for (int d = 0; d < 3; ++d) {
        gp.n[d] = c->grid.n[d];
        gp.bc_lo[d] = (d < grid->dim) ? grid->bc_lo[d] : MMF_BC_FREE_FLOW;
        gp.bc_hi[d] = (d < grid->dim) ? grid->bc_hi[d] : MMF_BC_FREE_FLOW;
    }
    dirichlet_conservatives(grid->dirichlet_prim, gp.dir_cons);
    const double h = grid->h;
    gp.area = (grid->dim == 3) ? h * h : h;
    gp.vol = (grid->dim == 3) ? h * h * h : h * h;
    gp.half_area_per_vol = 0.5 * gp.area / gp.vol;
    plan_cartesian(gp, grid->chunk, grid->order == 2 ? BY3D_O2 : BY3D, 0, grid->order == 1 ? TILE3D_DEFAULT : 0,
                   grid->order);
    const size_t bytes = sizeof(double) * NF * (size_t)gp.plane;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->U, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->R, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->W, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->aos, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->ctrl, sizeof(Ctrl));
    if (e == cudaSuccess) e = cudaMalloc(&c->rhs_maxeig, sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->flag, sizeof(int));
    if (e == cudaSuccess && grid->order == 2) {
        e = cudaMalloc(&c->Sl, bytes * grid->dim);
        if (e == cudaSuccess) e = cudaMalloc(&c->lim_flag, (size_t)gp.plane);
        if (e == cudaSuccess) e = cudaMalloc(&c->lim_active, (size_t)gp.plane);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->lim_flag, 0, (size_t)gp.plane, c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->lim_active, 0, (size_t)gp.plane, c->stream);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(c->U, 0, bytes, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->ctrl, 0, sizeof(Ctrl), c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        std::string msg = cudaGetErrorString(e);
        mmf_destroy(c);
        return fail(e == cudaErrorMemoryAllocation ? MMF_ERR_NOMEM : MMF_ERR_CUDA, msg);
    }
    *out = c;
    return MMF_OK;
}

int mmf_destroy(mmf_ctx *c)
{
    if (!c) return MMF_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph_many) cudaGraphExecDestroy(c->graph_many);
    if (c->graph_one) cudaGraphExecDestroy(c->graph_one);
    cudaFree(c->U); cudaFree(c->R); cudaFree(c->W); cudaFree(c->S); cudaFree(c->aos);
    cudaFree(c->raw_to_cell); cudaFree(c->ctrl); cudaFree(c->rhs_maxeig); cudaFree(c->flag);
    cudaFree(c->Sl); cudaFree(c->lim_flag); cudaFree(c->lim_active); cudaFree(c->steplog); cudaFree(c->ind_q);
    cudaFree(c->ind_raw); cudaFree(c->ind_tick);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->tr_stream) {
        cudaStreamSynchronize(c->tr_stream);
        cudaStreamDestroy(c->tr_stream);
    }
    for (int b = 0; b < mmf_ctx::MAX_BANDS; ++b) {
        if (c->band_stream[b]) { cudaStreamSynchronize(c->band_stream[b]); cudaStreamDestroy(c->band_stream[b]); }
        cudaEvent_t evs[5] = {c->ev_up[b], c->ev_tr[b], c->ev_s1[b], c->ev_dn[b], c->ev_s2b[b]};
        for (cudaEvent_t e : evs) if (e) cudaEventDestroy(e);
    }
    if (c->ev_start) cudaEventDestroy(c->ev_start);
    if (c->ev_s2) cudaEventDestroy(c->ev_s2);
    if (c->ev_flag) cudaEventDestroy(c->ev_flag);
    cudaFreeHost(c->h_flag);
    cudaFreeHost(c->h_ctrl);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return MMF_OK;
}

int mmf_set_cell_map(mmf_ctx *c, int64_t n_raw, const int64_t *raw_to_cell)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "n_raw must equal the cell count");
    if (!raw_to_cell) {
        cudaFree(c->raw_to_cell);
        c->raw_to_cell = nullptr;
        return MMF_OK;
    }
    // must be a permutation of the grid cells
    std::string seen((size_t)n_raw, '\0');
    for (int64_t r = 0; r < n_raw; ++r) {
        const int64_t g = raw_to_cell[r];
        if (g < 0 || g >= n_raw || seen[(size_t)g]) return fail(MMF_ERR_ARG, "cell map is not a permutation");
        seen[(size_t)g] = 1;
    }
    if (!c->raw_to_cell) MMF_CUDA(cudaMalloc(&c->raw_to_cell, sizeof(long long) * n_raw));
    MMF_CUDA(cudaMemcpyAsync(c->raw_to_cell, raw_to_cell, sizeof(long long) * n_raw, cudaMemcpyHostToDevice,
                             c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

static int to_soa(mmf_ctx *c, const double *d_aos, double *soa, int64_t n_raw)
{
    const unsigned blocks = (unsigned)((n_raw + 255) / 256);
    aos_to_soa_kernel<<<blocks, 256, 0, c->stream>>>(d_aos, soa, n_raw, c->gp.plane, c->raw_to_cell);
    ++c->launches;
    MMF_CUDA(cudaPeekAtLastError());
    return MMF_OK;
}

// After a state upload: choose the 2D kernels without z-momentum when that
// plane is identically zero (the graphs are rebuilt when the choice changes).
static int refresh_w_zero_impl(mmf_ctx *c)
{
    c->indicator_restart();   // a new state: the next step runs the indicator
    bool wz = false;
    if (c->gp.dim == 2 && c->grid.arith == MMF_ARITH_FAST) {
        MMF_CUDA(cudaMemsetAsync(c->flag, 0, sizeof(int), c->stream));
        const long long n = c->gp.plane;
        const unsigned blocks = (unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
        nonzero_plane_kernel<<<blocks, 256, 0, c->stream>>>(c->U + 3 * n, n, c->flag);
        ++c->launches;
        MMF_CUDA(cudaPeekAtLastError());
        int h = 1;
        MMF_CUDA(cudaMemcpyAsync(&h, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        MMF_CUDA(cudaStreamSynchronize(c->stream));
        wz = (h == 0);
    }
    if (wz != c->w_zero) {
        if (c->graph_many) { cudaGraphExecDestroy(c->graph_many); c->graph_many = nullptr; }
        if (c->graph_one) { cudaGraphExecDestroy(c->graph_one); c->graph_one = nullptr; }
        c->w_zero = wz;
    }
    return MMF_OK;
}

static int from_soa(mmf_ctx *c, const double *soa, double *d_aos, int64_t n_raw)
{
    const unsigned blocks = (unsigned)((n_raw + 255) / 256);
    soa_to_aos_kernel<<<blocks, 256, 0, c->stream>>>(soa, d_aos, n_raw, c->gp.plane, c->raw_to_cell);
    ++c->launches;
    MMF_CUDA(cudaPeekAtLastError());
    return MMF_OK;
}

int mmf_upload_state(mmf_ctx *c, const double *aos, int64_t n_raw)
{
    NvtxRange range_("mmf_upload_state");
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!aos || n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "bad state buffer");
    MMF_CUDA(cudaMemcpyAsync(c->aos, aos, sizeof(double) * NF * n_raw, cudaMemcpyHostToDevice, c->stream));
    if ((rc = to_soa(c, c->aos, c->U, n_raw))) return rc;
    return refresh_w_zero_impl(c);
}

int mmf_download_state(mmf_ctx *c, double *aos, int64_t n_raw)
{
    NvtxRange range_("mmf_download_state");
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!aos || n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "bad state buffer");
    if ((rc = from_soa(c, c->U, c->aos, n_raw))) return rc;
    MMF_CUDA(cudaMemcpyAsync(aos, c->aos, sizeof(double) * NF * n_raw, cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

int mmf_upload_state_device(mmf_ctx *c, const double *d_aos, int64_t n_raw)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!d_aos || n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "bad state buffer");
    if ((rc = to_soa(c, d_aos, c->U, n_raw))) return rc;
    return refresh_w_zero_impl(c);
}

int mmf_download_state_device(mmf_ctx *c, double *d_aos, int64_t n_raw)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!d_aos || n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "bad state buffer");
    return from_soa(c, c->U, d_aos, n_raw);
}

int mmf_compute_rhs(mmf_ctx *c, const double *cons, double *rhs, double *max_eig, int64_t n_raw)
{
    NvtxRange range_("mmf_compute_rhs");
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!cons || !rhs || n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "bad buffers");
    const size_t bytes = sizeof(double) * NF * (size_t)n_raw;
    if (!c->S) MMF_CUDA(cudaMalloc(&c->S, bytes));
    MMF_CUDA(cudaMemcpyAsync(c->aos, cons, bytes, cudaMemcpyHostToDevice, c->stream));
    if ((rc = to_soa(c, c->aos, c->S, n_raw))) return rc;
    MMF_CUDA(cudaMemsetAsync(c->rhs_maxeig, 0, sizeof(double), c->stream));
    // the residual of stage 'RHS' lands in R; S is the input state
    if (c->grid.order == 2) {
        MMF_CUDA(c->o2(O2_SLOPES, STAGE_RHS, c->S, nullptr, nullptr));
        MMF_CUDA(c->o2(O2_STAGE, STAGE_RHS, c->S, c->R, nullptr));
    } else {
        StageArgs sa;
        sa.U = c->S; sa.R = c->R; sa.W = c->W; sa.out = c->R; sa.ctrl = c->ctrl; sa.rhs_maxeig = c->rhs_maxeig;
        ++c->launches;
        MMF_CUDA(launch_stage_exact(STAGE_RHS, c->gp, sa, c->stream));
    }
    if ((rc = from_soa(c, c->R, c->aos, n_raw))) return rc;
    MMF_CUDA(cudaMemcpyAsync(rhs, c->aos, bytes, cudaMemcpyDeviceToHost, c->stream));
    double me = 0.0;
    MMF_CUDA(cudaMemcpyAsync(&me, c->rhs_maxeig, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    if (max_eig) *max_eig = me;
    return MMF_OK;
}

// grid-order byte array <-> raw order
__global__ void bytes_to_raw_kernel(const unsigned char *grid_v, unsigned char *raw_v, long long n,
                                    const long long *raw_to_cell)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    raw_v[r] = (g >= 0 && g < n) ? grid_v[g] : 0;
}

__global__ void bytes_from_raw_kernel(const unsigned char *raw_v, unsigned char *grid_v, long long n,
                                      const long long *raw_to_cell)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    if (g >= 0 && g < n) grid_v[g] = raw_v[r];
}

// slopes planes (grid order) -> AoS [n_raw][3][5] (raw order)
__global__ void slopes_to_raw_kernel(const double *S, double *out, long long n, int dim, const long long *raw_to_cell)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    if (g < 0 || g >= n) return;
    for (int d = 0; d < 3; ++d)
        for (int k = 0; k < NF; ++k) out[(r * 3 + d) * NF + k] = (d < dim) ? S[(long long)(d * NF + k) * n + g] : 0.0;
}

int mmf_compute_polynomials(mmf_ctx *c, const double *cons, double *slopes, unsigned char *limiter_active,
                            int64_t n_raw)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->grid.order == 1) return MMF_OK;   // src/reconstruction.cpp:47-55 is empty at order 1
    if (!cons || n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "bad state buffer");
    const size_t bytes = sizeof(double) * NF * (size_t)n_raw;
    if (!c->S) MMF_CUDA(cudaMalloc(&c->S, bytes));
    MMF_CUDA(cudaMemcpyAsync(c->aos, cons, bytes, cudaMemcpyHostToDevice, c->stream));
    if ((rc = to_soa(c, c->aos, c->S, n_raw))) return rc;
    MMF_CUDA(c->o2(O2_SLOPES, STAGE_RHS, c->S, nullptr, c->lim_active));
    const unsigned blocks = (unsigned)((n_raw + 255) / 256);
    if (slopes) {
        double *tmp = nullptr;
        MMF_CUDA(cudaMalloc(&tmp, bytes * 3));
        slopes_to_raw_kernel<<<blocks, 256, 0, c->stream>>>(c->Sl, tmp, n_raw, c->grid.dim, c->raw_to_cell);
        ++c->launches;
        cudaError_t e = cudaMemcpyAsync(slopes, tmp, bytes * 3, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(tmp);
        MMF_CUDA(e);
    }
    if (limiter_active) return mmf_get_limiter_activity(c, limiter_active, n_raw);
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

int mmf_set_limiter(mmf_ctx *c, int mode, const unsigned char *flags, int64_t n_raw)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (mode != LIMIT_ALL && mode != LIMIT_NONE && mode != LIMIT_FLAGGED) return fail(MMF_ERR_ARG, "unknown limiter mode");
    if (c->grid.order != 2) return fail(MMF_ERR_UNSUPPORTED, "the limiter applies to order 2");
    if (flags) {
        if (n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "flag count must equal the cell count");
        unsigned char *tmp = nullptr;
        MMF_CUDA(cudaMalloc(&tmp, (size_t)n_raw));
        cudaError_t e = cudaMemcpyAsync(tmp, flags, (size_t)n_raw, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) {
            bytes_from_raw_kernel<<<(unsigned)((n_raw + 255) / 256), 256, 0, c->stream>>>(tmp, c->lim_flag, n_raw,
                                                                                          c->raw_to_cell);
            ++c->launches;
            e = cudaPeekAtLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(tmp);
        MMF_CUDA(e);
    }
    c->limit_mode = mode;
    return MMF_OK;
}

int mmf_set_limiter_flags_device(mmf_ctx *c, const unsigned char *d_flags_grid)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->grid.order != 2 || !d_flags_grid) return fail(MMF_ERR_ARG, "order-2 context and flags required");
    MMF_CUDA(cudaMemcpyAsync(c->lim_flag, d_flags_grid, (size_t)c->gp.plane, cudaMemcpyDeviceToDevice, c->stream));
    c->limit_mode = LIMIT_FLAGGED;
    return MMF_OK;
}

int mmf_features(mmf_ctx *c, void *d_X)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!d_X) return fail(MMF_ERR_ARG, "null feature buffer");
    ++c->launches;
    MMF_CUDA(mlp_features(c->grid.dim, c->gp, c->U, d_X, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

int mmf_indicator(mmf_ctx *c, mmf_mlp *mlp, float threshold, float *prob, unsigned char *flags)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!mlp) return fail(MMF_ERR_ARG, "null MLP");
    if (c->grid.order != 2) return fail(MMF_ERR_UNSUPPORTED, "the indicator drives the order-2 limiter");
    if (mlp_dim(mlp) != c->grid.dim) return fail(MMF_ERR_ARG, "MLP dimension differs from the mesh");
    const long long n = c->gp.plane;
    float *dprob = nullptr, *q = nullptr;
    if (prob) MMF_CUDA(cudaMalloc(&dprob, sizeof(float) * (size_t)n));
    cudaError_t e = cudaMalloc(&q, sizeof(float) * 5 * (size_t)n);
    const bool dilate = c->ind_period > 1 && c->ind_raw;
    c->launches += dilate ? 3 : 2;
    if (e == cudaSuccess)
        e = mlp_indicator(mlp, c->gp, c->U, threshold, dprob, c->lim_flag, c->stream, q, dilate ? c->ind_raw : nullptr,
                          IndicatorStep{1, nullptr});
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(q);
    if (e == cudaSuccess && mlp_error(mlp)) { cudaFree(dprob); return fail(MMF_ERR_CUDA, "indicator: a wait gave up"); }
    if (e == cudaSuccess && prob) {
        std::vector<float> tmp((size_t)n);
        e = cudaMemcpy(tmp.data(), dprob, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) {
            std::vector<long long> map((size_t)n);
            if (c->raw_to_cell) e = cudaMemcpy(map.data(), c->raw_to_cell, sizeof(long long) * (size_t)n, cudaMemcpyDeviceToHost);
            for (long long r = 0; r < n && e == cudaSuccess; ++r) prob[r] = tmp[(size_t)(c->raw_to_cell ? map[(size_t)r] : r)];
        }
    }
    cudaFree(dprob);
    MMF_CUDA(e);
    c->limit_mode = LIMIT_FLAGGED;
    if (flags) {
        unsigned char *tmp = nullptr;
        MMF_CUDA(cudaMalloc(&tmp, (size_t)n));
        bytes_to_raw_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->lim_flag, tmp, n, c->raw_to_cell);
        ++c->launches;
        e = cudaPeekAtLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(flags, tmp, (size_t)n, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(tmp);
        MMF_CUDA(e);
    }
    return MMF_OK;
}

int mmf_limiter_labels(mmf_ctx *c, unsigned char *d_labels)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->grid.order != 2) return fail(MMF_ERR_UNSUPPORTED, "the limiter applies to order 2");
    if (!d_labels) return fail(MMF_ERR_ARG, "null label buffer");
    // the reference-arithmetic limiter on every cell, on the uploaded state
    const int saved = c->limit_mode;
    c->limit_mode = LIMIT_ALL;
    cudaError_t e = c->o2(O2_SLOPES, STAGE_RHS, c->U, nullptr, c->lim_active);
    c->limit_mode = saved;
    MMF_CUDA(e);
    MMF_CUDA(cudaMemcpyAsync(d_labels, c->lim_active, (size_t)c->gp.plane, cudaMemcpyDeviceToDevice, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

int mmf_set_indicator(mmf_ctx *c, mmf_mlp *mlp, float threshold)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (mlp && c->grid.order != 2) return fail(MMF_ERR_UNSUPPORTED, "the indicator drives the order-2 limiter");
    if (mlp && mlp_dim(mlp) != c->grid.dim) return fail(MMF_ERR_ARG, "MLP dimension differs from the mesh");
    if (mlp && !c->ind_q) MMF_CUDA(cudaMalloc(&c->ind_q, sizeof(float) * 5 * (size_t)c->gp.plane));
    c->indicator = mlp;
    c->ind_threshold = threshold;
    c->limit_mode = mlp ? LIMIT_FLAGGED : LIMIT_ALL;
    c->indicator_restart();
    if (c->graph_many) { cudaGraphExecDestroy(c->graph_many); c->graph_many = nullptr; }
    if (c->graph_one) { cudaGraphExecDestroy(c->graph_one); c->graph_one = nullptr; }
    return MMF_OK;
}

int mmf_set_indicator_period(mmf_ctx *c, int period)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (period != 1 && period != 2) return fail(MMF_ERR_ARG, "the indicator period must be 1 or 2");
    if (c->grid.order != 2) return fail(MMF_ERR_UNSUPPORTED, "the indicator drives the order-2 limiter");
    if (period > 1 && !c->ind_raw) {
        MMF_CUDA(cudaMalloc(&c->ind_raw, (size_t)c->gp.plane));
        MMF_CUDA(cudaMemsetAsync(c->ind_raw, 0, (size_t)c->gp.plane, c->stream));
    }
    if (period > 1 && !c->ind_tick) MMF_CUDA(cudaMalloc(&c->ind_tick, sizeof(int)));
    c->ind_period = period;
    c->indicator_restart();
    if (c->graph_many) { cudaGraphExecDestroy(c->graph_many); c->graph_many = nullptr; }
    if (c->graph_one) { cudaGraphExecDestroy(c->graph_one); c->graph_one = nullptr; }
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

int mmf_get_limiter_activity(mmf_ctx *c, unsigned char *active, int64_t n_raw)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (c->grid.order != 2) return fail(MMF_ERR_UNSUPPORTED, "the limiter applies to order 2");
    if (!active || n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "bad buffer");
    unsigned char *tmp = nullptr;
    MMF_CUDA(cudaMalloc(&tmp, (size_t)n_raw));
    bytes_to_raw_kernel<<<(unsigned)((n_raw + 255) / 256), 256, 0, c->stream>>>(c->lim_active, tmp, n_raw,
                                                                                c->raw_to_cell);
    ++c->launches;
    cudaError_t e = cudaPeekAtLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(active, tmp, (size_t)n_raw, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(tmp);
    MMF_CUDA(e);
    return MMF_OK;
}

int mmf_time_setup(mmf_ctx *c, double cfl, double t, double t_end, int64_t max_steps)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!(cfl > 0.0)) return fail(MMF_ERR_ARG, "CFL must be > 0");
    if (std::isinf(t_end) && max_steps < 0) return fail(MMF_ERR_ARG, "infinite end time needs max_steps");
    Ctrl h;
    memset(&h, 0, sizeof(h));
    h.t = t;
    h.t_end = t_end;
    h.cfl_h = 0.9 * cfl * c->grid.h;
    h.max_steps = (max_steps < 0) ? LLONG_MAX : max_steps;
    h.log = c->steplog;
    h.log_cap = c->steplog_cap;
    MMF_CUDA(cudaMemcpyAsync(c->ctrl, &h, sizeof(Ctrl), cudaMemcpyHostToDevice, c->stream));
    c->indicator_restart();
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    c->cfl = cfl;
    c->time_ready = true;
    return MMF_OK;
}

static int build_graph(mmf_ctx *c, int steps, cudaGraphExec_t *exec)
{
    cudaGraph_t g = nullptr;
    if (c->gp.dim == 3 && c->gp.tile3d == 2) {
        if (c->grid.arith == MMF_ARITH_REFERENCE) prime_tile3d_exact();
        else prime_tile3d_fast();
    }
    MMF_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    const long long before = c->launches;
    for (int s = 0; s < steps && err == cudaSuccess; ++s) err = c->rk_step();
    c->launches = before;   // captured, not executed
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (err != cudaSuccess) { if (g) cudaGraphDestroy(g); return fail(MMF_ERR_CUDA, cudaGetErrorString(err)); }
    if (e2 != cudaSuccess) return fail(MMF_ERR_CUDA, cudaGetErrorString(e2));
    cudaError_t e3 = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return fail(MMF_ERR_CUDA, cudaGetErrorString(e3));
    return MMF_OK;
}

int mmf_advance(mmf_ctx *c, int64_t n_steps, double *t_out, int64_t *steps_done)
{
    NvtxRange range_("mmf_advance");
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->time_ready) return fail(MMF_ERR_ARG, "mmf_time_setup first");
    if (n_steps < 0) return fail(MMF_ERR_ARG, "n_steps < 0");
    if (!c->graph_many && (rc = build_graph(c, GRAPH_STEPS, &c->graph_many))) return rc;
    if (!c->graph_one && (rc = build_graph(c, 1, &c->graph_one))) return rc;
    // The graphs are enqueued in rounds of at most CHECK_STEPS steps; after
    // each round the control block tells whether the run has ended (end time,
    // step limit or a non-physical state), so that asking for many more steps
    // than the run needs launches no idle graphs.
    constexpr int64_t CHECK_STEPS = 64 * GRAPH_STEPS;
    Ctrl before, after;
    MMF_CUDA(cudaMemcpyAsync(&before, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    int64_t left = n_steps;
    for (;;) {
        int64_t round = left < CHECK_STEPS ? left : CHECK_STEPS;
        left -= round;
        while (round >= GRAPH_STEPS) {
            MMF_CUDA(cudaGraphLaunch(c->graph_many, c->stream));
            c->launches += c->launches_per_step() * GRAPH_STEPS;
            round -= GRAPH_STEPS;
        }
        while (round-- > 0) {
            MMF_CUDA(cudaGraphLaunch(c->graph_one, c->stream));
            c->launches += c->launches_per_step();
        }
        MMF_CUDA(cudaMemcpyAsync(&after, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
        MMF_CUDA(cudaStreamSynchronize(c->stream));
        const bool ended = !(after.t < after.t_end && after.step < after.max_steps) || after.status != 0;
        if (left == 0 || ended) break;
    }
    if (t_out) *t_out = after.t;
    if (steps_done) *steps_done = after.step - before.step;
    if (after.status) return fail(MMF_ERR_STATE, "non-physical state (negative density/pressure or NaN)");
    return MMF_OK;
}

int mmf_advance_async(mmf_ctx *c, int64_t n_steps)
{
    NvtxRange range_("mmf_advance_async");
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->time_ready) return fail(MMF_ERR_ARG, "mmf_time_setup first");
    if (n_steps < 0) return fail(MMF_ERR_ARG, "n_steps < 0");
    if (!c->graph_many && (rc = build_graph(c, GRAPH_STEPS, &c->graph_many))) return rc;
    if (!c->graph_one && (rc = build_graph(c, 1, &c->graph_one))) return rc;
    int64_t left = n_steps;
    while (left >= GRAPH_STEPS) {
        MMF_CUDA(cudaGraphLaunch(c->graph_many, c->stream));
        c->launches += c->launches_per_step() * GRAPH_STEPS;
        left -= GRAPH_STEPS;
    }
    while (left-- > 0) {
        MMF_CUDA(cudaGraphLaunch(c->graph_one, c->stream));
        c->launches += c->launches_per_step();
    }
    return MMF_OK;
}

int mmf_time_info(mmf_ctx *c, double *t, int64_t *step)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    Ctrl h;
    MMF_CUDA(cudaMemcpyAsync(&h, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    if (t) *t = h.t;
    if (step) *step = h.step;
    return MMF_OK;
}

void *mmf_get_stream(mmf_ctx *c) { return c ? (void *)c->stream : nullptr; }

// ---- pipelined host round trip ------------------------------------------
// The state is cut into K bands along the slowest axis (rows in 2D, planes in
// 3D).  Band b's upload (copy stream) overlaps the transposition and the
// stage-1 kernels of the bands already on the device; the stage-1 band
// kernels run on one stream per band (band 0 at the highest priority) so that
// they overlap one another and the transpositions.  Stage 2 needs the step's
// dt, a max over every cell of stage 1, so it starts once stage 1 is done
// everywhere; in the last step it then runs band by band, each band's stage 3
// follows as soon as stage 2 is done on the rows it reads, and each band's
// stage 3 is followed by its transposition and its download (copy stream):
// bands finish in order and the downloads overlap the rest of the step.
// Band launches march short chunks so that each has work for every SM.
static constexpr int S3_STREAMS = 2;   // streams the stage-3 bands take in turn
static constexpr int S2_STREAMS = 2;   // streams the stage-2 bands take in turn

// The i-th stage-3 band launch takes the band streams of the highest
// priorities in turn; the i-th stage-2 band launch the next ones.  At most
// S2_STREAMS + S3_STREAMS band kernels then share the GPU, enough to fill it,
// so that bands finish roughly in order and the downloads start early.
static cudaStream_t s3_stream(mmf_ctx *c, int i) { return c->band_stream[i % S3_STREAMS]; }
static cudaStream_t s2_stream(mmf_ctx *c, int i) { return c->band_stream[S3_STREAMS + i % S2_STREAMS]; }

struct BandPlan {
    int K = 0;
    int rows = 0;          // rows (planes) per band, a multiple of chunk
    int chunk = 0;         // marching chunk of the band launches
    long long slab = 0;    // cells per row (plane)
    int n_slow = 0;
};

static BandPlan band_plan(const mmf_ctx *c)
{
    BandPlan p;
    const GridParams &gp = c->gp;
    p.n_slow = gp.dim == 2 ? gp.n[1] : gp.n[2];
    p.slab = gp.dim == 2 ? (long long)gp.n[0] : (long long)gp.n[0] * gp.n[1];
    if (p.n_slow < 64 || p.slab * p.n_slow < (1 << 18)) return p;   // too small to pay
    // measured best: 8 bands in 2D (1024^2 e2e 1.36-1.37 G cell-updates/s
    // against 1.33 with 12 bands and 1.25-1.26 with 16), 16 bands in 3D (256^3:
    // 1.193-1.195 against 1.176-1.182 with 8)
    const int K = gp.dim == 3 ? 16 : 8;
    int rows = (p.n_slow + K - 1) / K;
    // measured best: 8 rows for 1024^2 and 2048^2, 8 planes for 256^3 (16.00 ms
    // per round trip against 16.28 with 16 planes and 16.90 with 4)
    const int ch = std::min(8, rows);
    rows = (rows + ch - 1) / ch * ch;
    p.K = (p.n_slow + rows - 1) / rows;
    p.rows = rows;
    p.chunk = ch;
    return p;
}

static GridParams band_params(const mmf_ctx *c, const BandPlan &p, int b, int bookkeep)
{
    GridParams g = c->gp;
    const int r0 = b * p.rows, r1 = std::min(p.n_slow, r0 + p.rows);
    g.chunk = p.chunk;
    g.chunk0 = r0 / p.chunk;
    g.nchunk = (r1 - r0 + p.chunk - 1) / p.chunk;
    g.bookkeep = bookkeep;
    return g;
}


static int pipeline_resources(mmf_ctx *c)
{
    if (c->copy_stream) return MMF_OK;
    int least = 0, greatest = 0;
    MMF_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    MMF_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    MMF_CUDA(cudaStreamCreateWithPriority(&c->tr_stream, cudaStreamNonBlocking, greatest));
    for (int b = 0; b < mmf_ctx::MAX_BANDS; ++b) {
        const int prio = std::min(least, greatest + b);   // greatest is the numerically lowest
        MMF_CUDA(cudaStreamCreateWithPriority(&c->band_stream[b], cudaStreamNonBlocking, prio));
        MMF_CUDA(cudaEventCreateWithFlags(&c->ev_up[b], cudaEventDisableTiming));
        MMF_CUDA(cudaEventCreateWithFlags(&c->ev_tr[b], cudaEventDisableTiming));
        MMF_CUDA(cudaEventCreateWithFlags(&c->ev_s1[b], cudaEventDisableTiming));
        MMF_CUDA(cudaEventCreateWithFlags(&c->ev_dn[b], cudaEventDisableTiming));
        MMF_CUDA(cudaEventCreateWithFlags(&c->ev_s2b[b], cudaEventDisableTiming));
    }
    MMF_CUDA(cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming));
    MMF_CUDA(cudaEventCreateWithFlags(&c->ev_s2, cudaEventDisableTiming));
    MMF_CUDA(cudaEventCreateWithFlags(&c->ev_flag, cudaEventDisableTiming));
    MMF_CUDA(cudaHostAlloc(&c->h_flag, sizeof(int), cudaHostAllocDefault));
    MMF_CUDA(cudaHostAlloc(&c->h_ctrl, sizeof(Ctrl), cudaHostAllocDefault));
    return MMF_OK;
}

static bool pipeline_applies(const mmf_ctx *c, const double *aos, int64_t n_steps)
{
    // the learned indicator reads the whole state before the slopes: no bands
    if (c->raw_to_cell || n_steps < 1 || (c->grid.order == 2 && c->indicator)) return false;
    const BandPlan p = band_plan(c);
    if (p.K < 2 || p.K > mmf_ctx::MAX_BANDS) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, aos) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeHost;   // page-locked: the copies run asynchronously
}

static int advance_host_pipelined(mmf_ctx *c, double *aos, int64_t n_steps, double *t_out)
{
    int rc = pipeline_resources(c);
    if (rc) return rc;
    const BandPlan p = band_plan(c);
    const GridParams &gp = c->gp;
    const long long plane = gp.plane;
    const bool periodic_slow = (gp.dim == 2 ? gp.bc_lo[1] : gp.bc_lo[2]) == BC_PERIODIC;
    const bool check_w = gp.dim == 2 && c->grid.arith == MMF_ARITH_FAST;
    const bool o2 = c->grid.order == 2;
    const int K = p.K;
    auto band_cells = [&](int b, long long &base, long long &count) {
        const int r0 = b * p.rows, r1 = std::min(p.n_slow, r0 + p.rows);
        base = (long long)r0 * p.slab;
        count = (long long)(r1 - r0) * p.slab;
    };
    auto tr_blocks = [](long long count) { return (unsigned)std::min<long long>((count + 255) / 256, 4L * 152); };
    // stage 1 over the chunks of 'g' (order 2: with the slopes of its rows and
    // of the rows on both sides already computed)
    auto stage1 = [&](const GridParams &g, cudaStream_t s) {
        return o2 ? c->o2_gp(O2_STAGE, STAGE_1, g, c->U, c->R, nullptr, s, 0, 0)
                  : c->stage_gp(STAGE_1, g, c->U, c->R, s);
    };
    // order 2: the stage-1 slopes (and the limiter activity) of rows [r0, r1)
    auto slopes1 = [&](int r0, int r1, cudaStream_t s) {
        return c->o2_gp(O2_SLOPES, STAGE_1, c->gp, c->U, nullptr, c->lim_active, s, (long long)r0 * p.slab,
                        (long long)r1 * p.slab);
    };
    // the whole-grid stages on the context stream
    auto whole_stage1 = [&]() -> cudaError_t {
        if (!o2) return c->stage(STAGE_1, c->U, c->R);
        cudaError_t e = c->o2(O2_SLOPES, STAGE_1, c->U, nullptr, c->lim_active);
        return e == cudaSuccess ? c->o2(O2_STAGE, STAGE_1, c->U, c->R, nullptr) : e;
    };
    auto whole_stage2 = [&]() -> cudaError_t {
        if (!o2) return c->stage(STAGE_2, c->U, c->W);
        cudaError_t e = c->o2(O2_FORM_W1, STAGE_2, c->U, c->W, nullptr);
        if (e == cudaSuccess) e = c->o2(O2_SLOPES, STAGE_2, c->W, nullptr, nullptr);
        return e == cudaSuccess ? c->o2(O2_STAGE, STAGE_2, c->W, c->R, nullptr) : e;
    };
    auto whole_stage3 = [&]() -> cudaError_t {
        if (!o2) return c->stage(STAGE_3, c->U, c->U);
        cudaError_t e = c->o2(O2_SLOPES, STAGE_3, c->R, nullptr, nullptr);
        return e == cudaSuccess ? c->o2(O2_STAGE, STAGE_3, c->R, c->U, nullptr) : e;
    };
    // the download of band b after its stage 3, on stream bs
    auto download_band = [&](int b, cudaStream_t bs) -> cudaError_t {
        long long base, count;
        band_cells(b, base, count);
        soa_to_aos_band_kernel<<<tr_blocks(count), 256, 0, bs>>>(c->U, c->aos, base, count, plane);
        ++c->launches;
        cudaError_t e = cudaPeekAtLastError();
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_dn[b], bs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_stream, c->ev_dn[b], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(aos + NF * base, c->aos + NF * base, sizeof(double) * NF * count,
                                cudaMemcpyDeviceToHost, c->copy_stream);
        return e;
    };

    // upload and transposition, band by band; the device buffers are free once
    // the work enqueued before this call has run
    MMF_CUDA(cudaMemsetAsync(c->flag, 0, sizeof(int), c->stream));
    MMF_CUDA(cudaEventRecord(c->ev_start, c->stream));
    MMF_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_start, 0));
    MMF_CUDA(cudaStreamWaitEvent(c->tr_stream, c->ev_start, 0));
    for (int b = 0; b < K; ++b) {
        long long base, count;
        band_cells(b, base, count);
        MMF_CUDA(cudaMemcpyAsync(c->aos + NF * base, aos + NF * base, sizeof(double) * NF * count,
                                 cudaMemcpyHostToDevice, c->copy_stream));
        MMF_CUDA(cudaEventRecord(c->ev_up[b], c->copy_stream));
    }
    for (int b = 0; b < K; ++b) {
        long long base, count;
        band_cells(b, base, count);
        // the transpositions have a stream of the highest priority, so that the
        // stage-1 kernels already running do not hold them back
        MMF_CUDA(cudaStreamWaitEvent(c->tr_stream, c->ev_up[b], 0));
        aos_to_soa_band_kernel<<<tr_blocks(count), 256, 0, c->tr_stream>>>(c->aos, c->U, base, count, plane,
                                                                            check_w ? c->flag : nullptr);
        ++c->launches;
        MMF_CUDA(cudaPeekAtLastError());
        MMF_CUDA(cudaEventRecord(c->ev_tr[b], c->tr_stream));
    }
    if (check_w) {
        MMF_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_tr[K - 1], 0));
        MMF_CUDA(cudaMemcpyAsync(c->h_flag, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->copy_stream));
        MMF_CUDA(cudaEventRecord(c->ev_flag, c->copy_stream));
    }
    // Stage 1 chunk by chunk as soon as the rows it reads are on the device:
    // once bands 0..b are transposed (rows below r_b), the chunks whose top
    // neighbour row is below r_b run (on band b's stream); chunk 0 of a
    // periodic slow axis reads the last row and waits for the last band.
    // Order 2 first computes the slopes of band b's rows (they read one row
    // on each side, so they wait for band b + 1), and a stage-1 chunk also
    // reads the slopes of the rows on both sides (band b - 1's last row).
    {
        const int nch = (p.n_slow + p.chunk - 1) / p.chunk;
        int next = periodic_slow ? 1 : 0;   // first chunk not yet launched
        for (int b = 0; b < K; ++b) {
            cudaStream_t bs = c->band_stream[b];
            const int r0 = b * p.rows, rb = std::min(p.n_slow, (b + 1) * p.rows);
            int upto = (b == K - 1) ? nch : (rb - 1) / p.chunk;   // chunks [next, upto) are ready
            const bool first0 = periodic_slow && b == K - 1;
            if (o2) {
                MMF_CUDA(cudaStreamWaitEvent(bs, c->ev_tr[std::min(b + 1, K - 1)], 0));
                // a periodic row 0 reads the last row: its slopes come with the last band
                MMF_CUDA(slopes1(periodic_slow && b == 0 ? 1 : r0, rb, bs));
                if (periodic_slow && b == K - 1) MMF_CUDA(slopes1(0, 1, bs));
                // ev_s2b[b]: the slopes of bands 0..b are done (each band's event
                // follows the previous one's), as the chunks launched here may
                // reach back more than one band when a band is a single chunk
                if (b > 0) MMF_CUDA(cudaStreamWaitEvent(bs, c->ev_s2b[b - 1], 0));
                MMF_CUDA(cudaEventRecord(c->ev_s2b[b], bs));
            } else {
                MMF_CUDA(cudaStreamWaitEvent(bs, c->ev_tr[b], 0));
            }
            if (upto > next || first0) {
                GridParams g = c->gp;
                g.chunk = p.chunk;
                g.bookkeep = (next == 0 || first0) ? 1 : 0;   // once per stage (idempotent for stage 1)
                if (upto > next) {
                    g.chunk0 = next;
                    g.nchunk = upto - next;
                    MMF_CUDA(stage1(g, bs));
                    next = upto;
                }
                if (first0) {
                    g.chunk0 = 0;
                    g.nchunk = 1;
                    MMF_CUDA(stage1(g, bs));
                }
            }
            MMF_CUDA(cudaEventRecord(c->ev_s1[b], bs));
        }
    }
    for (int q = 0; q < K; ++q) MMF_CUDA(cudaStreamWaitEvent(c->stream, c->ev_s1[q], 0));
    if (check_w) {
        // the stage-1 kernels used the previous z-momentum choice; redo stage 1
        // on the whole grid if this state does not fit it
        MMF_CUDA(cudaEventSynchronize(c->ev_flag));
        const bool wz = (*c->h_flag == 0);
        if (wz != c->w_zero) {
            const bool redo = c->w_zero;   // the 4-field kernels skipped a non-zero plane
            c->w_zero = wz;
            if (c->graph_many) { cudaGraphExecDestroy(c->graph_many); c->graph_many = nullptr; }
            if (c->graph_one) { cudaGraphExecDestroy(c->graph_one); c->graph_one = nullptr; }
            if (redo) {
                MMF_CUDA(cudaMemsetAsync(&c->ctrl->maxeig_bits, 0, sizeof(unsigned long long), c->stream));
                MMF_CUDA(cudaMemsetAsync(&c->ctrl->status, 0, sizeof(unsigned), c->stream));
                MMF_CUDA(whole_stage1());
            }
        }
    }
    for (int64_t s = 0; s < n_steps; ++s) {
        if (s > 0) MMF_CUDA(whole_stage1());
        if (s + 1 < n_steps) {
            MMF_CUDA(whole_stage2());
            MMF_CUDA(whole_stage3());
            continue;
        }
        if (o2) {
            // last step, order 2: stage 2 and the stage-3 slopes on the whole
            // grid, then stage 3 band by band (a band reads W2 and the slopes
            // only, and writes U of its own cells), each followed by its
            // download, on two streams taken in turn
            MMF_CUDA(whole_stage2());
            MMF_CUDA(c->o2(O2_SLOPES, STAGE_3, c->R, nullptr, nullptr));
            MMF_CUDA(cudaEventRecord(c->ev_s2, c->stream));
            for (int b = 0; b < K; ++b) {
                cudaStream_t bs = s3_stream(c, b);
                if (b < S3_STREAMS) MMF_CUDA(cudaStreamWaitEvent(bs, c->ev_s2, 0));
                MMF_CUDA(c->o2_gp(O2_STAGE, STAGE_3, band_params(c, p, b, b == K - 1), c->R, c->U, nullptr, bs, 0, 0));
                MMF_CUDA(download_band(b, bs));
            }
            continue;
        }
        // last step, order 1: stage 2 band by band once stage 1 is done
        // everywhere (dt), stage 3 of a band once stage 2 is done on its rows
        // and the two neighbour rows, then its transposition and its download
        MMF_CUDA(cudaEventRecord(c->ev_s2, c->stream));   // stage 1 done
        for (int b = 0; b < K; ++b) {
            cudaStream_t bs = s2_stream(c, b);
            if (b < S2_STREAMS) MMF_CUDA(cudaStreamWaitEvent(bs, c->ev_s2, 0));
            // band 0 writes dt to the control block for stage 3
            MMF_CUDA(c->stage_gp(STAGE_2, band_params(c, p, b, b == 0), c->U, c->W, bs));
            MMF_CUDA(cudaEventRecord(c->ev_s2b[b], bs));
        }
        // stage-2 bands a stage-3 band waits for: its own, those of its two
        // neighbour rows (wrapped on a periodic slow axis; stage 3 writes U in
        // place, which those stage-2 bands read) and band 0 (dt).  Bands are
        // issued in the order their stage-2 inputs complete.
        std::vector<unsigned> dep(K);
        std::vector<int> order(K);
        for (int b = 0; b < K; ++b) {
            unsigned m = 1u | (1u << b);
            if (b > 0) m |= 1u << (b - 1);
            else if (periodic_slow) m |= 1u << (K - 1);
            if (b + 1 < K) m |= 1u << (b + 1);
            else if (periodic_slow) m |= 1u;
            dep[b] = m;
            order[b] = b;
        }
        auto ready = [&](int b) {   // the last stage-2 band it needs
            int r = 0;
            for (int q = 0; q < K; ++q) if (dep[b] & (1u << q)) r = q;
            return r;
        };
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return ready(x) < ready(y); });
        for (int i = 0; i < K; ++i) {
            const int b = order[i];
            cudaStream_t bs = s3_stream(c, i);
            // the last stage-3 launch advances the step in the control block
            // once every stage-2 band has read it
            const bool last = (i == K - 1);
            for (int q = 0; q < K; ++q)
                if (last || (dep[b] & (1u << q))) MMF_CUDA(cudaStreamWaitEvent(bs, c->ev_s2b[q], 0));
            MMF_CUDA(c->stage_gp(STAGE_3, band_params(c, p, b, last), c->U, c->U, bs));
            MMF_CUDA(download_band(b, bs));
        }
    }
    for (int b = 0; b < K; ++b) MMF_CUDA(cudaStreamWaitEvent(c->stream, c->ev_dn[b], 0));
    MMF_CUDA(cudaMemcpyAsync(c->h_ctrl, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->copy_stream));
    if (t_out) *t_out = c->h_ctrl->t;
    if (c->h_ctrl->status) return fail(MMF_ERR_STATE, "non-physical state (negative density/pressure or NaN)");
    return MMF_OK;
}

// Per-step log (the reference's "Ideal dt ... (maxEig = ...)", "Using dt",
// "Current time" lines, main.cpp:399-404): a device ring of 'capacity' steps
// written by the stage-3 bookkeeping; capacity 0 switches it off.
int mmf_set_step_log(mmf_ctx *c, int64_t capacity)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (capacity < 0) return fail(MMF_ERR_ARG, "capacity < 0");
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(c->steplog);
    c->steplog = nullptr;
    c->steplog_cap = 0;
    if (capacity > 0) {
        MMF_CUDA(cudaMalloc(&c->steplog, sizeof(double) * 3 * (size_t)capacity));
        c->steplog_cap = capacity;
    }
    Ctrl h;
    MMF_CUDA(cudaMemcpyAsync(&h, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    h.log = c->steplog;
    h.log_cap = c->steplog_cap;
    MMF_CUDA(cudaMemcpyAsync(c->ctrl, &h, sizeof(Ctrl), cudaMemcpyHostToDevice, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

int mmf_get_step_log(mmf_ctx *c, double *out, int64_t max_entries, int64_t *first_step, int64_t *n_entries)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!out || max_entries < 0 || !first_step || !n_entries) return fail(MMF_ERR_ARG, "bad arguments");
    Ctrl h;
    MMF_CUDA(cudaMemcpyAsync(&h, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    const long long avail = c->steplog ? std::min<long long>(h.step, c->steplog_cap) : 0;
    const long long n = std::min<long long>(avail, max_entries);
    std::vector<double> ring((size_t)(3 * c->steplog_cap));
    if (n > 0)
        MMF_CUDA(cudaMemcpy(ring.data(), c->steplog, sizeof(double) * ring.size(), cudaMemcpyDeviceToHost));
    const long long first = h.step - n;
    for (long long i = 0; i < n; ++i) {
        const long long slot = (first + i) % c->steplog_cap;
        for (int k = 0; k < 3; ++k) out[3 * i + k] = ring[(size_t)(3 * slot + k)];
    }
    *first_step = first;
    *n_entries = n;
    return MMF_OK;
}

// Chooses the decomposition (2D: rows per marching chunk and warps per block;
// 3D: planes per chunk) by timing a few steps of each candidate from the
// current state; the state and the time control are restored afterwards.
// Every decomposition gives the same bits (each cell's arithmetic is fixed
// and maxEig is a max), so only the speed changes.
int mmf_autotune(mmf_ctx *c, int trial_steps, int *chunk_out, int *warps_out)
{
    NvtxRange range_("mmf_autotune");
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->time_ready) return fail(MMF_ERR_ARG, "mmf_time_setup first");
    if (trial_steps < 1) trial_steps = 4;
    const size_t bytes = sizeof(double) * NF * (size_t)c->gp.plane;
    Ctrl saved;
    MMF_CUDA(cudaMemcpyAsync(c->aos, c->U, bytes, cudaMemcpyDeviceToDevice, c->stream));
    MMF_CUDA(cudaMemcpyAsync(&saved, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    Ctrl trial = saved;
    trial.t_end = HUGE_VAL;
    trial.max_steps = LLONG_MAX;
    trial.log = nullptr;   // the trial steps are not steps of the run
    std::vector<std::pair<int, int>> cand;
    if (c->gp.dim == 2) {
        for (int ch : {8, 12, 16, 20, 24, 28, 30, 32, 40, 48, 64})
            for (int w : {1, 2, 4}) cand.emplace_back(ch, w);
    } else {
        // order 1: both 3D kernels (second = 1: tile kernel, one block per
        // tile and chunk; 2: tile kernel, at most one block per resident
        // slot); order 2: row blocks
        for (int ch : {4, 6, 8, 12, 14, 16, 24, 32, 64}) {
            cand.emplace_back(ch, 0);
            if (c->grid.order == 1) cand.emplace_back(ch, 1);
        }
        if (c->grid.order == 1)
            for (int ch : {8, 16, 32, 64, 128}) cand.emplace_back(ch, 2);
    }
    const int by = c->grid.order == 2 ? BY3D_O2 : BY3D;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    MMF_CUDA(cudaEventCreate(&e0));
    MMF_CUDA(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    cudaError_t e = cudaSuccess;
    const bool d2 = c->gp.dim == 2;
    std::pair<int, int> best(c->gp.chunk, d2 ? c->gp.wpb : c->gp.tile3d);
    for (const auto &cd : cand) {
        plan_cartesian(c->gp, cd.first, by, d2 ? cd.second : 0, d2 ? 0 : cd.second, c->grid.order);
        e = cudaMemcpyAsync(c->U, c->aos, bytes, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->ctrl, &trial, sizeof(Ctrl), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = c->rk_step();
        if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
        for (int s = 0; s < trial_steps && e == cudaSuccess; ++s) e = c->rk_step();
        if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) break;
        if (ms < best_ms) { best_ms = ms; best = cd; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    plan_cartesian(c->gp, best.first, by, d2 ? best.second : 0, d2 ? 0 : best.second, c->grid.order);
    if (c->graph_many) { cudaGraphExecDestroy(c->graph_many); c->graph_many = nullptr; }
    if (c->graph_one) { cudaGraphExecDestroy(c->graph_one); c->graph_one = nullptr; }
    MMF_CUDA(e);
    MMF_CUDA(cudaMemcpyAsync(c->U, c->aos, bytes, cudaMemcpyDeviceToDevice, c->stream));
    MMF_CUDA(cudaMemcpyAsync(c->ctrl, &saved, sizeof(Ctrl), cudaMemcpyHostToDevice, c->stream));
    c->indicator_restart();
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    if (chunk_out) *chunk_out = c->gp.chunk;
    if (warps_out) *warps_out = d2 ? c->gp.wpb : -c->gp.tile3d;
    return MMF_OK;
}

int mmf_set_shape(mmf_ctx *c, int chunk, int variant)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (chunk < 1) return fail(MMF_ERR_ARG, "chunk must be >= 1");
    const bool d2 = c->gp.dim == 2;
    if (d2 && (variant < 1 || variant > WARPS_2D)) return fail(MMF_ERR_ARG, "2D: warps per block must be 1..4");
    if (!d2 && (variant < 0 || variant > 2))
        return fail(MMF_ERR_ARG, "3D: variant must be 0 (row blocks), 1 (tiles, one block per tile and chunk) or "
                                 "2 (tiles, one block per resident slot)");
    if (!d2 && variant >= 1 && c->grid.order != 1) return fail(MMF_ERR_UNSUPPORTED, "the 3D tile kernel is order 1");
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    plan_cartesian(c->gp, chunk, c->grid.order == 2 ? BY3D_O2 : BY3D, d2 ? variant : 0, d2 ? 0 : variant,
                   c->grid.order);
    if (c->graph_many) { cudaGraphExecDestroy(c->graph_many); c->graph_many = nullptr; }
    if (c->graph_one) { cudaGraphExecDestroy(c->graph_one); c->graph_one = nullptr; }
    return MMF_OK;
}

int mmf_advance_host(mmf_ctx *c, double *aos, int64_t n_raw, int64_t n_steps, double *t_out)
{
    NvtxRange range_("mmf_advance_host");
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!aos || n_raw != c->gp.plane) return fail(MMF_ERR_ARG, "bad state buffer");
    if (!c->time_ready) return fail(MMF_ERR_ARG, "mmf_time_setup first");
    if (n_steps < 0) return fail(MMF_ERR_ARG, "n_steps < 0");
    if (pipeline_applies(c, aos, n_steps)) return advance_host_pipelined(c, aos, n_steps, t_out);
    rc = mmf_upload_state(c, aos, n_raw);
    if (rc) return rc;
    int64_t done = 0;
    rc = mmf_advance(c, n_steps, t_out, &done);
    if (rc && rc != MMF_ERR_STATE) return rc;
    int rc2 = mmf_download_state(c, aos, n_raw);
    return rc ? rc : rc2;
}

int mmf_rk_stage(mmf_ctx *c, int stage)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!c->time_ready) return fail(MMF_ERR_ARG, "mmf_time_setup first");
    if (c->grid.order == 2) {
        cudaError_t e2 = cudaSuccess;
        switch (stage) {
        case 1:
            e2 = c->o2(O2_SLOPES, STAGE_1, c->U, nullptr, c->lim_active);
            if (e2 == cudaSuccess) e2 = c->o2(O2_STAGE, STAGE_1, c->U, c->R, nullptr);
            break;
        case 2:
            e2 = c->o2(O2_FORM_W1, STAGE_2, c->U, c->W, nullptr);
            if (e2 == cudaSuccess) e2 = c->o2(O2_SLOPES, STAGE_2, c->W, nullptr, nullptr);
            if (e2 == cudaSuccess) e2 = c->o2(O2_STAGE, STAGE_2, c->W, c->R, nullptr);
            break;
        case 3:
            e2 = c->o2(O2_SLOPES, STAGE_3, c->R, nullptr, nullptr);
            if (e2 == cudaSuccess) e2 = c->o2(O2_STAGE, STAGE_3, c->R, c->U, nullptr);
            break;
        default: return fail(MMF_ERR_ARG, "stage must be 1, 2 or 3");
        }
        if (e2 != cudaSuccess) return fail(MMF_ERR_CUDA, cudaGetErrorString(e2));
        return MMF_OK;
    }
    cudaError_t e;
    switch (stage) {
    case 1: e = c->stage(STAGE_1, c->U, c->R); break;
    case 2: e = c->stage(STAGE_2, c->U, c->W); break;
    case 3: e = c->stage(STAGE_3, c->U, c->U); break;
    default: return fail(MMF_ERR_ARG, "stage must be 1, 2 or 3");
    }
    if (e != cudaSuccess) return fail(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}

int mmf_last_step_info(mmf_ctx *c, double *dt, double *max_eig)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    Ctrl h;
    MMF_CUDA(cudaMemcpyAsync(&h, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    if (dt) *dt = h.dt;
    if (max_eig) *max_eig = h.last_maxeig;
    return MMF_OK;
}

int mmf_get_status(mmf_ctx *c, unsigned *status)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    Ctrl h;
    MMF_CUDA(cudaMemcpyAsync(&h, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    if (status) *status = h.status;
    const unsigned zero = 0;
    MMF_CUDA(cudaMemcpyAsync((char *)c->ctrl + offsetof(Ctrl, status), &zero, sizeof(unsigned),
                             cudaMemcpyHostToDevice, c->stream));
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

int mmf_synchronize(mmf_ctx *c)
{
    int rc = check_ctx(c);
    if (rc) return rc;
    MMF_CUDA(cudaStreamSynchronize(c->stream));
    return MMF_OK;
}

// ---- unit-level functions ------------------------------------------------

static int pointwise(int op, int64_t n, const double *a, const double *b, const double *nrm, int bc,
                     const double *dir_prim, double *out, double *out2)
{
    if (n < 0) return fail(MMF_ERR_ARG, "n < 0");
    if (n == 0) return MMF_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(MMF_ERR_CUDA, "no CUDA device available");
    const size_t s5 = sizeof(double) * NF * (size_t)n, s3 = sizeof(double) * 3 * (size_t)n;
    double *da = nullptr, *db = nullptr, *dn = nullptr, *dp = nullptr, *dout = nullptr, *dout2 = nullptr;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&da, s5);
    if (e == cudaSuccess && b) e = cudaMalloc(&db, s5);
    if (e == cudaSuccess && nrm) e = cudaMalloc(&dn, s3);
    if (e == cudaSuccess && dir_prim) e = cudaMalloc(&dp, sizeof(double) * NF);
    if (e == cudaSuccess) e = cudaMalloc(&dout, s5);
    if (e == cudaSuccess && out2) e = cudaMalloc(&dout2, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(da, a, s5, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && b) e = cudaMemcpyAsync(db, b, s5, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nrm) e = cudaMemcpyAsync(dn, nrm, s3, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && dir_prim) e = cudaMemcpyAsync(dp, dir_prim, sizeof(double) * NF, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_pointwise_exact(op, n, da, db, dn, bc, dp, dout, dout2, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, s5, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && out2) e = cudaMemcpyAsync(out2, dout2, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(da); cudaFree(db); cudaFree(dn); cudaFree(dp); cudaFree(dout); cudaFree(dout2);
    if (s) cudaStreamDestroy(s);
    if (e != cudaSuccess) return fail(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}

int mmf_cons2prim(int64_t n, const double *cons, double *prim)
{
    if (!cons || !prim) return fail(MMF_ERR_ARG, "null buffer");
    return pointwise(OP_CONS2PRIM, n, cons, nullptr, nullptr, 0, nullptr, prim, nullptr);
}

int mmf_prim2cons(int64_t n, const double *prim, double *cons)
{
    if (!cons || !prim) return fail(MMF_ERR_ARG, "null buffer");
    return pointwise(OP_PRIM2CONS, n, prim, nullptr, nullptr, 0, nullptr, cons, nullptr);
}

int mmf_eval_fluxes(int64_t n, const double *cons, const double *prim, const double *normal, double *flux)
{
    if (!cons || !prim || !normal || !flux) return fail(MMF_ERR_ARG, "null buffer");
    return pointwise(OP_FLUXES, n, cons, prim, normal, 0, nullptr, flux, nullptr);
}

int mmf_eval_splitting(int64_t n, const double *cons_l, const double *cons_r, const double *normal, double *flux,
                       double *lambda)
{
    if (!cons_l || !cons_r || !normal || !flux || !lambda) return fail(MMF_ERR_ARG, "null buffer");
    return pointwise(OP_SPLITTING, n, cons_l, cons_r, normal, 0, nullptr, flux, lambda);
}

int mmf_eval_bc_values(int64_t n, int bc_type, const double *normal, const double *cons,
                       const double *dirichlet_prim, double *cons_bc)
{
    if (!normal || !cons || !cons_bc) return fail(MMF_ERR_ARG, "null buffer");
    if (bc_type != MMF_BC_FREE_FLOW && bc_type != MMF_BC_REFLECTING && bc_type != MMF_BC_WALL &&
        bc_type != MMF_BC_DIRICHLET)
        return fail(MMF_ERR_ARG, "unknown border condition");
    if (bc_type == MMF_BC_DIRICHLET && !dirichlet_prim) return fail(MMF_ERR_ARG, "Dirichlet needs a state");
    return pointwise(OP_BC, n, cons, nullptr, normal, bc_type, dirichlet_prim, cons_bc, nullptr);
}

int mmf_newton_selftest(int64_t n, const double *x, double *rcp, double *sqrt_out)
{
    if (!x || !rcp || !sqrt_out || n < 0) return fail(MMF_ERR_ARG, "bad buffers");
    if (n == 0) return MMF_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(MMF_ERR_CUDA, "no CUDA device available");
    const size_t b = sizeof(double) * (size_t)n;
    double *dx = nullptr, *dr = nullptr, *dq = nullptr;
    cudaError_t e = cudaMalloc(&dx, b);
    if (e == cudaSuccess) e = cudaMalloc(&dr, b);
    if (e == cudaSuccess) e = cudaMalloc(&dq, b);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, b, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_newton_selftest(n, dx, dr, dq, 0);
    if (e == cudaSuccess) e = cudaMemcpy(rcp, dr, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(sqrt_out, dq, b, cudaMemcpyDeviceToHost);
    cudaFree(dx); cudaFree(dr); cudaFree(dq);
    if (e != cudaSuccess) return fail(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}

int mmf_o2_screen_selftest(int arith, int nv, int dim, int64_t n, const double *uc, const double *sig, int *dec,
                           unsigned char *ref)
{
    if (!uc || !sig || !dec || !ref || n < 0) return fail(MMF_ERR_ARG, "bad buffers");
    if ((dim != 2 && dim != 3) || (nv != 4 && nv != 5) || (nv == 4 && (dim != 2 || arith != MMF_ARITH_FAST)) ||
        (arith != MMF_ARITH_FAST && arith != MMF_ARITH_REFERENCE))
        return fail(MMF_ERR_ARG, "unsupported arithmetic / field count / dimension");
    if (n == 0) return MMF_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(MMF_ERR_CUDA, "no CUDA device available");
    const size_t bu = sizeof(double) * (size_t)n * nv, bs = bu * dim;
    double *du = nullptr, *ds = nullptr;
    int *dd = nullptr;
    unsigned char *dr = nullptr;
    cudaError_t e = cudaMalloc(&du, bu);
    if (e == cudaSuccess) e = cudaMalloc(&ds, bs);
    if (e == cudaSuccess) e = cudaMalloc(&dd, sizeof(int) * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&dr, (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(du, uc, bu, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ds, sig, bs, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = arith == MMF_ARITH_FAST ? launch_screen_selftest_fast(nv, dim, n, du, ds, dd, dr, 0)
                                    : launch_screen_selftest_exact(dim, n, du, ds, dd, dr, 0);
    if (e == cudaSuccess) e = cudaMemcpy(dec, dd, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ref, dr, (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(du); cudaFree(ds); cudaFree(dd); cudaFree(dr);
    if (e != cudaSuccess) return fail(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}

} // extern "C"

int mmf::refresh_w_zero(mmf_ctx *c) { return refresh_w_zero_impl(c); }
