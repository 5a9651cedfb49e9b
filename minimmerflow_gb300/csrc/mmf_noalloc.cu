// mmf_noalloc.cu -- euler::computeRHS for callers that cannot allocate device
// memory: code running while another library captures a CUDA graph on its
// stream (a cudaMalloc there would break the capture), real-time step loops
// that cannot afford the device-wide synchronisation an allocation implies,
// and processes whose device memory is already reserved by a pool allocator.
//
// The entry point takes device pointers for its inputs and outputs and keeps
// its working set -- the structure-of-arrays copy of the state, the residual
// planes and the max-eigenvalue slot -- in one file-scope device array of
// 2 * 5 * MMF_NOALLOC_MAX_CELLS + 32 doubles (about 5.2 MB), which every GPU
// that loads this library holds until the process exits.  No cudaMalloc,
// cudaFree or allocating library routine is called.
//
// In host code the array's name is only a host-side stand-in, not a device
// address, so the entry point asks the runtime for the device address with
// cudaGetSymbolAddress once per device (with that device current, on the
// first call made on it) and passes that address to the kernels.  That first
// call should therefore come before any stream capture.
//
// Every call shares the array and finds the previous call's contents in it:
// the max-eigenvalue slot is cleared at the start of each call, and the state
// and residual planes are fully rewritten.  Calls that overlap on the GPU
// (on different streams, or from different threads) race on the array.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/mmf_gb300.h"
#include "mmf_launch.cuh"

namespace mmf {
int set_last_error(int code, const char *msg);   // mmf_capi.cu
}

using namespace mmf;

namespace {

constexpr long long kMaxCells = MMF_NOALLOC_MAX_CELLS;
constexpr long long kSlot = 2LL * NF * kMaxCells;       // max-eigenvalue slot (256-byte aligned offset)
static __device__ __align__(256) double g_noalloc_scratch[2 * NF * MMF_NOALLOC_MAX_CELLS + 32];

constexpr int kMaxDevices = 64;
double *g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

__global__ void noalloc_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, long long n,
                                   const long long *__restrict__ raw_to_cell)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    if (g < 0 || g >= n) return;
#pragma unroll
    for (int k = 0; k < NF; ++k) soa[k * n + g] = aos[NF * r + k];
}

__global__ void noalloc_soa_to_aos(const double *__restrict__ soa, double *__restrict__ aos, long long n,
                                   const long long *__restrict__ raw_to_cell)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    if (g < 0 || g >= n) return;
#pragma unroll
    for (int k = 0; k < NF; ++k) aos[NF * r + k] = soa[k * n + g];
}

// Device address of the scratch array on the current device (set up once).
int scratch_of_current_device(double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_last_error(MMF_ERR_UNSUPPORTED, "device index above 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_last_error(MMF_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[dev];
    return MMF_OK;
}

} // namespace

extern "C" int mmf_compute_rhs_noalloc(const mmf_grid *grid, const double *d_cons, double *d_rhs,
                                       double *d_max_eig, const int64_t *d_raw_to_cell, void *stream)
{
    if (!grid || !d_cons || !d_rhs || !d_max_eig) return set_last_error(MMF_ERR_ARG, "null argument");
    if (grid->dim != 2 && grid->dim != 3) return set_last_error(MMF_ERR_ARG, "dim must be 2 or 3");
    if (grid->order != 1) return set_last_error(MMF_ERR_UNSUPPORTED, "only order 1 is supported");
    if (!(grid->h > 0.0)) return set_last_error(MMF_ERR_ARG, "h must be > 0");
    long long n = 1;
    for (int d = 0; d < grid->dim; ++d) {
        if (grid->n[d] < 1) return set_last_error(MMF_ERR_ARG, "cells per direction must be >= 1");
        if ((grid->bc_lo[d] == MMF_BC_PERIODIC) != (grid->bc_hi[d] == MMF_BC_PERIODIC))
            return set_last_error(MMF_ERR_ARG, "periodic borders must be paired");
        n *= grid->n[d];
    }
    if (n > kMaxCells)
        return set_last_error(MMF_ERR_ARG, "mmf_compute_rhs_noalloc: the mesh has more cells than "
                                           "MMF_NOALLOC_MAX_CELLS (65536)");
    double *scratch = nullptr;
    int rc = scratch_of_current_device(&scratch);
    if (rc) return rc;

    GridParams gp;
    memset(&gp, 0, sizeof(gp));
    gp.dim = grid->dim;
    for (int d = 0; d < 3; ++d) {
        gp.n[d] = (d < grid->dim) ? grid->n[d] : 1;
        gp.bc_lo[d] = (d < grid->dim) ? grid->bc_lo[d] : MMF_BC_FREE_FLOW;
        gp.bc_hi[d] = (d < grid->dim) ? grid->bc_hi[d] : MMF_BC_FREE_FLOW;
    }
    dirichlet_conservatives(grid->dirichlet_prim, gp.dir_cons);
    const double h = grid->h;
    gp.area = (grid->dim == 3) ? h * h : h;
    gp.vol = (grid->dim == 3) ? h * h * h : h * h;
    gp.half_area_per_vol = 0.5 * gp.area / gp.vol;
    plan_cartesian(gp, grid->chunk);

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *state = scratch, *rhs = scratch + NF * kMaxCells, *me = scratch + kSlot;
    const long long *map = reinterpret_cast<const long long *>(d_raw_to_cell);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    cudaError_t e = cudaMemsetAsync(me, 0, sizeof(double), s);
    if (e == cudaSuccess) {
        noalloc_aos_to_soa<<<blocks, 256, 0, s>>>(d_cons, state, n, map);
        e = cudaPeekAtLastError();
    }
    if (e == cudaSuccess) {
        StageArgs sa;
        sa.U = state; sa.R = rhs; sa.W = nullptr; sa.out = rhs; sa.ctrl = nullptr; sa.rhs_maxeig = me;
        e = launch_stage_exact(STAGE_RHS, gp, sa, s);
    }
    if (e == cudaSuccess) {
        noalloc_soa_to_aos<<<blocks, 256, 0, s>>>(rhs, d_rhs, n, map);
        e = cudaPeekAtLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_max_eig, me, sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}
