// mmf_noalloc.cu -- euler::computeRHS for callers that cannot allocate device
// memory: code running while another library captures a CUDA graph on its
// stream (a cudaMalloc there would break the capture), real-time step loops
// that cannot afford the device-wide synchronisation an allocation implies,
// and processes whose device memory is already reserved by a pool allocator.
//
// The entry point takes device pointers for its inputs and outputs and keeps
// its working set -- the structure-of-arrays copy of the state, the residual
// planes, a slot block (max eigenvalue, cell-map error count) and one counter
// per cell for the check of the cell map -- in one file-scope device array of
// 2 * 5 * MMF_NOALLOC_MAX_CELLS + 32 + MMF_NOALLOC_MAX_CELLS / 2 doubles
// (about 5.5 MB), which every GPU that loads this library holds until the
// process exits.  No cudaMalloc, cudaFree or allocating library routine is
// called.
//
// In host code the array's name is only a host-side stand-in, not a device
// address, so the entry point asks the runtime for the device address with
// cudaGetSymbolAddress once per device (with that device current, on the
// first call made on it) and passes that address to the kernels.  That first
// call should therefore come before any stream capture.
//
// Every call shares the array and finds the previous call's contents in it:
// the slot block and the per-cell counters are cleared at the start of each
// call, and the state and residual planes are fully rewritten when the cell
// map is a permutation.  When it is not (an entry out of range, a cell named
// twice, a cell never named), some state rows would keep the previous call's
// values, so the call writes NaN to every residual row and to the max
// eigenvalue instead of a result.  Calls that overlap on the GPU (on
// different streams, or from different threads) race on the array.
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
constexpr long long kSlot = 2LL * NF * kMaxCells;       // slot block (256-byte aligned offset)
constexpr long long kCount = kSlot + 32;                 // per-cell counters (int), 256-byte aligned
static __device__ __align__(256) double g_noalloc_scratch[2 * NF * MMF_NOALLOC_MAX_CELLS + 32 +
                                                          MMF_NOALLOC_MAX_CELLS / 2];

constexpr int kMaxDevices = 64;
double *g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mutex;

// AoS raw rows -> SoA grid cells.  With a map, each grid cell's counter
// counts the raw rows that name it, and entries out of [0, n) count as
// errors (and are not followed).
__global__ void noalloc_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, long long n,
                                   const long long *__restrict__ raw_to_cell, int *count,
                                   unsigned long long *map_err)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    if (g < 0 || g >= n) {
        atomicAdd(map_err, 1ull);
        return;
    }
    if (raw_to_cell) atomicAdd(count + g, 1);
#pragma unroll
    for (int k = 0; k < NF; ++k) soa[k * n + g] = aos[NF * r + k];
}

// The map is a permutation when every grid cell was named exactly once.
__global__ void noalloc_check_map(const int *__restrict__ count, long long n, unsigned long long *map_err)
{
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g < n && count[g] != 1) atomicAdd(map_err, 1ull);
}

// SoA residual -> AoS raw rows, and the max eigenvalue.  A map that was not
// a permutation leaves NaN everywhere (rows of cells never named would hold
// the previous call's state, so no row can be trusted).
__global__ void noalloc_soa_to_aos(const double *__restrict__ soa, double *__restrict__ aos, long long n,
                                   const long long *__restrict__ raw_to_cell,
                                   const unsigned long long *__restrict__ map_err, const double *__restrict__ me,
                                   double *max_eig)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool bad = *map_err != 0ull;
    if (r == 0) *max_eig = bad ? __longlong_as_double(0x7ff8000000000000ll) : *me;
    if (r >= n) return;
    const long long g = raw_to_cell ? raw_to_cell[r] : r;
    if (bad || g < 0 || g >= n) {
#pragma unroll
        for (int k = 0; k < NF; ++k) aos[NF * r + k] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
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

namespace mmf {
int check_grid(const mmf_grid *grid);   // mmf_capi.cu
}

extern "C" int mmf_compute_rhs_noalloc(const mmf_grid *grid, const double *d_cons, double *d_rhs,
                                       double *d_max_eig, const int64_t *d_raw_to_cell, void *stream)
{
    if (!grid || !d_cons || !d_rhs || !d_max_eig) return set_last_error(MMF_ERR_ARG, "null argument");
    int rc = mmf::check_grid(grid);
    if (rc) return rc;
    if (grid->order != 1) return set_last_error(MMF_ERR_UNSUPPORTED, "only order 1 is supported");
    if (grid->arith != MMF_ARITH_REFERENCE)
        return set_last_error(MMF_ERR_UNSUPPORTED, "only the reference arithmetic is supported");
    long long n = 1;
    for (int d = 0; d < grid->dim; ++d) {
        n *= grid->n[d];   // n <= 65536 before, n[d] < 2^31: no overflow
        if (n > kMaxCells)
            return set_last_error(MMF_ERR_ARG, "mmf_compute_rhs_noalloc: the mesh has more cells than "
                                               "MMF_NOALLOC_MAX_CELLS (65536)");
    }
    double *scratch = nullptr;
    rc = scratch_of_current_device(&scratch);
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
    unsigned long long *map_err = reinterpret_cast<unsigned long long *>(scratch + kSlot + 1);
    int *count = reinterpret_cast<int *>(scratch + kCount);
    const long long *map = reinterpret_cast<const long long *>(d_raw_to_cell);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    // the max-eigenvalue slot and the map error count start at zero
    cudaError_t e = cudaMemsetAsync(me, 0, 32 * sizeof(double), s);
    if (e == cudaSuccess && map) e = cudaMemsetAsync(count, 0, sizeof(int) * n, s);
    if (e == cudaSuccess) {
        noalloc_aos_to_soa<<<blocks, 256, 0, s>>>(d_cons, state, n, map, count, map_err);
        e = cudaPeekAtLastError();
    }
    if (e == cudaSuccess && map) {
        noalloc_check_map<<<blocks, 256, 0, s>>>(count, n, map_err);
        e = cudaPeekAtLastError();
    }
    if (e == cudaSuccess) {
        StageArgs sa;
        sa.U = state; sa.R = rhs; sa.W = nullptr; sa.out = rhs; sa.ctrl = nullptr; sa.rhs_maxeig = me;
        e = launch_stage_exact(STAGE_RHS, gp, sa, s);
    }
    if (e == cudaSuccess) {
        noalloc_soa_to_aos<<<blocks, 256, 0, s>>>(rhs, d_rhs, n, map, map_err, me, d_max_eig);
        e = cudaPeekAtLastError();
    }
    if (e != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}
