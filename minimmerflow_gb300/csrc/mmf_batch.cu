// mmf_batch.cu -- C ABI of the batched solver (many independent 2D cases in
// one persistent launch per RK stage, CUDA-graph replay) and its autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/mmf_gb300.h"
#include "mmf_batch.cuh"
#include "mmf_launch.cuh"
#include "mmf_nvtx.h"

namespace mmf {
int set_last_error(int code, const char *msg);
cudaError_t mlp_indicator_batch(mmf_mlp *p, const CaseDesc *cases, const long long *offsets, int ncases,
                                long long total, const double *U, float thr, unsigned char *flags, cudaStream_t s,
                                float *Q, unsigned char *raw, IndicatorStep is);
int mlp_dim(const mmf_mlp *p);
}
using namespace mmf;

namespace {

#define BATCH_CUDA(call)                                                                               \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return set_last_error(MMF_ERR_CUDA, (std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
    } while (0)

constexpr int GRAPH_STEPS = 16;

__global__ void batch_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, long long n)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
#pragma unroll
    for (int k = 0; k < NF; ++k) soa[k * n + r] = aos[NF * r + k];
}

__global__ void batch_soa_to_aos(const double *__restrict__ soa, double *__restrict__ aos, long long n)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
#pragma unroll
    for (int k = 0; k < NF; ++k) aos[NF * r + k] = soa[k * n + r];
}

__global__ void batch_nonzero(const double *__restrict__ v, long long n, int *flag)
{
    bool nz = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        nz |= (mmf::dbits(v[i]) << 1) != 0;
    if (__any_sync(0xffffffffu, nz) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// tuned (chunk, blocks per SM) by workload signature
std::mutex g_tune_mutex;
std::map<std::tuple<int, long long, int, int>, std::pair<int, int>> g_tuned;

} // namespace

struct mmf_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    int arith = MMF_ARITH_FAST;
    bool w_zero = false;
    int ncases = 0;
    long long total = 0;
    std::vector<mmf_grid> grids;
    std::vector<long long> offsets;
    CaseDesc *cases = nullptr;
    int *item_case = nullptr;
    int nitems = 0;
    int chunk = 32;
    int blocks_per_sm = 0;     // 0 = occupancy maximum
    int blocks = 0;
    int slope_blocks = 0;      // the slope kernel's own grid (its occupancy maximum)
    int sms = 0;
    double *U = nullptr, *R = nullptr, *W = nullptr, *aos = nullptr;
    Ctrl *ctrl = nullptr;
    int *flag = nullptr;
    cudaGraphExec_t g_many = nullptr, g_one = nullptr;
    long long launches = 0;
    bool time_ready = false;
    // order 2
    int order = 1;
    double *S = nullptr;
    unsigned char *lim_flag = nullptr, *lim_active = nullptr;
    int limit_mode = LIMIT_ALL;
    long long *d_offsets = nullptr;
    mmf_mlp *indicator = nullptr;
    float ind_threshold = 0.5f;
    float *ind_q = nullptr;   // the indicator's FP32 primitive planes (5 x total)
    int ind_period = 1;                 // the indicator runs every ind_period steps (1 or 2)
    int *ind_tick = nullptr;            // device step counter of the period
    unsigned char *ind_raw = nullptr;   // the network's flags before the dilation (period 2)

    // the next step runs the indicator (after a change of the state or of the time control)
    void indicator_restart()
    {
        if (ind_tick) cudaMemsetAsync(ind_tick, 0, sizeof(int), stream);
    }

    void drop_graphs()
    {
        if (g_many) { cudaGraphExecDestroy(g_many); g_many = nullptr; }
        if (g_one) { cudaGraphExecDestroy(g_one); g_one = nullptr; }
    }

    cudaError_t stage(int st, double *out)
    {
        StageArgs base;
        base.U = U; base.R = R; base.W = W; base.out = out; base.ctrl = nullptr; base.rhs_maxeig = nullptr;
        ++launches;
        return arith == MMF_ARITH_FAST
                   ? launch_batch_fast(st, cases, item_case, nitems, ctrl, base, blocks, stream, w_zero)
                   : launch_batch_exact(st, cases, item_case, nitems, ctrl, base, blocks, stream);
    }
    cudaError_t o2(int op, int st, const double *state, double *out)
    {
        StageArgs base;
        base.U = U; base.R = R; base.W = W; base.out = out; base.ctrl = nullptr; base.rhs_maxeig = nullptr;
        O2Batch ob;
        ob.S = S; ob.flag = lim_flag; ob.active = (op == BO2_SLOPES && st == STAGE_1) ? lim_active : nullptr;
        ob.limit_mode = limit_mode;
        // a step's stage-1 slopes advance the indicator's step counter
        ob.tick = (op == BO2_SLOPES && st == STAGE_1 && indicator && ind_period > 1) ? ind_tick : nullptr;
        ++launches;
        return arith == MMF_ARITH_FAST
                   ? launch_batch_o2_fast(op, st, cases, item_case, nitems, ctrl, base, state, ob, W,
                                          op == BO2_SLOPES ? slope_blocks : blocks, stream, w_zero)
                   : launch_batch_o2_exact(op, st, cases, item_case, nitems, ctrl, base, state, ob, W,
                                           op == BO2_SLOPES ? slope_blocks : blocks, stream);
    }
    cudaError_t rk_step()
    {
        cudaError_t e;
        if (order == 2) {
            if (indicator) {
                launches += ind_period > 1 ? 3 : 2;   // primitives, features + MLP (, dilation)
                if ((e = mlp_indicator_batch(indicator, cases, d_offsets, ncases, total, U, ind_threshold, lim_flag,
                                             stream, ind_q, ind_period > 1 ? ind_raw : nullptr,
                                             IndicatorStep{ind_period, ind_tick})) != cudaSuccess)
                    return e;
            }
            if ((e = o2(BO2_SLOPES, STAGE_1, U, nullptr)) != cudaSuccess) return e;
            if ((e = o2(BO2_STAGE, STAGE_1, U, R)) != cudaSuccess) return e;
            if ((e = o2(BO2_FORM_W1, STAGE_2, U, W)) != cudaSuccess) return e;
            if ((e = o2(BO2_SLOPES, STAGE_2, W, nullptr)) != cudaSuccess) return e;
            if ((e = o2(BO2_STAGE, STAGE_2, W, R)) != cudaSuccess) return e;
            if ((e = o2(BO2_SLOPES, STAGE_3, R, nullptr)) != cudaSuccess) return e;
            return o2(BO2_STAGE, STAGE_3, R, U);
        }
        if ((e = stage(STAGE_1, R)) != cudaSuccess) return e;
        if ((e = stage(STAGE_2, W)) != cudaSuccess) return e;
        return stage(STAGE_3, U);
    }
    int launches_per_step() const { return order == 2 ? (indicator ? (ind_period > 1 ? 10 : 9) : 7) : 3; }
};

static int batch_plan(mmf_batch *b, int chunk, int blocks_per_sm)
{
    std::vector<CaseDesc> hc((size_t)b->ncases);
    std::vector<int> item_case;
    for (int c = 0; c < b->ncases; ++c) {
        const mmf_grid &g = b->grids[(size_t)c];
        GridParams &gp = hc[(size_t)c].gp;
        memset(&gp, 0, sizeof(gp));
        gp.dim = 2;
        for (int d = 0; d < 3; ++d) {
            gp.n[d] = (d < 2) ? g.n[d] : 1;
            gp.bc_lo[d] = (d < 2) ? g.bc_lo[d] : MMF_BC_FREE_FLOW;
            gp.bc_hi[d] = (d < 2) ? g.bc_hi[d] : MMF_BC_FREE_FLOW;
        }
        dirichlet_conservatives(g.dirichlet_prim, gp.dir_cons);
        gp.area = g.h;
        gp.vol = g.h * g.h;
        gp.half_area_per_vol = 0.5 * gp.area / gp.vol;
        plan_cartesian(gp, chunk);
        gp.plane = b->total;
        hc[(size_t)c].offset = b->offsets[(size_t)c];
        hc[(size_t)c].item0 = (int)item_case.size();
        const int items = gp.nseg * gp.nchunk;
        for (int i = 0; i < items; ++i) item_case.push_back(c);
    }
    cudaFree(b->cases);
    cudaFree(b->item_case);
    b->cases = nullptr;
    b->item_case = nullptr;
    BATCH_CUDA(cudaMalloc(&b->cases, sizeof(CaseDesc) * hc.size()));
    BATCH_CUDA(cudaMalloc(&b->item_case, sizeof(int) * item_case.size()));
    BATCH_CUDA(cudaMemcpyAsync(b->cases, hc.data(), sizeof(CaseDesc) * hc.size(), cudaMemcpyHostToDevice, b->stream));
    BATCH_CUDA(cudaMemcpyAsync(b->item_case, item_case.data(), sizeof(int) * item_case.size(), cudaMemcpyHostToDevice,
                               b->stream));
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    b->nitems = (int)item_case.size();
    b->chunk = chunk;
    const int maxb = batch_max_blocks_per_sm(b->arith, b->w_zero, b->order);
    b->blocks_per_sm = (blocks_per_sm > 0) ? std::min(blocks_per_sm, maxb) : maxb;
    b->blocks = b->sms * b->blocks_per_sm;
    b->slope_blocks = b->sms * batch_slope_blocks_per_sm(b->arith, b->w_zero);
    b->drop_graphs();
    return MMF_OK;
}

static int batch_graph(mmf_batch *b, int steps, cudaGraphExec_t *exec)
{
    cudaGraph_t g = nullptr;
    BATCH_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    const long long before = b->launches;
    for (int s = 0; s < steps && err == cudaSuccess; ++s) err = b->rk_step();
    b->launches = before;
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (err != cudaSuccess) { if (g) cudaGraphDestroy(g); return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(err)); }
    if (e2 != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e2));
    cudaError_t e3 = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e3));
    return MMF_OK;
}

static int batch_check(mmf_batch *b)
{
    if (!b) return set_last_error(MMF_ERR_ARG, "null batch");
    cudaError_t e = cudaSetDevice(b->device);
    if (e != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}

static int batch_enqueue(mmf_batch *b, int64_t n_steps)
{
    int rc;
    if (!b->g_many && (rc = batch_graph(b, GRAPH_STEPS, &b->g_many))) return rc;
    if (!b->g_one && (rc = batch_graph(b, 1, &b->g_one))) return rc;
    int64_t left = n_steps;
    while (left >= GRAPH_STEPS) {
        BATCH_CUDA(cudaGraphLaunch(b->g_many, b->stream));
        b->launches += b->launches_per_step() * GRAPH_STEPS;
        left -= GRAPH_STEPS;
    }
    while (left-- > 0) {
        BATCH_CUDA(cudaGraphLaunch(b->g_one, b->stream));
        b->launches += b->launches_per_step();
    }
    return MMF_OK;
}

extern "C" {

int mmf_batch_create(int ncases, const mmf_grid *grids, int device, mmf_batch **out)
{
    if (!grids || !out || ncases < 1) return set_last_error(MMF_ERR_ARG, "bad arguments");
    *out = nullptr;
    const int arith = grids[0].arith;
    long long total = 0;
    std::vector<long long> offsets((size_t)ncases);
    for (int c = 0; c < ncases; ++c) {
        const mmf_grid &g = grids[c];
        if (g.dim != 2) return set_last_error(MMF_ERR_UNSUPPORTED, "batched cases are 2D");
        if (g.order != 1 && g.order != 2) return set_last_error(MMF_ERR_UNSUPPORTED, "order must be 1 or 2");
        if (g.order != grids[0].order) return set_last_error(MMF_ERR_ARG, "all cases need the same order");
        if (g.arith != arith) return set_last_error(MMF_ERR_ARG, "all cases need the same arithmetic");
        if (arith != MMF_ARITH_REFERENCE && arith != MMF_ARITH_FAST) return set_last_error(MMF_ERR_ARG, "unknown arithmetic");
        if (!(g.h > 0.0) || g.n[0] < 1 || g.n[1] < 1) return set_last_error(MMF_ERR_ARG, "bad grid");
        for (int d = 0; d < 2; ++d)
            if ((g.bc_lo[d] == MMF_BC_PERIODIC) != (g.bc_hi[d] == MMF_BC_PERIODIC))
                return set_last_error(MMF_ERR_ARG, "periodic borders must be paired");
        offsets[(size_t)c] = total;
        total += (long long)g.n[0] * g.n[1];
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return set_last_error(MMF_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev) return set_last_error(MMF_ERR_ARG, "device index out of range");
    BATCH_CUDA(cudaSetDevice(device));
    mmf_batch *b = new mmf_batch();
    b->device = device;
    b->arith = arith;
    b->ncases = ncases;
    b->total = total;
    b->grids.assign(grids, grids + ncases);
    b->offsets = offsets;
    b->order = grids[0].order;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    b->sms = (e == cudaSuccess) ? prop.multiProcessorCount : 1;
    const size_t bytes = sizeof(double) * NF * (size_t)total;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&b->U, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->R, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->W, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->aos, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&b->ctrl, sizeof(Ctrl) * ncases);
    if (e == cudaSuccess) e = cudaMalloc(&b->flag, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->U, 0, bytes, b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->ctrl, 0, sizeof(Ctrl) * ncases, b->stream);
    if (e == cudaSuccess && b->order == 2) {
        e = cudaMalloc(&b->S, bytes * 2);
        if (e == cudaSuccess) e = cudaMalloc(&b->lim_flag, (size_t)total);
        if (e == cudaSuccess) e = cudaMalloc(&b->lim_active, (size_t)total);
        if (e == cudaSuccess) e = cudaMalloc(&b->d_offsets, sizeof(long long) * (ncases + 1));
        if (e == cudaSuccess) e = cudaMemsetAsync(b->lim_flag, 0, (size_t)total, b->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(b->lim_active, 0, (size_t)total, b->stream);
        std::vector<long long> offs(offsets);
        offs.push_back(total);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b->d_offsets, offs.data(), sizeof(long long) * offs.size(), cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    }
    if (e != cudaSuccess) {
        std::string msg = cudaGetErrorString(e);
        mmf_batch_destroy(b);
        return set_last_error(e == cudaErrorMemoryAllocation ? MMF_ERR_NOMEM : MMF_ERR_CUDA, msg.c_str());
    }
    int rc = batch_plan(b, 32, 0);
    if (rc) { mmf_batch_destroy(b); return rc; }
    *out = b;
    return MMF_OK;
}

int mmf_batch_destroy(mmf_batch *b)
{
    if (!b) return MMF_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->drop_graphs();
    cudaFree(b->U); cudaFree(b->R); cudaFree(b->W); cudaFree(b->aos); cudaFree(b->ctrl); cudaFree(b->flag);
    cudaFree(b->cases); cudaFree(b->item_case);
    cudaFree(b->S); cudaFree(b->lim_flag); cudaFree(b->lim_active); cudaFree(b->d_offsets); cudaFree(b->ind_q);
    cudaFree(b->ind_raw); cudaFree(b->ind_tick);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MMF_OK;
}

int64_t mmf_batch_cell_count(const mmf_batch *b) { return b ? b->total : 0; }
int64_t mmf_batch_launch_count(const mmf_batch *b) { return b ? b->launches : 0; }
void *mmf_batch_get_stream(mmf_batch *b) { return b ? (void *)b->stream : nullptr; }

int mmf_batch_upload(mmf_batch *b, const double *aos, int64_t total)
{
    int rc = batch_check(b);
    if (rc) return rc;
    if (!aos || total != b->total) return set_last_error(MMF_ERR_ARG, "bad state buffer");
    const size_t bytes = sizeof(double) * NF * (size_t)total;
    BATCH_CUDA(cudaMemcpyAsync(b->aos, aos, bytes, cudaMemcpyHostToDevice, b->stream));
    b->indicator_restart();
    batch_aos_to_soa<<<(unsigned)((total + 255) / 256), 256, 0, b->stream>>>(b->aos, b->U, total);
    ++b->launches;
    BATCH_CUDA(cudaPeekAtLastError());
    bool wz = false;
    if (b->arith == MMF_ARITH_FAST) {
        BATCH_CUDA(cudaMemsetAsync(b->flag, 0, sizeof(int), b->stream));
        batch_nonzero<<<1024, 256, 0, b->stream>>>(b->U + 3 * total, total, b->flag);
        ++b->launches;
        BATCH_CUDA(cudaPeekAtLastError());
        int h = 1;
        BATCH_CUDA(cudaMemcpyAsync(&h, b->flag, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        BATCH_CUDA(cudaStreamSynchronize(b->stream));
        wz = (h == 0);
    }
    if (wz != b->w_zero) {
        b->w_zero = wz;
        if ((rc = batch_plan(b, b->chunk, b->blocks_per_sm))) return rc;
    }
    return MMF_OK;
}

int mmf_batch_download(mmf_batch *b, double *aos, int64_t total)
{
    int rc = batch_check(b);
    if (rc) return rc;
    if (!aos || total != b->total) return set_last_error(MMF_ERR_ARG, "bad state buffer");
    batch_soa_to_aos<<<(unsigned)((total + 255) / 256), 256, 0, b->stream>>>(b->U, b->aos, total);
    ++b->launches;
    BATCH_CUDA(cudaPeekAtLastError());
    BATCH_CUDA(cudaMemcpyAsync(aos, b->aos, sizeof(double) * NF * (size_t)total, cudaMemcpyDeviceToHost, b->stream));
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    return MMF_OK;
}

int mmf_batch_time_setup(mmf_batch *b, const double *cfl, const double *t_end, int64_t max_steps)
{
    int rc = batch_check(b);
    if (rc) return rc;
    if (!cfl) return set_last_error(MMF_ERR_ARG, "null CFL array");
    std::vector<Ctrl> h((size_t)b->ncases);
    for (int c = 0; c < b->ncases; ++c) {
        Ctrl &x = h[(size_t)c];
        memset(&x, 0, sizeof(x));
        const double te = t_end ? t_end[c] : INFINITY;
        if (!(cfl[c] > 0.0)) return set_last_error(MMF_ERR_ARG, "CFL must be > 0");
        if (std::isinf(te) && max_steps < 0) return set_last_error(MMF_ERR_ARG, "infinite end time needs max_steps");
        x.t = 0.0;
        x.t_end = te;
        x.cfl_h = 0.9 * cfl[c] * b->grids[(size_t)c].h;
        x.max_steps = (max_steps < 0) ? LLONG_MAX : max_steps;
    }
    BATCH_CUDA(cudaMemcpyAsync(b->ctrl, h.data(), sizeof(Ctrl) * h.size(), cudaMemcpyHostToDevice, b->stream));
    b->indicator_restart();
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    b->time_ready = true;
    return MMF_OK;
}

int mmf_batch_advance_async(mmf_batch *b, int64_t n_steps)
{
    NvtxRange range_("mmf_batch_advance_async");
    int rc = batch_check(b);
    if (rc) return rc;
    if (!b->time_ready) return set_last_error(MMF_ERR_ARG, "mmf_batch_time_setup first");
    if (n_steps < 0) return set_last_error(MMF_ERR_ARG, "n_steps < 0");
    return batch_enqueue(b, n_steps);
}

int mmf_batch_synchronize(mmf_batch *b)
{
    int rc = batch_check(b);
    if (rc) return rc;
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    return MMF_OK;
}

int mmf_batch_case_info(mmf_batch *b, int c, double *t, int64_t *steps, unsigned *status)
{
    int rc = batch_check(b);
    if (rc) return rc;
    if (c < 0 || c >= b->ncases) return set_last_error(MMF_ERR_ARG, "case index out of range");
    Ctrl h;
    BATCH_CUDA(cudaMemcpyAsync(&h, b->ctrl + c, sizeof(Ctrl), cudaMemcpyDeviceToHost, b->stream));
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    if (t) *t = h.t;
    if (steps) *steps = h.step;
    if (status) *status = h.status;
    return MMF_OK;
}

int mmf_batch_set_shape(mmf_batch *b, int chunk, int blocks_per_sm)
{
    int rc = batch_check(b);
    if (rc) return rc;
    if (chunk < 1 || blocks_per_sm < 0) return set_last_error(MMF_ERR_ARG, "bad shape");
    return batch_plan(b, chunk, blocks_per_sm);
}

int mmf_batch_get_shape(mmf_batch *b, int *chunk, int *blocks_per_sm)
{
    if (!b) return set_last_error(MMF_ERR_ARG, "null batch");
    if (chunk) *chunk = b->chunk;
    if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
    return MMF_OK;
}

int mmf_batch_set_limiter(mmf_batch *b, int mode)
{
    int rc = batch_check(b);
    if (rc) return rc;
    if (b->order != 2) return set_last_error(MMF_ERR_UNSUPPORTED, "the limiter applies to order 2");
    if (mode != LIMIT_ALL && mode != LIMIT_NONE && mode != LIMIT_FLAGGED) return set_last_error(MMF_ERR_ARG, "unknown limiter mode");
    b->limit_mode = mode;
    b->drop_graphs();
    return MMF_OK;
}

int mmf_batch_set_indicator(mmf_batch *b, mmf_mlp *mlp, float threshold)
{
    int rc = batch_check(b);
    if (rc) return rc;
    if (b->order != 2) return set_last_error(MMF_ERR_UNSUPPORTED, "the indicator drives the order-2 limiter");
    if (mlp && mlp_dim(mlp) != 2) return set_last_error(MMF_ERR_ARG, "batched cases need a 2D indicator");
    if (mlp && !b->ind_q) {
        const cudaError_t e = cudaMalloc(&b->ind_q, sizeof(float) * 5 * (size_t)b->total);
        if (e != cudaSuccess) return set_last_error(MMF_ERR_NOMEM, cudaGetErrorString(e));
    }
    b->indicator = mlp;
    b->ind_threshold = threshold;
    b->indicator_restart();
    b->limit_mode = mlp ? LIMIT_FLAGGED : LIMIT_ALL;
    b->drop_graphs();
    return MMF_OK;
}

int mmf_batch_set_indicator_period(mmf_batch *b, int period)
{
    int rc = batch_check(b);
    if (rc) return rc;
    if (period != 1 && period != 2) return set_last_error(MMF_ERR_ARG, "the indicator period must be 1 or 2");
    if (b->order != 2) return set_last_error(MMF_ERR_UNSUPPORTED, "the indicator drives the order-2 limiter");
    if (period > 1 && !b->ind_raw) {
        BATCH_CUDA(cudaMalloc(&b->ind_raw, (size_t)b->total));
        BATCH_CUDA(cudaMemsetAsync(b->ind_raw, 0, (size_t)b->total, b->stream));
    }
    if (period > 1 && !b->ind_tick) BATCH_CUDA(cudaMalloc(&b->ind_tick, sizeof(int)));
    b->ind_period = period;
    b->indicator_restart();
    b->drop_graphs();
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    return MMF_OK;
}

int mmf_batch_autotune(mmf_batch *b, int trial_steps, int *chunk_out, int *blocks_per_sm_out)
{
    NvtxRange range_("mmf_batch_autotune");
    int rc = batch_check(b);
    if (rc) return rc;
    if (!b->time_ready) return set_last_error(MMF_ERR_ARG, "mmf_batch_time_setup first");
    if (trial_steps < 1) trial_steps = 4;
    const auto key = std::make_tuple(b->arith * 8 + (b->w_zero ? 1 : 0) + (b->order == 2 ? 2 : 0) + (b->indicator ? 4 : 0),
                                     b->total, b->ncases, b->sms);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            if ((rc = batch_plan(b, it->second.first, it->second.second))) return rc;
            if (chunk_out) *chunk_out = b->chunk;
            if (blocks_per_sm_out) *blocks_per_sm_out = b->blocks_per_sm;
            return MMF_OK;
        }
    }
    // snapshot: the trials advance the state, which is restored afterwards
    const size_t bytes = sizeof(double) * NF * (size_t)b->total;
    std::vector<Ctrl> saved((size_t)b->ncases);
    BATCH_CUDA(cudaMemcpyAsync(b->aos, b->U, bytes, cudaMemcpyDeviceToDevice, b->stream));
    BATCH_CUDA(cudaMemcpyAsync(saved.data(), b->ctrl, sizeof(Ctrl) * saved.size(), cudaMemcpyDeviceToHost, b->stream));
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    const int maxb = batch_max_blocks_per_sm(b->arith, b->w_zero, b->order);
    const int chunks[] = {8, 16, 32, 64};
    std::vector<int> bps;
    for (int v = maxb; v >= 1 && (int)bps.size() < 3; v = v / 2) bps.push_back(v);
    cudaEvent_t e0, e1;
    BATCH_CUDA(cudaEventCreate(&e0));
    BATCH_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_chunk = b->chunk, best_bps = b->blocks_per_sm;
    for (int ch : chunks) {
        for (int bp : bps) {
            if ((rc = batch_plan(b, ch, bp))) break;
            if ((rc = batch_enqueue(b, 1))) break;       // warm-up + graph build
            cudaEventRecord(e0, b->stream);
            if ((rc = batch_enqueue(b, trial_steps))) break;
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) { best = ms; best_chunk = ch; best_bps = bp; }
            // restore the state for the next trial
            cudaMemcpyAsync(b->U, b->aos, bytes, cudaMemcpyDeviceToDevice, b->stream);
            cudaMemcpyAsync(b->ctrl, saved.data(), sizeof(Ctrl) * saved.size(), cudaMemcpyHostToDevice, b->stream);
            cudaStreamSynchronize(b->stream);
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaMemcpyAsync(b->U, b->aos, bytes, cudaMemcpyDeviceToDevice, b->stream);
    cudaMemcpyAsync(b->ctrl, saved.data(), sizeof(Ctrl) * saved.size(), cudaMemcpyHostToDevice, b->stream);
    b->indicator_restart();
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    if (rc) return rc;
    if ((rc = batch_plan(b, best_chunk, best_bps))) return rc;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tuned[key] = std::make_pair(best_chunk, best_bps);
    }
    if (chunk_out) *chunk_out = best_chunk;
    if (blocks_per_sm_out) *blocks_per_sm_out = b->blocks_per_sm;
    return MMF_OK;
}

} // extern "C"
