// mmf_umesh.cu -- C ABI of the face-list solver (mmf_umesh_*): contexts built
// from MeshGeometricalInfo-like arrays, the residual entry point and the
// CUDA-graph SSP-RK3 loop.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mmf_gb300.h"
#include "mmf_umesh.cuh"
#include "mmf_nvtx.h"

namespace mmf {
int set_last_error(int code, const char *msg);
}
using namespace mmf;

#define UM_CUDA(call)                                                                                    \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return set_last_error(MMF_ERR_CUDA, (std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
    } while (0)

namespace {

constexpr int GRAPH_STEPS = 16;

__global__ void um_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, long long n)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
#pragma unroll
    for (int k = 0; k < NF; ++k) soa[k * n + r] = aos[NF * r + k];
}

__global__ void um_soa_to_aos(const double *__restrict__ soa, double *__restrict__ aos, long long n)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
#pragma unroll
    for (int k = 0; k < NF; ++k) aos[NF * r + k] = soa[k * n + r];
}

inline unsigned grid_for(long long n)
{
    const long long b = (n + 255) / 256;
    return (unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}

} // namespace

struct mmf_umesh {
    int device = 0;
    cudaStream_t stream = nullptr;
    int arith = MMF_ARITH_REFERENCE;
    UMesh m;
    double min_size = 0.0;
    // device arrays
    double *vol = nullptr, *area = nullptr, *normal = nullptr;
    double *inv_vol = nullptr;   // fast arithmetic: 1 / volume per cell
    unsigned char *solved = nullptr;
    long long *owner = nullptr, *neigh = nullptr, *csr_off = nullptr, *csr_face = nullptr;
    int *bc = nullptr;
    double *U = nullptr, *R = nullptr, *W = nullptr, *P = nullptr, *S = nullptr, *aos = nullptr;
    double *rec = nullptr;    // fast arithmetic: 6 record planes
    Ctrl *ctrl = nullptr;
    double *rhs_maxeig = nullptr;
    cudaGraphExec_t g_many = nullptr, g_one = nullptr;
    long long launches = 0;
    bool time_ready = false;

    template <int STAGE>
    cudaError_t face(const double *state)
    {
        ++launches;
        if (arith == MMF_ARITH_FAST && STAGE != STAGE_RHS) {
            urec_kernel<<<grid_for(m.ncells), 256, 0, stream>>>(m, state, ctrl, STAGE);
            ++launches;
            uface_kernel<FastArith, STAGE><<<grid_for(m.nfaces), 256, 0, stream>>>(m, state, P, ctrl, rhs_maxeig);
        } else {
            uface_kernel<ExactArith, STAGE><<<grid_for(m.nfaces), 256, 0, stream>>>(m, state, P, ctrl, rhs_maxeig);
        }
        return cudaPeekAtLastError();
    }
    template <int STAGE>
    cudaError_t cell(const double *state, double *out)
    {
        ++launches;
        if (arith == MMF_ARITH_FAST && STAGE != STAGE_RHS)
            ucell_kernel<FastArith, STAGE><<<grid_for(m.ncells), 256, 0, stream>>>(m, P, U, state, out, ctrl);
        else
            ucell_kernel<ExactArith, STAGE><<<grid_for(m.ncells), 256, 0, stream>>>(m, P, U, state, out, ctrl);
        return cudaPeekAtLastError();
    }
    // face (+ record) and cell kernels of three stages and the W1 kernel
    int launches_per_step() const { return arith == MMF_ARITH_FAST ? 10 : 7; }
    cudaError_t rk_step()
    {
        cudaError_t e;
        if ((e = face<STAGE_1>(U)) != cudaSuccess) return e;
        if ((e = cell<STAGE_1>(U, R)) != cudaSuccess) return e;
        ++launches;
        if (arith == MMF_ARITH_FAST) uform_w1_kernel<FastArith><<<grid_for(m.ncells), 256, 0, stream>>>(m, U, R, W, ctrl);
        else uform_w1_kernel<ExactArith><<<grid_for(m.ncells), 256, 0, stream>>>(m, U, R, W, ctrl);
        if ((e = cudaPeekAtLastError()) != cudaSuccess) return e;
        if ((e = face<STAGE_2>(W)) != cudaSuccess) return e;
        if ((e = cell<STAGE_2>(W, R)) != cudaSuccess) return e;       // R := W2
        if ((e = face<STAGE_3>(R)) != cudaSuccess) return e;
        return cell<STAGE_3>(R, U);
    }
};

static int um_graph(mmf_umesh *u, int steps, cudaGraphExec_t *exec)
{
    cudaGraph_t g = nullptr;
    UM_CUDA(cudaStreamBeginCapture(u->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t err = cudaSuccess;
    const long long before = u->launches;
    for (int s = 0; s < steps && err == cudaSuccess; ++s) err = u->rk_step();
    u->launches = before;
    cudaError_t e2 = cudaStreamEndCapture(u->stream, &g);
    if (err != cudaSuccess) { if (g) cudaGraphDestroy(g); return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(err)); }
    if (e2 != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e2));
    cudaError_t e3 = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e3));
    return MMF_OK;
}

static int um_check(mmf_umesh *u)
{
    if (!u) return set_last_error(MMF_ERR_ARG, "null context");
    cudaError_t e = cudaSetDevice(u->device);
    if (e != cudaSuccess) return set_last_error(MMF_ERR_CUDA, cudaGetErrorString(e));
    return MMF_OK;
}

extern "C" {

int mmf_umesh_create(const mmf_umesh_desc *d, int device, mmf_umesh **out)
{
    if (!d || !out) return set_last_error(MMF_ERR_ARG, "null argument");
    *out = nullptr;
    if (d->n_cells < 1 || d->n_faces < 1) return set_last_error(MMF_ERR_ARG, "empty mesh");
    if (!d->cell_volume || !d->cell_size || !d->owner || !d->neigh || !d->area || !d->normal || !d->bc)
        return set_last_error(MMF_ERR_ARG, "missing mesh arrays");
    if (d->arith != MMF_ARITH_REFERENCE && d->arith != MMF_ARITH_FAST) return set_last_error(MMF_ERR_ARG, "unknown arithmetic");
    const long long n = d->n_cells, nf = d->n_faces;
    // validate topology, build the cell -> faces lists in face order
    std::vector<long long> off((size_t)n + 1, 0);
    for (long long f = 0; f < nf; ++f) {
        const long long o = d->owner[f], nb = d->neigh[f];
        if (o < 0 || o >= n || nb >= n) return set_last_error(MMF_ERR_ARG, "face references a cell out of range");
        if (nb < 0 && d->bc[f] == MMF_BC_NONE) return set_last_error(MMF_ERR_ARG, "border face without a border condition");
        off[(size_t)o + 1]++;
        if (nb >= 0) off[(size_t)nb + 1]++;
    }
    for (long long c = 0; c < n; ++c) off[(size_t)c + 1] += off[(size_t)c];
    std::vector<long long> fill(off.begin(), off.end() - 1), csr((size_t)off[(size_t)n]);
    for (long long f = 0; f < nf; ++f) {
        csr[(size_t)fill[(size_t)d->owner[f]]++] = -f - 1;
        if (d->neigh[f] >= 0) csr[(size_t)fill[(size_t)d->neigh[f]]++] = f;
    }
    std::vector<double> nrm((size_t)(3 * nf));
    for (long long f = 0; f < nf; ++f)
        for (int q = 0; q < 3; ++q) nrm[(size_t)(q * nf + f)] = d->normal[3 * f + q];
    std::vector<unsigned char> solved((size_t)n, 1);
    if (d->solved) for (long long c = 0; c < n; ++c) solved[(size_t)c] = d->solved[c] ? 1 : 0;
    double min_size = INFINITY;
    for (long long c = 0; c < n; ++c) min_size = std::fmin(d->cell_size[c], min_size);   // main.cpp:351-356
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return set_last_error(MMF_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= ndev) return set_last_error(MMF_ERR_ARG, "device index out of range");
    UM_CUDA(cudaSetDevice(device));
    mmf_umesh *u = new mmf_umesh();
    u->device = device;
    u->arith = d->arith;
    u->min_size = min_size;
    const size_t sb = sizeof(double) * NF * (size_t)n;
    cudaError_t e = cudaStreamCreateWithFlags(&u->stream, cudaStreamNonBlocking);
    auto A = [&](void **p, size_t b) { if (e == cudaSuccess) e = cudaMalloc(p, b); };
    A((void **)&u->vol, sizeof(double) * n);
    A((void **)&u->solved, (size_t)n);
    A((void **)&u->owner, sizeof(long long) * nf);
    A((void **)&u->neigh, sizeof(long long) * nf);
    A((void **)&u->area, sizeof(double) * nf);
    A((void **)&u->normal, sizeof(double) * 3 * nf);
    A((void **)&u->bc, sizeof(int) * nf);
    A((void **)&u->csr_off, sizeof(long long) * (n + 1));
    A((void **)&u->csr_face, sizeof(long long) * csr.size());
    A((void **)&u->U, sb);
    A((void **)&u->R, sb);
    A((void **)&u->W, sb);
    A((void **)&u->S, sb);
    A((void **)&u->aos, sb);
    A((void **)&u->P, sizeof(double) * NF * nf);
    std::vector<double> inv_vol;
    if (d->arith == MMF_ARITH_FAST) {
        A((void **)&u->rec, sizeof(double) * 6 * n);
        A((void **)&u->inv_vol, sizeof(double) * n);
        inv_vol.resize(n);
        for (long long c = 0; c < n; ++c) inv_vol[c] = 1.0 / d->cell_volume[c];
    }
    A((void **)&u->ctrl, sizeof(Ctrl));
    A((void **)&u->rhs_maxeig, sizeof(double));
    auto H = [&](void *dst, const void *src, size_t b) { if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, u->stream); };
    H(u->vol, d->cell_volume, sizeof(double) * n);
    if (d->arith == MMF_ARITH_FAST) H(u->inv_vol, inv_vol.data(), sizeof(double) * n);
    H(u->solved, solved.data(), (size_t)n);
    H(u->owner, d->owner, sizeof(long long) * nf);
    H(u->neigh, d->neigh, sizeof(long long) * nf);
    H(u->area, d->area, sizeof(double) * nf);
    H(u->normal, nrm.data(), sizeof(double) * 3 * nf);
    H(u->bc, d->bc, sizeof(int) * nf);
    H(u->csr_off, off.data(), sizeof(long long) * (n + 1));
    H(u->csr_face, csr.data(), sizeof(long long) * csr.size());
    if (e == cudaSuccess) e = cudaMemsetAsync(u->U, 0, sb, u->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(u->W, 0, sb, u->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(u->ctrl, 0, sizeof(Ctrl), u->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(u->stream);
    if (e != cudaSuccess) {
        std::string msg = cudaGetErrorString(e);
        mmf_umesh_destroy(u);
        return set_last_error(MMF_ERR_CUDA, msg.c_str());
    }
    UMesh &m = u->m;
    m.ncells = n;
    m.nfaces = nf;
    m.vol = u->vol;
    m.inv_vol = u->inv_vol;
    m.solved = u->solved;
    m.owner = u->owner;
    m.neigh = u->neigh;
    m.area = u->area;
    m.normal = u->normal;
    m.bc = u->bc;
    m.csr_off = u->csr_off;
    m.csr_face = u->csr_face;
    m.rec = u->rec;
    dirichlet_conservatives(d->dirichlet_prim, m.dir_cons);
    *out = u;
    return MMF_OK;
}

int mmf_umesh_destroy(mmf_umesh *u)
{
    if (!u) return MMF_OK;
    cudaSetDevice(u->device);
    if (u->stream) cudaStreamSynchronize(u->stream);
    if (u->g_many) cudaGraphExecDestroy(u->g_many);
    if (u->g_one) cudaGraphExecDestroy(u->g_one);
    cudaFree(u->vol); cudaFree(u->solved); cudaFree(u->owner); cudaFree(u->neigh); cudaFree(u->area);
    cudaFree(u->normal); cudaFree(u->bc); cudaFree(u->csr_off); cudaFree(u->csr_face);
    cudaFree(u->U); cudaFree(u->R); cudaFree(u->W); cudaFree(u->S); cudaFree(u->aos); cudaFree(u->P);
    cudaFree(u->ctrl); cudaFree(u->rhs_maxeig); cudaFree(u->rec); cudaFree(u->inv_vol);
    if (u->stream) cudaStreamDestroy(u->stream);
    delete u;
    return MMF_OK;
}

int64_t mmf_umesh_launch_count(const mmf_umesh *u) { return u ? u->launches : 0; }

int mmf_umesh_upload(mmf_umesh *u, const double *aos, int64_t n)
{
    int rc = um_check(u);
    if (rc) return rc;
    if (!aos || n != u->m.ncells) return set_last_error(MMF_ERR_ARG, "bad state buffer");
    UM_CUDA(cudaMemcpyAsync(u->aos, aos, sizeof(double) * NF * (size_t)n, cudaMemcpyHostToDevice, u->stream));
    um_aos_to_soa<<<(unsigned)((n + 255) / 256), 256, 0, u->stream>>>(u->aos, u->U, n);
    ++u->launches;
    UM_CUDA(cudaPeekAtLastError());
    return MMF_OK;
}

int mmf_umesh_download(mmf_umesh *u, double *aos, int64_t n)
{
    int rc = um_check(u);
    if (rc) return rc;
    if (!aos || n != u->m.ncells) return set_last_error(MMF_ERR_ARG, "bad state buffer");
    um_soa_to_aos<<<(unsigned)((n + 255) / 256), 256, 0, u->stream>>>(u->U, u->aos, n);
    ++u->launches;
    UM_CUDA(cudaPeekAtLastError());
    UM_CUDA(cudaMemcpyAsync(aos, u->aos, sizeof(double) * NF * (size_t)n, cudaMemcpyDeviceToHost, u->stream));
    UM_CUDA(cudaStreamSynchronize(u->stream));
    return MMF_OK;
}

int mmf_umesh_compute_rhs(mmf_umesh *u, const double *cons, double *rhs, double *max_eig, int64_t n)
{
    NvtxRange range_("mmf_umesh_compute_rhs");
    int rc = um_check(u);
    if (rc) return rc;
    if (!cons || !rhs || n != u->m.ncells) return set_last_error(MMF_ERR_ARG, "bad buffers");
    const size_t b = sizeof(double) * NF * (size_t)n;
    UM_CUDA(cudaMemcpyAsync(u->aos, cons, b, cudaMemcpyHostToDevice, u->stream));
    um_aos_to_soa<<<(unsigned)((n + 255) / 256), 256, 0, u->stream>>>(u->aos, u->S, n);
    ++u->launches;
    UM_CUDA(cudaMemsetAsync(u->rhs_maxeig, 0, sizeof(double), u->stream));
    UM_CUDA(u->face<STAGE_RHS>(u->S));
    UM_CUDA(u->cell<STAGE_RHS>(u->S, u->R));
    um_soa_to_aos<<<(unsigned)((n + 255) / 256), 256, 0, u->stream>>>(u->R, u->aos, n);
    ++u->launches;
    UM_CUDA(cudaPeekAtLastError());
    UM_CUDA(cudaMemcpyAsync(rhs, u->aos, b, cudaMemcpyDeviceToHost, u->stream));
    double me = 0.0;
    UM_CUDA(cudaMemcpyAsync(&me, u->rhs_maxeig, sizeof(double), cudaMemcpyDeviceToHost, u->stream));
    UM_CUDA(cudaStreamSynchronize(u->stream));
    if (max_eig) *max_eig = me;
    return MMF_OK;
}

int mmf_umesh_time_setup(mmf_umesh *u, double cfl, double t, double t_end, int64_t max_steps)
{
    int rc = um_check(u);
    if (rc) return rc;
    if (!(cfl > 0.0)) return set_last_error(MMF_ERR_ARG, "CFL must be > 0");
    if (std::isinf(t_end) && max_steps < 0) return set_last_error(MMF_ERR_ARG, "infinite end time needs max_steps");
    Ctrl h;
    memset(&h, 0, sizeof(h));
    h.t = t;
    h.t_end = t_end;
    h.cfl_h = 0.9 * cfl * u->min_size;
    h.max_steps = (max_steps < 0) ? LLONG_MAX : max_steps;
    UM_CUDA(cudaMemcpyAsync(u->ctrl, &h, sizeof(Ctrl), cudaMemcpyHostToDevice, u->stream));
    UM_CUDA(cudaStreamSynchronize(u->stream));
    u->time_ready = true;
    return MMF_OK;
}

int mmf_umesh_advance(mmf_umesh *u, int64_t n_steps, double *t_out, int64_t *steps_done)
{
    NvtxRange range_("mmf_umesh_advance");
    int rc = um_check(u);
    if (rc) return rc;
    if (!u->time_ready) return set_last_error(MMF_ERR_ARG, "mmf_umesh_time_setup first");
    if (!u->g_many && (rc = um_graph(u, GRAPH_STEPS, &u->g_many))) return rc;
    if (!u->g_one && (rc = um_graph(u, 1, &u->g_one))) return rc;
    // rounds of at most CHECK_STEPS steps, stopping once the run has ended
    constexpr int64_t CHECK_STEPS = 64 * GRAPH_STEPS;
    Ctrl before, after;
    UM_CUDA(cudaMemcpyAsync(&before, u->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, u->stream));
    int64_t left = n_steps;
    for (;;) {
        int64_t round = left < CHECK_STEPS ? left : CHECK_STEPS;
        left -= round;
        while (round >= GRAPH_STEPS) {
            UM_CUDA(cudaGraphLaunch(u->g_many, u->stream));
            u->launches += u->launches_per_step() * GRAPH_STEPS;
            round -= GRAPH_STEPS;
        }
        while (round-- > 0) {
            UM_CUDA(cudaGraphLaunch(u->g_one, u->stream));
            u->launches += u->launches_per_step();
        }
        UM_CUDA(cudaMemcpyAsync(&after, u->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, u->stream));
        UM_CUDA(cudaStreamSynchronize(u->stream));
        if (left == 0 || !(after.t < after.t_end && after.step < after.max_steps) || after.status) break;
    }
    if (t_out) *t_out = after.t;
    if (steps_done) *steps_done = after.step - before.step;
    if (after.status) return set_last_error(MMF_ERR_STATE, "non-physical state (negative density/pressure or NaN)");
    return MMF_OK;
}

} // extern "C"
