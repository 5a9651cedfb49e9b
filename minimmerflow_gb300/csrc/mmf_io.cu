// mmf_io.cu -- initial states and the L1 density error on the device
// (problem.cpp:247-392, main.cpp:335-344 and 550-567), VTK output of the
// fields the reference writes (solver_writer.cpp:56-119), and a raw
// checkpoint that restores a run (the reference writes VTK only).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mmf_context.cuh"

namespace mmf {
int set_last_error(int code, const char *msg);
}

#define IO_CUDA(call)                                                                                    \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return set_last_error(MMF_ERR_CUDA, (std::string(#call) + ": " + cudaGetErrorString(e_)).c_str()); \
    } while (0)

namespace {

// problem.cpp:247-392 (exact / initial conservative state at a point)
__device__ void exact_conservatives(const mmf_problem &pr, int dim, const double *origin, double length, double x,
                                    double y, double z, double t, double *c)
{
    double prim[NF] = {0, 0, 0, 0, 0};
    double pt[3] = {x, y, z};
    const int P = pr.problem;
    if (P == MMF_VORTEX_XY || P == MMF_VORTEX_ZX || P == MMF_VORTEX_YZ) {
        double uinf[3] = {1.0, 1.0, 1.0};
        if (P == MMF_VORTEX_XY) uinf[2] = 0.0;
        else if (P == MMF_VORTEX_ZX) uinf[1] = 0.0;
        else uinf[0] = 0.0;
        for (int d = 0; d < 3; ++d) pt[d] -= t * uinf[d];
        if (pr.periodic_exact)
            for (int d = 0; d < dim; ++d) {
                while (pt[d] < origin[d]) pt[d] += length;
                while (pt[d] >= origin[d] + length) pt[d] -= length;
            }
        double csi, eta;
        if (P == MMF_VORTEX_XY) { csi = pt[0]; eta = pt[1]; }
        else if (P == MMF_VORTEX_ZX) { csi = pt[2]; eta = pt[0]; }
        else { csi = pt[1]; eta = pt[2]; }
        const double r = sqrt(csi * csi + eta * eta);
        const double shape = pr.vortex_beta / (2 * M_PI) * exp(0.5 * (1 - r * r));
        double du = 0, dv = 0, dw = 0;
        if (P == MMF_VORTEX_XY) { du = -eta * shape; dv = csi * shape; }
        else if (P == MMF_VORTEX_ZX) { dw = -eta * shape; du = csi * shape; }
        else { dv = -eta * shape; dw = csi * shape; }
        const double dT = -(GAMMA - 1.0) / (2 * GAMMA) * shape * shape;
        const double dp = pow(1.0 + dT, GAMMA / (GAMMA - 1.0)) - 1.0;
        prim[0] = 1.0 + dp;
        prim[1] = uinf[0] + du;
        prim[2] = uinf[1] + dv;
        prim[3] = (dim == 3) ? uinf[2] + dw : 0;
        prim[4] = 1.0 + dT;
    } else if (P == MMF_RADSOD) {
        const double r = sqrt(pt[0] * pt[0] + pt[1] * pt[1] + pt[2] * pt[2]);
        if (r < pr.sod_radius) { prim[0] = pr.sod_p_in; prim[4] = pr.sod_p_in / pr.sod_rho_in; }
        else { prim[0] = pr.sod_p_out; prim[4] = pr.sod_p_out / pr.sod_rho_out; }
    } else if (P == MMF_SOD_X || P == MMF_SOD_Y || P == MMF_SOD_Z) {
        const double r = (P == MMF_SOD_X) ? pt[0] : (P == MMF_SOD_Y) ? pt[1] : pt[2];
        if (r < 0.) { prim[0] = 1.0; prim[4] = 1.0 / 1.0; }
        else { prim[0] = 0.1; prim[4] = 0.1 / 0.125; }
    } else {   // forward-facing step inflow state
        prim[0] = 1.0; prim[1] = 3.0; prim[4] = 1.0 / 1.4;
    }
    ExactArith::prim2cons(prim, c);
}

struct GridGeom {
    int dim;
    int n[3];
    double origin[3];
    double h;
    double length;
};

__device__ __forceinline__ void centroid(const GridGeom &g, long long cell, double *x)
{
    const long long i = cell % g.n[0], j = (cell / g.n[0]) % g.n[1], k = cell / ((long long)g.n[0] * g.n[1]);
    x[0] = g.origin[0] + ((double)i + 0.5) * g.h;
    x[1] = g.origin[1] + ((double)j + 0.5) * g.h;
    x[2] = (g.dim == 3) ? g.origin[2] + ((double)k + 0.5) * g.h : g.origin[2];
}

__global__ void init_kernel(GridGeom g, mmf_problem pr, double *U, long long n)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double x[3], v[NF];
        centroid(g, c, x);
        exact_conservatives(pr, g.dim, g.origin, g.length, x[0], x[1], x[2], 0.0, v);
        for (int k = 0; k < NF; ++k) U[k * n + c] = v[k];
    }
}

// per-block partial sums of |rho - rho_exact(t)| V (second pass adds them on the host)
__global__ void error_kernel(GridGeom g, mmf_problem pr, const double *U, long long n, double t, double vol,
                             double *partial)
{
    __shared__ double red[256];
    double s = 0.0;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double x[3], v[NF];
        centroid(g, c, x);
        exact_conservatives(pr, g.dim, g.origin, g.length, x[0], x[1], x[2], t, v);
        s += fabs(U[c] - v[0]) * vol;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// primitive fields for output: rho, u, v, w, p, T (6 planes)
__global__ void prim_kernel(const double *U, double *P, long long n)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double cc[NF], pp[NF];
        for (int k = 0; k < NF; ++k) cc[k] = U[k * n + c];
        ExactArith::cons2prim(cc, pp);
        P[c] = cc[0];
        P[n + c] = pp[1];
        P[2 * n + c] = pp[2];
        P[3 * n + c] = pp[3];
        P[4 * n + c] = pp[0];
        P[5 * n + c] = pp[4];
    }
}

GridGeom geom_of(const mmf_ctx *c)
{
    GridGeom g;
    g.dim = c->grid.dim;
    for (int d = 0; d < 3; ++d) { g.n[d] = c->gp.n[d]; g.origin[d] = c->grid.origin[d]; }
    g.h = c->grid.h;
    g.length = c->grid.h * c->grid.n[0];
    return g;
}

constexpr uint64_t CKPT_MAGIC = 0x3230504b43464d4dull;   // "MMFCKP02"

} // namespace

extern "C" {

int mmf_init_state(mmf_ctx *c, const mmf_problem *pr)
{
    if (!c || !pr) return set_last_error(MMF_ERR_ARG, "null argument");
    IO_CUDA(cudaSetDevice(c->device));
    const long long n = c->gp.plane;
    init_kernel<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, c->stream>>>(geom_of(c), *pr, c->U, n);
    ++c->launches;
    IO_CUDA(cudaPeekAtLastError());
    IO_CUDA(cudaStreamSynchronize(c->stream));
    return refresh_w_zero(c);
}

int mmf_l1_density_error(mmf_ctx *c, const mmf_problem *pr, double t, double *error)
{
    if (!c || !pr || !error) return set_last_error(MMF_ERR_ARG, "null argument");
    IO_CUDA(cudaSetDevice(c->device));
    const long long n = c->gp.plane;
    const int blocks = 1024;
    double *partial = nullptr;
    IO_CUDA(cudaMalloc(&partial, sizeof(double) * blocks));
    const double vol = (c->grid.dim == 3) ? c->grid.h * c->grid.h * c->grid.h : c->grid.h * c->grid.h;
    error_kernel<<<blocks, 256, 0, c->stream>>>(geom_of(c), *pr, c->U, n, t, vol, partial);
    ++c->launches;
    std::vector<double> h(blocks);
    cudaError_t e = cudaPeekAtLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), partial, sizeof(double) * blocks, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(partial);
    IO_CUDA(e);
    double s = 0.0;
    for (double v : h) s += v;
    *error = s;
    return MMF_OK;
}

int mmf_write_vtk(mmf_ctx *c, const char *path)
{
    if (!c || !path) return set_last_error(MMF_ERR_ARG, "null argument");
    IO_CUDA(cudaSetDevice(c->device));
    const long long n = c->gp.plane;
    // planes 0-5: rho, u, v, w, p, T; planes 6-10: the residual of the state
    // (reference arithmetic, the computeRHS of the context's order)
    double *P = nullptr;
    IO_CUDA(cudaMalloc(&P, sizeof(double) * 11 * n));
    prim_kernel<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, c->stream>>>(c->U, P, n);
    ++c->launches;
    cudaError_t e = cudaPeekAtLastError();
    if (e == cudaSuccess) {
        if (c->grid.order == 2) {
            e = c->o2(O2_SLOPES, STAGE_RHS, c->U, nullptr, nullptr);
            if (e == cudaSuccess) e = c->o2(O2_STAGE, STAGE_RHS, c->U, P + 6 * n, nullptr);
        } else {
            StageArgs sa;
            sa.U = c->U; sa.R = c->R; sa.W = c->W; sa.out = P + 6 * n; sa.ctrl = c->ctrl;
            sa.rhs_maxeig = c->rhs_maxeig;
            ++c->launches;
            e = launch_stage_exact(STAGE_RHS, c->gp, sa, c->stream);
        }
    }
    std::vector<double> h((size_t)(11 * n));
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), P, sizeof(double) * 11 * n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(P);
    IO_CUDA(e);
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return set_last_error(MMF_ERR_ARG, "cannot open the output file");
    // VTK XML ImageData, raw appended data (little endian, 64-bit block headers)
    const bool d3 = c->grid.dim == 3;
    const int nx = c->gp.n[0], ny = c->gp.n[1], nz = d3 ? c->gp.n[2] : 0;
    const double h0 = c->grid.h;
    const uint64_t sb = sizeof(double) * (uint64_t)n, vb = 3 * sb, ib = sizeof(int32_t) * (uint64_t)n;
    std::fprintf(fp, "<?xml version=\"1.0\"?>\n<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" "
                     "header_type=\"UInt64\">\n<ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"%.17g %.17g %.17g\" "
                     "Spacing=\"%.17g %.17g %.17g\">\n<Piece Extent=\"0 %d 0 %d 0 %d\">\n<CellData>\n",
                 nx, ny, nz, c->grid.origin[0], c->grid.origin[1], c->grid.origin[2], h0, h0, d3 ? h0 : 1.0, nx, ny, nz);
    // the fields of the reference's writer, in its order (main.cpp:289-298)
    struct Field { const char *name; int plane; int comps; };
    const Field fields[] = {{"solved", -1, 1},      {"velocity", 1, 3},   {"pressure", 4, 1},
                            {"temperature", 5, 1},  {"density", 0, 1},    {"residualC", 6, 1},
                            {"residualMX", 7, 1},   {"residualMY", 8, 1}, {"residualMZ", 9, 1},
                            {"residualE", 10, 1}};
    uint64_t off = 0;
    for (const Field &f : fields) {
        if (f.plane < 0)
            std::fprintf(fp, "<DataArray type=\"Int32\" Name=\"%s\" format=\"appended\" offset=\"%llu\"/>\n", f.name,
                         (unsigned long long)off);
        else
            std::fprintf(fp, "<DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"%d\" format=\"appended\" "
                             "offset=\"%llu\"/>\n", f.name, f.comps, (unsigned long long)off);
        off += 8 + (f.plane < 0 ? ib : f.comps == 3 ? vb : sb);
    }
    std::fprintf(fp, "</CellData>\n</Piece>\n</ImageData>\n<AppendedData encoding=\"raw\">\n_");
    for (const Field &f : fields) {
        if (f.plane < 0) {
            std::vector<int32_t> solved((size_t)n, 1);   // every cell of a Cartesian context is solved
            std::fwrite(&ib, 8, 1, fp);
            std::fwrite(solved.data(), sizeof(int32_t), (size_t)n, fp);
        } else if (f.comps == 3) {
            std::vector<double> vel((size_t)(3 * n));
            for (long long i = 0; i < n; ++i)
                for (int q = 0; q < 3; ++q) vel[(size_t)(3 * i + q)] = h[(size_t)((f.plane + q) * n + i)];
            std::fwrite(&vb, 8, 1, fp);
            std::fwrite(vel.data(), sizeof(double), (size_t)(3 * n), fp);
        } else {
            std::fwrite(&sb, 8, 1, fp);
            std::fwrite(h.data() + (size_t)f.plane * n, sizeof(double), (size_t)n, fp);
        }
    }
    std::fprintf(fp, "\n</AppendedData>\n</VTKFile>\n");
    const bool ok = std::ferror(fp) == 0;
    std::fclose(fp);
    if (!ok) return set_last_error(MMF_ERR_ARG, "write error");
    return MMF_OK;
}

int mmf_save_checkpoint(mmf_ctx *c, const char *path)
{
    if (!c || !path) return set_last_error(MMF_ERR_ARG, "null argument");
    IO_CUDA(cudaSetDevice(c->device));
    const long long n = c->gp.plane;
    std::vector<double> u((size_t)(NF * n));
    Ctrl h;
    IO_CUDA(cudaMemcpyAsync(u.data(), c->U, sizeof(double) * NF * n, cudaMemcpyDeviceToHost, c->stream));
    IO_CUDA(cudaMemcpyAsync(&h, c->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream));
    IO_CUDA(cudaStreamSynchronize(c->stream));
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return set_last_error(MMF_ERR_ARG, "cannot open the checkpoint file");
    const int64_t hdr[6] = {(int64_t)CKPT_MAGIC, c->grid.dim, c->gp.n[0], c->gp.n[1], c->gp.n[2], NF};
    std::fwrite(hdr, sizeof(hdr), 1, fp);
    std::fwrite(&h, sizeof(Ctrl), 1, fp);
    std::fwrite(u.data(), sizeof(double), u.size(), fp);
    const bool ok = std::ferror(fp) == 0;
    std::fclose(fp);
    if (!ok) return set_last_error(MMF_ERR_ARG, "write error");
    return MMF_OK;
}

int mmf_load_checkpoint(mmf_ctx *c, const char *path)
{
    if (!c || !path) return set_last_error(MMF_ERR_ARG, "null argument");
    IO_CUDA(cudaSetDevice(c->device));
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return set_last_error(MMF_ERR_ARG, "cannot open the checkpoint file");
    int64_t hdr[6];
    Ctrl h;
    const long long n = c->gp.plane;
    std::vector<double> u((size_t)(NF * n));
    bool ok = std::fread(hdr, sizeof(hdr), 1, fp) == 1 && hdr[0] == (int64_t)CKPT_MAGIC && hdr[1] == c->grid.dim &&
              hdr[2] == c->gp.n[0] && hdr[3] == c->gp.n[1] && hdr[4] == c->gp.n[2] && hdr[5] == NF &&
              std::fread(&h, sizeof(Ctrl), 1, fp) == 1 && std::fread(u.data(), sizeof(double), u.size(), fp) == u.size();
    std::fclose(fp);
    if (!ok) return set_last_error(MMF_ERR_ARG, "checkpoint does not match this context");
    h.log = c->steplog;          // the log of this context, not the one of the saved run
    h.log_cap = c->steplog_cap;
    IO_CUDA(cudaMemcpyAsync(c->U, u.data(), sizeof(double) * NF * n, cudaMemcpyHostToDevice, c->stream));
    IO_CUDA(cudaMemcpyAsync(c->ctrl, &h, sizeof(Ctrl), cudaMemcpyHostToDevice, c->stream));
    IO_CUDA(cudaStreamSynchronize(c->stream));
    c->time_ready = true;
    return refresh_w_zero(c);
}

} // extern "C"
