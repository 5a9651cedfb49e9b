// mmf_umesh.cuh -- the Euler step on a general face list: the structure of
// MeshGeometricalInfo (mesh_info.hpp:31-105) with per-face border conditions
// and per-cell solved flags, i.e. the reference's computeRHS
// (euler.cpp:127-249) on any mesh -- refined octrees, immersed bodies
// (BC_WALL faces between fluid and solid cells, main.cpp:251-277), the
// forward-facing step's Dirichlet / free-flow / reflecting borders.
//
//   urec_kernel    fast arithmetic: the per-cell record (u, v, w, p, sound
//                  speed, rho H) of the stage input, once per cell, so that
//                  the face kernel converts no interior state.
//   uface_kernel   one thread per interface: the face states (order 1: the
//                  cell means; a border or wall face: the ghost of the fluid
//                  side with the normal flipped when the neighbour is the
//                  fluid, euler.cpp:197-226), the LLF flux, P_f = area * F
//                  (5 planes over the faces), the face max eigenvalue.
//   ucell_kernel   one thread per cell: the residual R = sum of -P_f (owner)
//                  and +P_f (neighbour) over the cell's faces in face-list
//                  order (a CSR list built on the host, so the sum is the
//                  reference's, atomic-free), then the stage combination.
//   uform_w1       W1 = U + dt R1 / V materialised for stage 2.
//
// State planes are indexed by raw id; unsolved cells keep their state and get
// no residual, as in the reference.
#pragma once

#include "mmf_cartesian.cuh"

namespace mmf {

struct UMesh {
    long long ncells, nfaces;
    const double *vol;            // per cell
    const double *inv_vol;        // fast arithmetic: 1 / vol per cell (no FP64 division in the kernels)
    const unsigned char *solved;  // per cell
    const long long *owner, *neigh;
    const double *area;           // per face
    const double *normal;         // 3 planes over the faces
    const int *bc;                // per face (BC_NONE interior)
    const long long *csr_off;     // per cell: [off[c], off[c+1]) into csr_face
    const long long *csr_face;    // face index, negated - 1 when the cell is the owner
    double *rec;                  // fast arithmetic: per-cell record, 6 planes (u, v, w, p, a, rho H)
    double dir_cons[NF];   // Dirichlet ghost state (conservative, dirichlet_conservatives)
};

// stage state of cell c (materialised planes)
__device__ __forceinline__ void uload(const double *S, long long n, long long c, double *u)
{
#pragma unroll
    for (int k = 0; k < NF; ++k) u[k] = __ldg(S + k * n + c);
}

// Fast arithmetic: the record of a state (one reciprocal and one square root).
__device__ __forceinline__ void fast_record(const double *c, double *r)
{
    const double ri = rcp_newton(c[0]);
    const double u = c[1] * ri, v = c[2] * ri, w = c[3] * ri;
    const double p = (GAMMA - 1.0) * fma(-0.5, fma(c[3], w, fma(c[2], v, c[1] * u)), c[4]);
    r[0] = u;
    r[1] = v;
    r[2] = w;
    r[3] = p;
    r[4] = sqrt_newton(GAMMA * p * ri);
    r[5] = c[4] + p;
}

// Fast arithmetic: the LLF flux (times half the area) of a face from the two
// sides' states and records; returns the face eigenvalue.
__device__ __forceinline__ double fast_split(const double *cl, const double *rl, const double *cr, const double *rr,
                                             const double *nrm, double half_area, double *F)
{
    double f[2][NF], lam[2];
    const double *cs[2] = {cl, cr}, *rs[2] = {rl, rr};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const double *c = cs[s], *r = rs[s];
        const double un = fma(r[2], nrm[2], fma(r[1], nrm[1], r[0] * nrm[0]));
        const double mn = c[0] * un;
        f[s][0] = mn;
        f[s][1] = fma(mn, r[0], r[3] * nrm[0]);
        f[s][2] = fma(mn, r[1], r[3] * nrm[1]);
        f[s][3] = fma(mn, r[2], r[3] * nrm[2]);
        f[s][4] = un * r[5];
        lam[s] = fabs(un) + r[4];
    }
    const double lambda = max_nonneg(lam[0], lam[1]);
#pragma unroll
    for (int k = 0; k < NF; ++k) F[k] = half_area * fma(-lambda, cr[k] - cl[k], f[0][k] + f[1][k]);
    return lambda;
}

// Reference arithmetic: euler.cpp:42-73 on the two side states.
__device__ __forceinline__ double exact_split(const double *cl, const double *cr, const double *nrm, double *F)
{
    double pl[NF], pr[NF], fl[NF], fr[NF];
    ExactArith::cons2prim(cl, pl);
    ExactArith::cons2prim(cr, pr);
    ExactArith::eval_fluxes(cl, pl, nrm, fl);
    ExactArith::eval_fluxes(cr, pr, nrm, fr);
    const double lamL = fabs(ExactArith::normal_velocity(pl, nrm)) + sqrt(GAMMA * pl[4]);
    const double lamR = fabs(ExactArith::normal_velocity(pr, nrm)) + sqrt(GAMMA * pr[4]);
    return ExactArith::face(cl, fl, lamL, cr, fr, lamR, F);
}

// Fast arithmetic: the record planes of every cell of the stage input.
__global__ void __launch_bounds__(256) urec_kernel(UMesh m, const double *state, const Ctrl *ctrl, int stage)
{
    if (stage >= STAGE_1) {
        const bool active = (stage == STAGE_1) ? (ctrl->t < ctrl->t_end) && (ctrl->step < ctrl->max_steps)
                                               : ctrl->active != 0;
        if (!active) return;
    }
    const long long n = m.ncells;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double u[NF], r[6];
        uload(state, n, c, u);
        fast_record(u, r);
#pragma unroll
        for (int k = 0; k < 6; ++k) m.rec[k * n + c] = r[k];
    }
}

template <class A, int STAGE>
__global__ void __launch_bounds__(256) uface_kernel(UMesh m, const double *state, double *P, Ctrl *ctrl,
                                                    double *rhs_maxeig)
{
    if (STAGE != STAGE_RHS) {
        const bool active = (STAGE == STAGE_1) ? (ctrl->t < ctrl->t_end) && (ctrl->step < ctrl->max_steps)
                                               : ctrl->active != 0;
        if (!active) return;
    }
    const long long n = m.ncells, nf = m.nfaces;
    double lmax = 0.0;
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf; f += (long long)gridDim.x * blockDim.x) {
        const long long o = m.owner[f], nb = m.neigh[f];
        const bool os = m.solved[o] != 0;
        const bool ns = nb >= 0 && m.solved[nb] != 0;
        double F[NF] = {0.0, 0.0, 0.0, 0.0, 0.0};
        if (os || ns) {
            const double nrm[3] = {__ldg(m.normal + f), __ldg(m.normal + nf + f), __ldg(m.normal + 2 * nf + f)};
            double co[NF], cn[NF], ro[6], rn[6];
            const int bc = m.bc[f];
            if (bc == BC_NONE) {
                uload(state, n, o, co);
                uload(state, n, nb, cn);
                if (!IsExact<A>::value) {
#pragma unroll
                    for (int k = 0; k < 6; ++k) { ro[k] = __ldg(m.rec + k * n + o); rn[k] = __ldg(m.rec + k * n + nb); }
                }
            } else {
                // the fluid side's state and its ghost, placed by selects (no
                // run-time pointer into the local arrays, which would move
                // them to local memory); the ghost is computed out of line
                const long long fc = os ? o : nb;
                StateV<NF> fl, dp;
                uload(state, n, fc, fl.v);
#pragma unroll
                for (int k = 0; k < NF; ++k) dp.v[k] = m.dir_cons[k];
                const double sgn = os ? 1.0 : -1.0;   // the ghost faces the fluid cell
                const StateV<NF> gv = ghost_state_ool<ExactArith>(bc, sgn * nrm[0], sgn * nrm[1], sgn * nrm[2], fl, dp);
#pragma unroll
                for (int k = 0; k < NF; ++k) { co[k] = os ? fl.v[k] : gv.v[k]; cn[k] = os ? gv.v[k] : fl.v[k]; }
                if (!IsExact<A>::value) {
                    double rf[6], rv[6];
#pragma unroll
                    for (int k = 0; k < 6; ++k) rf[k] = __ldg(m.rec + k * n + fc);
                    fast_record(gv.v, rv);
#pragma unroll
                    for (int k = 0; k < 6; ++k) { ro[k] = os ? rf[k] : rv[k]; rn[k] = os ? rv[k] : rf[k]; }
                }
            }
            const double ar = __ldg(m.area + f);
            double lam;
            if (IsExact<A>::value) {
                lam = exact_split(co, cn, nrm, F);
#pragma unroll
                for (int k = 0; k < NF; ++k) F[k] = ar * F[k];
            } else {
                lam = fast_split(co, ro, cn, rn, nrm, half_ftz(ar), F);
            }
            lmax = max_nonneg(lmax, lam);
        }
#pragma unroll
        for (int k = 0; k < NF; ++k) P[k * nf + f] = F[k];
    }
    if (STAGE <= STAGE_1) {
        lmax = warp_max(lmax);
        if ((threadIdx.x & 31) == 0) {
            unsigned long long *dst = (STAGE == STAGE_RHS) ? (unsigned long long *)rhs_maxeig : &ctrl->maxeig_bits;
            atomicMax(dst, (unsigned long long)dbits(lmax));
        }
    }
}

// Residual gather + stage combination (state = this stage's input, out = its output).
template <class A, int STAGE>
__global__ void __launch_bounds__(256) ucell_kernel(UMesh m, const double *P, const double *U, const double *state,
                                                    double *out, Ctrl *ctrl)
{
    StepScalars sc;
    sc.dt = 0.0;
    sc.s = 0.0;
    sc.active = true;
    if (STAGE != STAGE_RHS) {
        if (STAGE == STAGE_1) {
            sc.active = (ctrl->t < ctrl->t_end) && (ctrl->step < ctrl->max_steps);
            if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->active = sc.active ? 1 : 0;
        } else {
            sc.active = ctrl->active != 0;
            sc.dt = ctrl->dt;
        }
        if (STAGE == STAGE_3 && sc.active && blockIdx.x == 0 && threadIdx.x == 0) {
            ctrl->last_maxeig = bitsd((long long)ctrl->maxeig_bits);
            ctrl->t += sc.dt;
            ctrl->step += 1;
            ctrl->maxeig_bits = 0ull;
        }
        if (!sc.active) return;
    }
    const long long n = m.ncells, nf = m.nfaces;
    unsigned status = 0;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        double acc[NF] = {0., 0., 0., 0., 0.};
        const bool solved = m.solved[c] != 0;
        if (STAGE == STAGE_1 && solved) {
            // the stage input of a solved cell: rho < 0, p < 0 (2 rho E < |m|^2
            // for rho > 0, division-free) or NaN, as the Cartesian kernels flag
            // it (the reference only logs it, euler.cpp:93-101)
            double u[NF];
            uload(state, n, c, u);
            const double m2 = fma(u[3], u[3], fma(u[2], u[2], u[1] * u[1]));
            const double q = fma(twice_exact(u[0]), u[4], -m2);
            // compares on the bit patterns (integer pipe): rho > 0, q NaN
            const long long ir = dbits(u[0]), iq = dbits(q);
            status |= state_flags(u[0], (ir > 0 && ir <= 0x7ff0000000000000ll) ? q : 0.0);
            if ((iq & 0x7fffffffffffffffll) > 0x7ff0000000000000ll) status |= 4u;
        }
        if (solved) {
            const long long e = m.csr_off[c + 1];
            for (long long i = m.csr_off[c]; i < e; ++i) {
                const long long code = m.csr_face[i];
                const bool owner = code < 0;
                const long long f = owner ? -code - 1 : code;
                // acc -+ P (euler.cpp:237-247) as one fused operation with the
                // sign as a factor: exact product, one rounding, the same bits
                const double sg = owner ? -1.0 : 1.0;
#pragma unroll
                for (int k = 0; k < NF; ++k) acc[k] = fma(sg, __ldg(P + k * nf + f), acc[k]);
            }
        }
        const double V = m.vol[c];
        const double s = IsExact<A>::value ? 0.0 : sc.dt * (solved ? __ldg(m.inv_vol + c) : 0.0);
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            const long long o = k * n + c;
            if (STAGE == STAGE_RHS || STAGE == STAGE_1) {
                out[o] = acc[k];
            } else if (!solved) {
                continue;                          // unsolved cells keep their state (main.cpp:411-414)
            } else if (STAGE == STAGE_2) {
                const double u = __ldg(U + o), w = __ldg(state + o);
                out[o] = IsExact<A>::value ? 0.75 * u + 0.25 * (w + sc.dt * acc[k] / V)
                                           : fma(0.25, fma(s, acc[k], w), 0.75 * u);
            } else {
                const double u = U[o], w = __ldg(state + o);
                out[o] = IsExact<A>::value ? (1. / 3) * u + (2. / 3) * (w + sc.dt * acc[k] / V)
                                           : fma(2.0 / 3.0, fma(s, acc[k], w), u * (1.0 / 3.0));
            }
        }
    }
    if (STAGE == STAGE_1) {
        status = __reduce_or_sync(0xffffffffu, status);
        if ((threadIdx.x & 31) == 0 && status) atomicOr(&ctrl->status, status);
    }
}

// W1 = U + dt R1 / V for solved cells, with the dt of main.cpp:398-402.
template <class A>
__global__ void __launch_bounds__(256) uform_w1_kernel(UMesh m, const double *U, const double *R, double *W, Ctrl *ctrl)
{
    const bool active = ctrl->active != 0;
    if (!active) return;
    const double maxEig = bitsd((long long)ctrl->maxeig_bits);
    double dt = ctrl->cfl_h / maxEig;
    if (ctrl->t + dt > ctrl->t_end) dt = ctrl->t_end - ctrl->t;
    if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->dt = dt;
    const long long n = m.ncells;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        if (!m.solved[c]) continue;
        const double V = m.vol[c];
        const double s = IsExact<A>::value ? 0.0 : dt * __ldg(m.inv_vol + c);
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            const long long i = k * n + c;
            const double u = __ldg(U + i), r = __ldg(R + i);
            W[i] = IsExact<A>::value ? u + dt * r / V : fma(s, r, u);
        }
    }
}

} // namespace mmf
