// mmf_physics.cuh -- FP64 device physics of the minimmerflow Euler step.
//
// Two arithmetic variants share one interface:
//
//  * ExactArith restates the reference operation order exactly
//    (utils.cpp:37-83, euler.cpp:42-113, euler.cpp:298-376).  Translation
//    units that instantiate it are compiled with -fmad=false, so with IEEE
//    division and square root it reproduces the reference's CPU results bit
//    for bit (same accumulation order per cell, see mmf_cartesian.cuh).
//
//  * FastArith is the same mathematics rearranged for a GPU whose FP64 pipe
//    is narrow: one division (1/rho) and one square root per cell, the
//    physical flux of a cell built once per direction from the conservative
//    momentum and total enthalpy rho*H = E + p, the 1/2 and the face area
//    folded into the stage update, and FMA contraction allowed.  It agrees
//    with the reference to round-off (about 1e-15 relative per step).
#pragma once

#include <cstdint>

namespace mmf {

constexpr int NF = 5;               // constants.hpp:35
constexpr double GAMMA = 1.4;       // constants.hpp:55

// constants.hpp:58-62 (+ periodic, which has no reference counterpart)
enum BCType : int { BC_NONE = -1, BC_FREE_FLOW = 0, BC_REFLECTING = 1, BC_WALL = 2, BC_DIRICHLET = 3,
                    BC_PERIODIC = 16 };

// Cell record: the state and what the faces of the cell need from it.
// f[d][k] is the physical flux along +e_d, lam[d] the wave speed |u_d| + a.
template <int DIM>
struct CellRec {
    double c[NF];
    double f[DIM][NF];
    double lam[DIM];
};

struct ExactArith {
    // utils.cpp:48-63
    __device__ __forceinline__ static void cons2prim(const double *c, double *p)
    {
        double K = (c[1] * c[1] + c[2] * c[2] + c[3] * c[3]) / (c[0] * c[0]);
        p[4] = (2.0 * c[4] / c[0] - K) / (2.0 / (GAMMA - 1.0));
        p[1] = c[1] / c[0];
        p[2] = c[2] / c[0];
        p[3] = c[3] / c[0];
        p[0] = c[0] * p[4];
    }
    // utils.cpp:71-83
    __device__ __forceinline__ static void prim2cons(const double *p, double *c)
    {
        c[0] = p[0] / p[4];
        c[1] = c[0] * p[1];
        c[2] = c[0] * p[2];
        c[3] = c[0] * p[3];
        c[4] = c[0] * p[4] / (GAMMA - 1.0) + 0.5 * c[0] * (p[1] * p[1] + p[2] * p[2] + p[3] * p[3]);
    }
    // utils.cpp:37-40
    __device__ __forceinline__ static double normal_velocity(const double *p, const double *n)
    {
        return (p[1] * n[0] + p[2] * n[1] + p[3] * n[2]);
    }
    // euler.cpp:83-113
    __device__ __forceinline__ static void eval_fluxes(const double *c, const double *p, const double *n, double *f)
    {
        double u = p[1], v = p[2], w = p[3];
        double vel2 = u * u + v * v + w * w;
        double un = normal_velocity(p, n);
        double pr = p[0];
        double rho = c[0];
        double eto = pr / (GAMMA - 1.) + 0.5 * rho * vel2;
        double massFlux = rho * un;
        f[0] = massFlux;
        f[1] = massFlux * u + pr * n[0];
        f[2] = massFlux * v + pr * n[1];
        f[3] = massFlux * w + pr * n[2];
        f[4] = un * (eto + pr);
    }
    // Cell record: the per-side part of euler.cpp:42-65 evaluated once per cell
    // and direction (cons2prim, evalFluxes, |u.n| + sqrt(gamma T)).
    template <int DIM>
    __device__ __forceinline__ static void record(CellRec<DIM> &r, unsigned *status)
    {
        double p[NF];
        cons2prim(r.c, p);
        if (status) {
            if (r.c[0] < 0.0) *status |= 1u;   // euler.cpp:98-101 logs this
            if (p[0] < 0.0) *status |= 2u;     // euler.cpp:93-96 logs this
            if (r.c[0] != r.c[0] || p[0] != p[0]) *status |= 4u;
        }
        double a = sqrt(GAMMA * p[4]);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            double n[3] = {d == 0 ? 1.0 : 0.0, d == 1 ? 1.0 : 0.0, d == 2 ? 1.0 : 0.0};
            eval_fluxes(r.c, p, n, r.f[d]);
            r.lam[d] = fabs(normal_velocity(p, n)) + a;
        }
    }
    // euler.cpp:67-72 for a face with normal +e_d between records L and R;
    // returns the face eigenvalue, writes F (the reference's fluxes).
    __device__ __forceinline__ static double face(const double *cL, const double *fL, double lamL,
                                                  const double *cR, const double *fR, double lamR, double *F)
    {
        double lambda = (lamR < lamL) ? lamL : lamR;   // std::max(lambdaR, lambdaL)
#pragma unroll
        for (int k = 0; k < NF; ++k) F[k] = 0.5 * ((fR[k] + fL[k]) - lambda * (cR[k] - cL[k]));
        return lambda;
    }
    // euler.cpp:318-337
    __device__ __forceinline__ static void reflect(const double *n, const double *c, double *cbc)
    {
        double prim[NF];
        cons2prim(c, prim);
        double u0 = prim[1], u1 = prim[2], u2 = prim[3];
        double un = normal_velocity(prim, n);
        double un0 = un * n[0], un1 = un * n[1], un2 = un * n[2];
        prim[1] = u0 - 2 * un0;
        prim[2] = u1 - 2 * un1;
        prim[3] = u2 - 2 * un2;
        prim2cons(prim, cbc);
    }
};

struct FastArith {
    // Same record in the fast formulation: u = m / rho with one division,
    // p = (gamma-1)(E - m.u/2), a = sqrt(gamma p / rho), flux from m and E+p.
    template <int DIM>
    __device__ __forceinline__ static void record(CellRec<DIM> &r, unsigned *status)
    {
        const double rho = r.c[0];
        const double rinv = 1.0 / rho;
        const double u = r.c[1] * rinv, v = r.c[2] * rinv, w = r.c[3] * rinv;
        const double q = fma(r.c[3], w, fma(r.c[2], v, r.c[1] * u));       // rho |u|^2
        const double p = (GAMMA - 1.0) * fma(-0.5, q, r.c[4]);
        if (status) {
            if (rho < 0.0) *status |= 1u;
            if (p < 0.0) *status |= 2u;
            if (rho != rho || p != p) *status |= 4u;
        }
        const double a = sqrt(GAMMA * p * rinv);
        const double H = r.c[4] + p;                                    // rho * total enthalpy
        const double vel[3] = {u, v, w};
        const double muv = r.c[1] * v;                                  // rho u v, shared by f_x[2], f_y[1]
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const double m = r.c[1 + d];
            r.f[d][0] = m;
            r.f[d][1] = (d == 0) ? fma(m, u, p) : (d == 1 ? muv : m * u);
            r.f[d][2] = (d == 1) ? fma(m, v, p) : (d == 0 ? muv : m * v);
            r.f[d][3] = (d == 2) ? fma(m, w, p) : m * w;
            r.f[d][4] = vel[d] * H;
            r.lam[d] = fabs(vel[d]) + a;
        }
    }
    // G = (f_L + f_R) - lambda (U_R - U_L): the face flux times 2 (the 1/2 and
    // the area are applied in the stage update).
    __device__ __forceinline__ static double face(const double *cL, const double *fL, double lamL,
                                                  const double *cR, const double *fR, double lamR, double *G)
    {
        double lambda = fmax(lamL, lamR);
#pragma unroll
        for (int k = 0; k < NF; ++k) G[k] = fma(-lambda, cR[k] - cL[k], fL[k] + fR[k]);
        return lambda;
    }
    __device__ __forceinline__ static void reflect(const double *n, const double *c, double *cbc)
    {
        // mirror the normal momentum: rho and E are unchanged
        const double mn = c[1] * n[0] + c[2] * n[1] + c[3] * n[2];
        cbc[0] = c[0];
        cbc[1] = fma(-2.0 * mn, n[0], c[1]);
        cbc[2] = fma(-2.0 * mn, n[1], c[2]);
        cbc[3] = fma(-2.0 * mn, n[2], c[3]);
        cbc[4] = c[4];
    }
};

// Ghost state behind a border face (euler.cpp:261-308, 347-376).  'n' is the
// outward normal of the border face; dir_prim is the Dirichlet primitive state.
template <class A>
__device__ __forceinline__ void ghost_state(int bc, const double *n, const double *c, const double *dir_prim,
                                            double *g)
{
    if (bc == BC_REFLECTING || bc == BC_WALL) {
        A::reflect(n, c, g);
    } else if (bc == BC_DIRICHLET) {
        ExactArith::prim2cons(dir_prim, g);
    } else {
#pragma unroll
        for (int k = 0; k < NF; ++k) g[k] = c[k];
    }
}

} // namespace mmf
