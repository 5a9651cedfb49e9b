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

// Bit patterns of doubles through opaque register moves.  With the
// compiler's own bit casts, integer tricks on the patterns are folded back
// into floating-point operations (masking the sign bit becomes an FP64
// absolute value, a select on compared patterns an FP64 minimum or maximum,
// an OR-ed sign bit an FP64 copysign), which run on the narrow FP64 pipe of
// this GPU; behind these moves they stay on the integer pipe.
__device__ __forceinline__ long long dbits(double x)
{
    long long i;
    asm("mov.b64 %0, %1;" : "=l"(i) : "d"(x));
    return i;
}

__device__ __forceinline__ double bitsd(long long i)
{
    double x;
    asm("mov.b64 %0, %1;" : "=d"(x) : "l"(i));
    return x;
}

constexpr int NF = 5;               // constants.hpp:35
constexpr double GAMMA = 1.4;       // constants.hpp:55

// constants.hpp:58-62 (+ periodic, which has no reference counterpart)
enum BCType : int { BC_NONE = -1, BC_FREE_FLOW = 0, BC_REFLECTING = 1, BC_WALL = 2, BC_DIRICHLET = 3,
                    BC_PERIODIC = 16 };

// Cell record: the state and what the faces of the cell need from it.
// f[d][k] is the physical flux along +e_d, lam[d] the wave speed |u_d| + a.
template <int DIM, int NV>
struct CellRecV {
    double c[NV];
    double f[DIM][NV];
    double lam[DIM];
};
template <int DIM>
using CellRec = CellRecV<DIM, NF>;

struct ExactArith {
    static constexpr int NVAR = NF;
    __host__ __device__ static constexpr int field(int k) { return k; }
    __device__ __forceinline__ static void dirichlet(const double *dir_cons, double *g);
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

// Reciprocal by one third-order iteration y <- y (1 + e + e^2), e = 1 - x y
// (the Newton-Raphson step y + y e with the next term of the series for
// 1 / (1 - e)), seeded with the hardware reciprocal approximation of the high
// word (rcp.approx.ftz.f64): it cubes the seed error, one fused multiply-add
// fewer than two Newton-Raphson steps.  For positive normal x (densities);
// checked against IEEE division in the GPU tests.
__device__ __forceinline__ double rcp_newton(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

// x / 2 and 2 x by moving the exponent field (integer pipe; the FP64 pipe
// is the narrow one).  Exact wherever the result is a normal number; half_ftz
// flushes results below the normal range to a signed zero, twice_exact doubles
// zero and subnormal x by a shift of the significand; infinities and NaNs keep
// their value (and twice_exact does not guard against overflow: it is used
// on physical magnitudes, far below 1e308).
__device__ __forceinline__ double half_ftz(double x)
{
    const long long ix = dbits(x);
    const long long e = ix & 0x7ff0000000000000ll;
    if (e == 0x7ff0000000000000ll) return x;
    return bitsd(e > 0x0010000000000000ll ? ix - 0x0010000000000000ll
                                                         : ix & (long long)0x8000000000000000ull);
}

__device__ __forceinline__ double twice_exact(double x)
{
    const long long ix = dbits(x);
    const long long e = ix & 0x7ff0000000000000ll;
    if (e == 0x7ff0000000000000ll) return x;
    const long long sign = ix & (long long)0x8000000000000000ull;
    return bitsd(e != 0 ? ix + 0x0010000000000000ll : ((ix ^ sign) << 1) | sign);
}

// Square root from the rsqrt.approx.ftz.f64 seed y by one third-order step:
// with s = x y and 2e = 1 - x y^2 (e = 1/2 - s y/2, exact in one FMA),
// sqrt(x) = s (1 - 2e)^(-1/2) = s (1 + e + 3/2 e^2 + O(e^3)).  Five FP64
// instructions (a coupled Newton iteration plus a correction takes six); the
// seed's relative error cubed is far below an ulp.  x >= 0; x = 0 returns 0
// (selected on the bit pattern, no FP64 compare).
__device__ __forceinline__ double sqrt_newton(double x)
{
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double s = x * y;
    const double e = fma(-s, half_ftz(y), 0.5);
    const double g = e * fma(1.5, e, 1.0);
    const double r = fma(s, g, s);
    return (dbits(x) == 0ll) ? 0.0 : r;
}

// max of two non-negative doubles through their bit patterns (integer pipe)
__device__ __forceinline__ double max_nonneg(double a, double b)
{
    const long long ia = dbits(a), ib = dbits(b);
    return bitsd(ia > ib ? ia : ib);
}

// status bits from the sign / exponent bits (integer pipe): rho < 0, p < 0, NaN
__device__ __forceinline__ unsigned state_flags(double rho, double p)
{
    const long long ir = dbits(rho), ip = dbits(p);
    unsigned f = 0;
    if (ir < 0) f |= 1u;
    if (ip < 0) f |= 2u;
    if (((ir >> 52) & 0x7ff) == 0x7ff || ((ip >> 52) & 0x7ff) == 0x7ff) f |= 4u;
    return f;
}

// Fast arithmetic.  NV = number of stored fields: 5 = (rho, mx, my, mz, E);
// 4 = (rho, mx, my, E) for 2D states whose z-momentum is identically zero
// (the reference keeps it exactly +0 in 2D, problem.cpp:319-323), which
// removes a fifth of the work.
template <int NV>
struct FastArithT {
    static constexpr int NVAR = NV;
    static constexpr int IE = NV - 1;   // index of rho E in the stored fields

    // physical field plane of stored field k
    __host__ __device__ static constexpr int field(int k) { return (NV == 4 && k == 3) ? 4 : k; }

    template <int DIM>
    __device__ __forceinline__ static void record(CellRecV<DIM, NV> &r, unsigned *status)
    {
        const double rho = r.c[0];
        const double rinv = rcp_newton(rho);
        const double u = r.c[1] * rinv, v = r.c[2] * rinv;
        const double w = (NV == 5) ? r.c[3] * rinv : 0.0;
        double q = fma(r.c[2], v, r.c[1] * u);              // rho |u|^2
        if (NV == 5) q = fma(r.c[3], w, q);
        const double E = r.c[IE];
        const double p = fma(-0.5 * (GAMMA - 1.0), q, (GAMMA - 1.0) * E);
        if (status) *status |= state_flags(rho, p);
        const double a = sqrt_newton(GAMMA * p * rinv);
        const double H = E + p;                             // rho * total enthalpy
        // the momentum fluxes rho u_i u_j (i != j) once each
        const double muv = r.c[1] * v;                      // rho u v
        const double muw = (NV == 5) ? r.c[1] * w : 0.0;    // rho u w
        const double mvw = (NV == 5) ? r.c[2] * w : 0.0;    // rho v w
        const double vel[3] = {u, v, w};
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const double m = r.c[1 + d];
            r.f[d][0] = m;
            r.f[d][1] = (d == 0) ? fma(m, u, p) : (d == 1 ? muv : muw);
            r.f[d][2] = (d == 1) ? fma(m, v, p) : (d == 0 ? muv : mvw);
            if (NV == 5) r.f[d][3] = (d == 2) ? fma(m, w, p) : (d == 0 ? muw : mvw);
            r.f[d][IE] = vel[d] * H;
            r.lam[d] = fabs(vel[d]) + a;
        }
    }
    // G = (f_L + f_R) - lambda (U_R - U_L): twice the face flux (the 1/2 and the
    // area are applied in the stage update).
    __device__ __forceinline__ static double face(const double *cL, const double *fL, double lamL,
                                                  const double *cR, const double *fR, double lamR, double *G)
    {
        const double lambda = max_nonneg(lamL, lamR);
#pragma unroll
        for (int k = 0; k < NV; ++k) G[k] = fma(-lambda, cR[k] - cL[k], fL[k] + fR[k]);
        return lambda;
    }
    // mirror the normal momentum; rho and E are unchanged
    __device__ __forceinline__ static void reflect(const double *n, const double *c, double *cbc)
    {
        double mn = c[1] * n[0] + c[2] * n[1];
        if (NV == 5) mn = fma(c[3], n[2], mn);
        cbc[0] = c[0];
        cbc[1] = fma(-2.0 * mn, n[0], c[1]);
        cbc[2] = fma(-2.0 * mn, n[1], c[2]);
        if (NV == 5) cbc[3] = fma(-2.0 * mn, n[2], c[3]);
        cbc[IE] = c[IE];
    }
    // Dirichlet ghost: the inflow state, precomputed (dirichlet_conservatives)
    __device__ __forceinline__ static void dirichlet(const double *dir_cons, double *g)
    {
#pragma unroll
        for (int k = 0; k < NV; ++k) g[k] = dir_cons[field(k)];
    }
};

using FastArith = FastArithT<5>;
using FastArith2DW0 = FastArithT<4>;

__device__ __forceinline__ void ExactArith::dirichlet(const double *dir_cons, double *g)
{
#pragma unroll
    for (int k = 0; k < NF; ++k) g[k] = dir_cons[k];   // euler.cpp:366-376, precomputed
}

// The Dirichlet ghost's conservative state, prim2cons (utils.cpp:71-83) of the
// inflow primitive state in the reference's operation order, computed once on
// the host.  Every product and quotient goes through a volatile so that the
// host compiler cannot fuse a multiply-add: the bits are those of the device's
// ExactArith::prim2cons (IEEE operations, no contraction).
inline void dirichlet_conservatives(const double *p, double *c)
{
    volatile double c0 = p[0] / p[4];
    volatile double c1 = c0 * p[1], c2 = c0 * p[2], c3 = c0 * p[3];
    volatile double t1 = c0 * p[4];
    volatile double t2 = t1 / (GAMMA - 1.0);
    volatile double s1 = p[1] * p[1], s2 = p[2] * p[2], s3 = p[3] * p[3];
    volatile double s12 = s1 + s2;
    volatile double ss = s12 + s3;
    volatile double h = 0.5 * c0;
    volatile double t3 = h * ss;
    c[0] = c0;
    c[1] = c1;
    c[2] = c2;
    c[3] = c3;
    c[4] = t2 + t3;
}

// Ghost state behind a border face (euler.cpp:261-308, 347-376).  'n' is the
// outward normal of the border face; dir_cons is the Dirichlet conservative
// state (dirichlet_conservatives).
template <class A>
__device__ __forceinline__ void ghost_state(int bc, const double *n, const double *c, const double *dir_cons,
                                            double *g)
{
    if (bc == BC_REFLECTING || bc == BC_WALL) {
        A::reflect(n, c, g);
    } else if (bc == BC_DIRICHLET) {
        A::dirichlet(dir_cons, g);
    } else {
#pragma unroll
        for (int k = 0; k < A::NVAR; ++k) g[k] = c[k];
    }
}

template <int NV>
struct StateV {
    double v[NV];
};

// ghost_state out of line, every argument by value, for kernels where the
// ghost branch is rare and its registers would weigh on the common path.
template <class A>
__device__ __noinline__ StateV<A::NVAR> ghost_state_ool(int bc, double n0, double n1, double n2, StateV<A::NVAR> c,
                                                        StateV<NF> dir_cons)
{
    const double n[3] = {n0, n1, n2};
    StateV<A::NVAR> g;
    ghost_state<A>(bc, n, c.v, dir_cons.v, g.v);
    return g;
}

// c := the ghost of c across the border face of outward normal +-e_dir
// (side); OOL takes the out-of-line ghost_state (the order-2 kernels, whose
// register budget is tight), else it is inlined (the order-1 marches).
template <class A, bool OOL = false>
__device__ __forceinline__ void ghost_in_place(int bc, int dir, int side, double *c, const double *dir_cons)
{
    const double s = side < 0 ? -1.0 : 1.0;
    if (OOL) {
        StateV<A::NVAR> in;
        StateV<NF> dc;
#pragma unroll
        for (int k = 0; k < A::NVAR; ++k) in.v[k] = c[k];
#pragma unroll
        for (int k = 0; k < NF; ++k) dc.v[k] = dir_cons[k];
        const StateV<A::NVAR> g = ghost_state_ool<A>(bc, dir == 0 ? s : 0.0, dir == 1 ? s : 0.0, dir == 2 ? s : 0.0,
                                                     in, dc);
#pragma unroll
        for (int k = 0; k < A::NVAR; ++k) c[k] = g.v[k];
    } else {
        double n[3] = {0.0, 0.0, 0.0};
        n[dir] = s;
        double g[A::NVAR];
        ghost_state<A>(bc, n, c, dir_cons, g);
#pragma unroll
        for (int k = 0; k < A::NVAR; ++k) c[k] = g[k];
    }
}

} // namespace mmf
