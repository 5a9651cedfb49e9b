// mmf_order2.cuh -- order-2 limited reconstruction on the uniform Cartesian grid.
//
// The reference's reconstruction has a polynomial hook, reconstruction::
// computePolynomials (reconstruction.cpp:47-55), and evaluates order 1 only
// (reconstruction.cpp:67-79); order 2 is a project extension on that hook:
//
//   slopes_kernel       computePolynomials: MUSCL slopes per direction and
//                       conservative field with the monotonised-central (MC)
//                       limiter sigma = minmod(2a, 2b, c), a = U_i - U_{i-1},
//                       b = U_{i+1} - U_i, c = (U_{i+1} - U_{i-1}) / 2 the
//                       central slope (border neighbours are the ghost states
//                       of euler.cpp:261-376), then a positivity fallback: if any
//                       face state U +- sigma/2 has rho <= 0 or p <= 0 the cell
//                       falls back to order 1.  A per-cell flag (limit / central)
//                       selects the limiter; the kernel reports where the limiter
//                       changed a slope by more than 1e-6 (|rho| + |rho E|) of
//                       the cell, or fell back (the troubled-cell labels).
//   stage2d_o2_kernel / stage3d_o2_kernel
//                       computeRHS with face states U +- sigma/2: every cell
//                       evaluates a record per face side; border faces use the
//                       ghost of the reconstructed face state, as the reference's
//                       face loop does (euler.cpp:197-226).
//   form_w1_kernel      W1 = U + dt R1 / V materialised for stage 2 (the
//                       slopes need W1 at the neighbours).
//
// Buffers per step: U, R (stage-1 residual, then the stage-2 result W2 in
// place), W (W1), S (slopes, DIM x NV planes), flags.
#pragma once

#include "mmf_cartesian.cuh"

namespace mmf {

// Limiter modes (per launch): every cell, no cell (central slopes), or the
// cells whose flag byte is non-zero.
enum { LIMIT_ALL = 0, LIMIT_NONE = 1, LIMIT_FLAGGED = 2 };

struct O2Args {
    const double *state;     // stage state planes (U, W1 or W2)
    double *S;               // slopes: plane (d * NV + k)
    const unsigned char *flag;
    unsigned char *active;   // nullable: 1 where the limiter changed a slope
    int limit_mode;
    Ctrl *ctrl;
    int stage;               // 0 = residual-only call, 1..3 = RK stage
    long long cell0, cell1;  // slopes of grid cells [cell0, cell1) (a band of rows or planes)
    int *tick = nullptr;     // the indicator's step counter, advanced by a step's stage-1 slopes (nullable)
};

// When the indicator runs every 'period' steps: the launches of a step whose
// counter (advanced by each step's stage-1 slopes, reset to 0 when the state
// or the time control changes) is not a multiple of the period do nothing,
// and the flags of the last run stand, dilated by one cell.
struct IndicatorStep {
    int period;        // 1: every step
    const int *tick;   // the step counter (period > 1)
};

__device__ __forceinline__ bool indicator_idle(const IndicatorStep &is)
{
    return is.period > 1 && (*is.tick % is.period) != 0;
}

// a*b <= 0 -> 0; else sign(a) min(2|a|, 2|b|, |central|)  (oracle orc_compute_polynomials)
template <class A>
__device__ __forceinline__ double mc_slope(double a, double b, double central)
{
    if (IsExact<A>::value) {
        if (a * b <= 0.0) return 0.0;
        double lim = fmin(2.0 * fabs(a), 2.0 * fabs(b));
        double mag = fmin(lim, fabs(central));
        return (a > 0.0) ? mag : -mag;
    } else {
        if (a * b <= 0.0) return 0.0;
        const double mag = fmin(fmin(2.0 * fabs(a), 2.0 * fabs(b)), fabs(central));
        return (a > 0.0) ? mag : -mag;
    }
}

// |x| as the bit pattern of a non-negative double (integer pipe); these
// compare like the values they encode
__device__ __forceinline__ long long abs_bits(double x)
{
    return dbits(x) & 0x7fffffffffffffffll;
}

// Fast arithmetic: the MC slope with its compares, absolute values, minima
// and sign on the integer pipe: a and b of opposite signs (or one of them
// zero) -> 0; else sign(a) min(2 min(|a|, |b|), |central|), where the
// doubling is exact.  Equal to mc_slope except when a b underflows to zero
// with a and b of the same sign (|a|, |b| below 1e-154).
__device__ __forceinline__ double mc_slope_bits(double a, double b, double central)
{
    const long long ia = dbits(a), ib = dbits(b);
    const long long ma = ia & 0x7fffffffffffffffll, mb = ib & 0x7fffffffffffffffll;
    if ((ia ^ ib) < 0 || ma == 0 || mb == 0) return 0.0;
    const long long m2 = dbits(twice_exact(bitsd(ma < mb ? ma : mb)));
    const long long mc = abs_bits(central);
    return bitsd((m2 < mc ? m2 : mc) | (ia & (long long)0x8000000000000000ull));
}

// division-free admissibility of a state: rho > 0 and 2 rho E > |m|^2
template <class A>
__device__ __forceinline__ bool admissible(const double *c)
{
    constexpr int NV = A::NVAR;
    if (IsExact<A>::value) {
        if (!(c[0] > 0.0)) return false;
        double m2 = c[1] * c[1] + c[2] * c[2];
        if (NV == 5) m2 = m2 + c[3] * c[3];
        return (2.0 * c[0] * c[NV - 1] - m2) > 0.0;
    }
    // fast: "x > 0" as 0 < bits(x) < bits(+inf) on the integer pipe (NaN fails, as in the compare)
    const long long inf = 0x7ff0000000000000ll;
    const long long ir = dbits(c[0]);
    if (!(ir > 0 && ir <= inf)) return false;
    double m2 = fma(c[2], c[2], c[1] * c[1]);
    if (NV == 5) m2 = fma(c[3], c[3], m2);
    const long long iq = dbits(fma(twice_exact(c[0]), c[NV - 1], -m2));
    return iq > 0 && iq <= inf;
}

// reconstructed face state U + off sigma (off = +-1/2)
template <class A>
__device__ __forceinline__ double face_value(double u, double off, double sigma)
{
    return IsExact<A>::value ? u + off * sigma : fma(off, sigma, u);
}

template <class A>
__device__ __forceinline__ void load_plain(const double *planes, long long plane, long long g, double *c)
{
#pragma unroll
    for (int k = 0; k < A::NVAR; ++k) c[k] = __ldg(planes + (long long)A::field(k) * plane + g);
}

// Positivity of the face states U -+ sigma / 2 of one direction of a cell,
// in FP64 (the arithmetic's own operations).
template <class A>
__device__ __forceinline__ bool dir_admissible(const double *uc, const double *sig)
{
    constexpr int NV = A::NVAR;
    double fm[NV], fp[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        fm[k] = IsExact<A>::value ? uc[k] - 0.5 * sig[k] : fma(-0.5, sig[k], uc[k]);
        fp[k] = face_value<A>(uc[k], 0.5, sig[k]);
    }
    return admissible<A>(fm) && admissible<A>(fp);
}

// ... of every direction
template <class A, int DIM>
__device__ __forceinline__ bool faces_admissible(const double *uc, const double (*sig)[A::NVAR])
{
    bool ok = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ok = ok && dir_admissible<A>(uc, sig[d]);
    return ok;
}

// x / 2^(emax - 1023) as a float (the value with exponent field emax maps to
// [1, 2)), its significand truncated to 20 bits, on the integer pipe; scaled
// magnitudes below 2^-126 flush to 0.  Error < 2^-20 |result| + 2^-126.
__device__ __forceinline__ float scaled_f32(double x, int emax)
{
    const unsigned hi = (unsigned)((unsigned long long)dbits(x) >> 32);
    const int e = (int)((hi >> 20) & 0x7ff) - emax + 127;
    return e > 0 ? __uint_as_float((hi & 0x80000000u) | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3)) : 0.0f;
}

// The positivity test of dir_admissible decided in FP32 where the margins
// allow it: 1 = every face state has rho > 0 and 2 rho E > |m|^2, 0 = some
// face state has not, -1 = undecided.  FP64 instructions cost about as much
// as 30 FP32 ones on this GPU, so the FP32 screen with an FP64 fallback for
// the undecided cells is the cheaper route to the same answer.
//
// The cell's values and the direction's slopes are scaled by a common power
// of two and truncated (scaled_f32).  Each FP32 face value carries a bound
// e_k at least 3.7 times its distance to the FP64 face value (truncation
// 2^-20, FP32 rounding 2^-24, FP64 rounding 2^-53, relative to |u| +
// |sigma|/2; flushing, absolute), and the bound of Q = 2 rho E - |m|^2
// doubles the propagated error and adds 2^-20 of the magnitudes for the
// roundings of Q itself (FP32, and FP64 in the test it replaces) and 2^-100
// for underflowed terms.  A sign decided outside these bounds is the sign of
// the FP64 evaluation.
template <class A>
__device__ __forceinline__ int screen_dir(const double *uc, const double *sig)
{
    constexpr int NV = A::NVAR;
    constexpr int IE = NV - 1;
    int emax = 0;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        emax = max(emax, (int)((dbits(uc[k]) >> 52) & 0x7ff));
        emax = max(emax, (int)((dbits(sig[k]) >> 52) & 0x7ff));
    }
    if (emax >= 0x7ff) return -1;   // an infinity or a NaN
    float u[NV], au[NV], sg[NV], e[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        u[k] = scaled_f32(uc[k], emax);
        au[k] = fabsf(u[k]);
        sg[k] = scaled_f32(sig[k], emax);
        e[k] = fmaf(0x1p-18f, fmaf(0.5f, fabsf(sg[k]), au[k]), 0x1p-120f);
    }
    bool sure_ok = true, sure_bad = false;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        float f[NV], af[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) { f[k] = fmaf(side ? 0.5f : -0.5f, sg[k], u[k]); af[k] = fabsf(f[k]); }
        float m2 = 0.0f, em = 0.0f;
#pragma unroll
        for (int k = 1; k < IE; ++k) {
            m2 = fmaf(f[k], f[k], m2);
            em = fmaf(e[k], fmaf(2.0f, af[k], e[k]), em);
        }
        const float Q = fmaf(2.0f * f[0], f[IE], -m2);
        const float eQ = fmaf(2.0f, fmaf(2.0f, fmaf(e[0], af[IE], fmaf(e[IE], af[0], e[0] * e[IE])), em),
                              fmaf(0x1p-20f, fmaf(2.0f * af[0], af[IE], m2), 0x1p-100f));
        sure_ok = sure_ok && (f[0] > e[0]) && (Q > eQ);
        sure_bad = sure_bad || (f[0] < -e[0]) || (Q < -eQ);
    }
    return sure_bad ? 0 : (sure_ok ? 1 : -1);
}

// ... of every direction: 0 if a direction's is 0, 1 if every one's is 1
template <class A, int DIM>
__device__ __forceinline__ int screen_faces(const double *uc, const double (*sig)[A::NVAR])
{
    int dec = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const int r = screen_dir<A>(uc, sig[d]);
        if (r == 0) return 0;
        if (r < 0) dec = -1;
    }
    return dec;
}

// Self-test of screen_faces: for each sample, the FP32 decision and the FP64
// test it stands for (uc [n][NV], sig [n][DIM][NV]).
template <class A, int DIM>
__global__ void __launch_bounds__(128) screen_selftest_kernel(long long n, const double *uc, const double *sig,
                                                              int *dec, unsigned char *ref)
{
    constexpr int NV = A::NVAR;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double u[NV], s[DIM][NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) u[k] = uc[i * NV + k];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
        for (int k = 0; k < NV; ++k) s[d][k] = sig[(i * DIM + d) * NV + k];
    dec[i] = screen_faces<A, DIM>(u, s);
    ref[i] = faces_admissible<A, DIM>(u, s) ? 1 : 0;
}

template <class A>
inline cudaError_t launch_screen_selftest(int dim, long long n, const double *uc, const double *sig, int *dec,
                                          unsigned char *ref, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((n + 127) / 128);
    if (dim == 2) screen_selftest_kernel<A, 2><<<blocks, 128, 0, st>>>(n, uc, sig, dec, ref);
    else screen_selftest_kernel<A, 3><<<blocks, 128, 0, st>>>(n, uc, sig, dec, ref);
    return cudaPeekAtLastError();
}

// computePolynomials of grid cell g (index inside the grid; field planes of
// the grid are gp.plane apart).  One direction at a time: its neighbours,
// its slopes, their positivity test (the face states of a direction depend
// on its slopes only) and their store; a failed test in any direction sets
// every slope of the cell to zero (order 1), the rest are not evaluated.
template <class A, int DIM>
__device__ __forceinline__ void slopes_cell(const GridParams &gp, const O2Args &oa, long long g)
{
    constexpr int NV = A::NVAR;
    const int nx = gp.n[0], ny = gp.n[1];
    const long long n = gp.plane;
    int idx[3];
    cell_coords(gp, g, idx[0], idx[1], idx[2]);
    double uc[NV];
    load_plain<A>(oa.state, n, g, uc);
    const bool limit = (oa.limit_mode == LIMIT_ALL) || (oa.limit_mode == LIMIT_FLAGGED && oa.flag[g]);
    // positivity fallback, also for the cells a flag leaves on central
    // slopes; decided in FP32 where the margins allow, else in FP64
    const bool screen = limit || oa.limit_mode == LIMIT_FLAGGED;
    bool act = false, ok = true;
    const bool track = oa.active != nullptr;
    // fast arithmetic: the activity threshold as the bit pattern of a non-negative double
    const long long act_thr = (IsExact<A>::value || !track) ? 0 : abs_bits(1e-6 * (fabs(uc[0]) + fabs(uc[NV - 1])));
    // one direction at a time (not unrolled: only one direction's values are live)
#pragma unroll 1
    for (int d = 0; d < DIM; ++d) {
        if (!ok) break;
        double ul[NV], ur[NV], sig[NV];
        const int id = d == 0 ? idx[0] : (d == 1 ? idx[1] : idx[2]);
        const int nd = d == 0 ? gp.n[0] : (d == 1 ? gp.n[1] : gp.n[2]);
        const bool per = (d == 0 ? gp.bc_lo[0] : (d == 1 ? gp.bc_lo[1] : gp.bc_lo[2])) == BC_PERIODIC;
        const long long stride = (d == 0) ? 1 : (d == 1) ? nx : (long long)nx * ny;
        for (int s = 0; s < 2; ++s) {
            double *u = s ? ur : ul;
            const int q = id + (s ? 1 : -1);
            if (q >= 0 && q < nd) {
                load_plain<A>(oa.state, n, g + (s ? stride : -stride), u);
            } else if (per) {
                const long long wrap = (long long)(nd - 1) * stride;
                load_plain<A>(oa.state, n, s ? g - wrap : g + wrap, u);
            } else {
#pragma unroll
                for (int k = 0; k < NV; ++k) u[k] = uc[k];
                const int bc = s ? (d == 0 ? gp.bc_hi[0] : (d == 1 ? gp.bc_hi[1] : gp.bc_hi[2]))
                                 : (d == 0 ? gp.bc_lo[0] : (d == 1 ? gp.bc_lo[1] : gp.bc_lo[2]));
                ghost_in_place<A, true>(bc, d, s ? 1 : -1, u, gp.dir_cons);
            }
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            // the central slope is one difference; the one-sided ones are
            // only needed where the limiter runs
            const double central = IsExact<A>::value ? 0.5 * (ur[k] - ul[k]) : half_ftz(ur[k] - ul[k]);
            double sl = central;
            if (limit) {
                const double a = uc[k] - ul[k];
                const double b = ur[k] - uc[k];
                // the activity is only recorded where a caller keeps it (stage 1)
                if (IsExact<A>::value) {
                    sl = mc_slope<A>(a, b, central);
                    if (track && fabs(sl - central) > 1e-6 * (fabs(uc[0]) + fabs(uc[NV - 1]))) act = true;
                } else {
                    sl = mc_slope_bits(a, b, central);
                    if (track) act |= abs_bits(sl - central) > act_thr;
                }
            }
            sig[k] = sl;
        }
        if (screen) {
            const int dec = screen_dir<A>(uc, sig);
            ok = dec > 0 || (dec < 0 && dir_admissible<A>(uc, sig));
        }
        if (ok) {
#pragma unroll
            for (int k = 0; k < NV; ++k) oa.S[(long long)(d * NV + k) * n + g] = sig[k];
        }
    }
    if (!ok) {
#pragma unroll
        for (int d = 0; d < DIM; ++d)
#pragma unroll
            for (int k = 0; k < NV; ++k) oa.S[(long long)(d * NV + k) * n + g] = 0.0;
        act = true;
    }
    if (oa.active) oa.active[g] = act ? 1 : 0;
}

__device__ __forceinline__ bool o2_step_active(const Ctrl *ctrl, int stage)
{
    if (stage < 1) return true;
    return (stage == 1) ? (ctrl->t < ctrl->t_end) && (ctrl->step < ctrl->max_steps) : ctrl->active != 0;
}

// Blocks per SM the slope kernel is compiled for: four (64 registers) for
// the fast arithmetic, whose one-direction-at-a-time evaluation fits them.
template <class A> struct SlopesMinBlocks { static constexpr int value = 1; };
template <int NV> struct SlopesMinBlocks<FastArithT<NV>> { static constexpr int value = 4; };

// computePolynomials over a grid: one thread per cell (grid-stride).
template <class A, int DIM>
__global__ void __launch_bounds__(256, SlopesMinBlocks<A>::value) slopes_kernel(GridParams gp, O2Args oa)
{
    if (!o2_step_active(oa.ctrl, oa.stage)) return;
    // no block of this launch reads the counter
    if (oa.tick && blockIdx.x == 0 && threadIdx.x == 0) *oa.tick += 1;
    for (long long g = oa.cell0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; g < oa.cell1;
         g += (long long)gridDim.x * blockDim.x)
        slopes_cell<A, DIM>(gp, oa, g);
}

template <class A>
__device__ __forceinline__ double form_w1_value(const StageArgs &sa, const GridParams &gp, const StepScalars &sc,
                                                long long o)
{
    const double u = __ldg(sa.U + o), r = __ldg(sa.R + o);
    return IsExact<A>::value ? u + sc.dt * r / gp.vol : fma(sc.s, r, u);
}

// W1 = U + dt R1 / V (stage 2 input), with the stage-2 dt bookkeeping.
template <class A>
__global__ void __launch_bounds__(256) form_w1_kernel(GridParams gp, StageArgs sa, double *W1)
{
    const StepScalars sc = step_scalars<A, STAGE_2>(gp, sa.ctrl);
    if (blockIdx.x == 0 && threadIdx.x == 0 && sc.active) sa.ctrl->dt = sc.dt;
    if (!sc.active) return;
    const long long n = gp.plane;
#pragma unroll
    for (int k = 0; k < A::NVAR; ++k) {
        const long long base = (long long)A::field(k) * n;
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
            W1[base + i] = form_w1_value<A>(sa, gp, sc, base + i);
    }
}

// ---- face-side records ----------------------------------------------------
// The state a cell (or a ghost) presents on side (d, s) of its faces:
// interior U + s sigma_d / 2 (reconstruction eval, oracle eval_side); a ghost
// across the border of direction d shows the ghost of the neighbouring
// interior cell's face state (euler.cpp:224-225).

// Record for one face side: record() on a face state, keeping direction d only.
template <class A, int DIM>
__device__ __forceinline__ void side_record(const double *c, int d, CellRecV<1, A::NVAR> &out, unsigned *status)
{
    CellRecV<DIM, A::NVAR> full;
#pragma unroll
    for (int k = 0; k < A::NVAR; ++k) full.c[k] = c[k];
    A::template record<DIM>(full, status);
#pragma unroll
    for (int k = 0; k < A::NVAR; ++k) { out.c[k] = full.c[k]; out.f[0][k] = full.f[d][k]; }
    out.lam[0] = full.lam[d];
}

// What a cell's face-side records are made from: the stage state and slopes
// of an interior cell, or the ghost face state of a ghost position (which
// every side of the ghost shows).  The marches keep this for the next row or
// plane (12 doubles in 2D, 20 in 3D) instead of its 4 or 6 records (36, 66)
// and evaluate each record where its face is.
template <class A, int DIM>
struct SideSrc {
    double uc[A::NVAR];
    double sg[DIM][A::NVAR];
    bool ghost;
};

// SideSrc of the cell at (x, y, z), which may be a ghost position.
template <class A, int DIM>
__device__ __forceinline__ void load_src(const GridParams &gp, const double *state, const double *S, int x, int y,
                                         int z, SideSrc<A, DIM> &src)
{
    constexpr int NV = A::NVAR;
    int gx, gy, gz = 0;
    const int ix = resolve_index(x, gp.n[0], gp.bc_lo[0] == BC_PERIODIC, gx);
    const int iy = resolve_index(y, gp.n[1], gp.bc_lo[1] == BC_PERIODIC, gy);
    const int iz = (DIM == 3) ? resolve_index(z, gp.n[2], gp.bc_lo[2] == BC_PERIODIC, gz) : 0;
    const long long n = gp.plane;
    const long long g = (long long)ix + (long long)gp.n[0] * ((long long)iy + (long long)gp.n[1] * iz);
    load_plain<A>(state, n, g, src.uc);
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
        for (int k = 0; k < NV; ++k) src.sg[d][k] = __ldg(S + (long long)(d * NV + k) * n + g);
    const int gh[3] = {gx, gy, gz};
    int gdir = -1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) if (gh[d] != 0 && gdir < 0) gdir = d;
    src.ghost = gdir >= 0;
    if (gdir >= 0) {
        // ghost across the border of direction gdir on side gh[gdir]: the face
        // it shares with the interior cell is on its side -gh[gdir]; the
        // interior face state is on the interior cell's side gh[gdir]
        double gs[NV];
        const double off = gh[gdir] > 0 ? 0.5 : -0.5;
#pragma unroll
        for (int k = 0; k < NV; ++k) gs[k] = face_value<A>(src.uc[k], off, src.sg[gdir][k]);
        ghost_in_place<A, true>(gh[gdir] < 0 ? gp.bc_lo[gdir] : gp.bc_hi[gdir], gdir, gh[gdir], gs, gp.dir_cons);
#pragma unroll
        for (int k = 0; k < NV; ++k) src.uc[k] = gs[k];
    }
}

// Record of side (d, s: 0 = -e_d, 1 = +e_d) of src.  The state checks
// (status) are taken on the + sides of interior cells.
template <class A, int DIM>
__device__ __forceinline__ void side_of(const SideSrc<A, DIM> &src, int d, int s, CellRecV<1, A::NVAR> &out,
                                        unsigned *status)
{
    constexpr int NV = A::NVAR;
    double fs[NV];
    const double off = s ? 0.5 : -0.5;
#pragma unroll
    for (int k = 0; k < NV; ++k) fs[k] = src.ghost ? src.uc[k] : face_value<A>(src.uc[k], off, src.sg[d][k]);
    side_record<A, DIM>(fs, d, out, (s == 1 && !src.ghost) ? status : nullptr);
}

template <class A>
__device__ __forceinline__ double side_face(const CellRecV<1, A::NVAR> &L, const CellRecV<1, A::NVAR> &R, double *F)
{
    return A::face(L.c, L.f[0], L.lam[0], R.c, R.f[0], R.lam[0], F);
}

// x faces of a warp row from the +x record of each lane and the -x record of the next lane
template <class A>
__device__ __forceinline__ double xfaces_o2(const CellRecV<1, A::NVAR> &plus, const CellRecV<1, A::NVAR> &minus,
                                            double *Flo, double *Fhi)
{
    constexpr int NV = A::NVAR;
    CellRecV<1, NV> R;
#pragma unroll
    for (int k = 0; k < NV; ++k) { R.c[k] = shfl_down(minus.c[k], 1); R.f[0][k] = shfl_down(minus.f[0][k], 1); }
    R.lam[0] = shfl_down(minus.lam[0], 1);
    const double lam = side_face<A>(plus, R, Fhi);
#pragma unroll
    for (int k = 0; k < NV; ++k) Flo[k] = shfl_up(Fhi[k], 1);
    return lam;
}

// Output of one cell: stage state from the materialised planes.
template <class A, int STAGE>
__device__ __forceinline__ void store_output_o2(const StageArgs &sa, const GridParams &gp, const StepScalars &sc,
                                                const double *state, long long g, const double *acc)
{
#pragma unroll
    for (int k = 0; k < A::NVAR; ++k) {
        const long long o = (long long)A::field(k) * gp.plane + g;
        const double cs = __ldg(state + o);
        double v;
        if (STAGE == STAGE_RHS || STAGE == STAGE_1) {
            v = acc[k];
        } else if (STAGE == STAGE_2) {
            const double u = __ldg(sa.U + o);
            if (IsExact<A>::value) v = 0.75 * u + 0.25 * (cs + sc.dt * acc[k] / gp.vol);
            else v = fma(0.25, fma(sc.s, acc[k], cs), 0.75 * u);
        } else {
            const double u = sa.U[o];
            if (IsExact<A>::value) v = (1. / 3) * u + (2. / 3) * (cs + sc.dt * acc[k] / gp.vol);
            else v = fma(2.0 / 3.0, fma(sc.s, acc[k], cs), u * (1.0 / 3.0));
        }
        sa.out[o] = v;
    }
}

// ---------------------------------------------------------------- 2D, order 2
// One warp's work item (as march2d, with face-side records).  The next row
// is kept as its state and slopes (SideSrc) and each face-side record is
// evaluated where its face is: the +x and -x records for the x faces, this
// row's +y record and the next row's -y record for the y face.
template <class A, int STAGE>
__device__ __forceinline__ void march2d_o2(const GridParams &gp, const StageArgs &sa, const double *state,
                                           const double *S, const StepScalars &sc, int seg, int chunk, double &lmax,
                                           unsigned &status)
{
    constexpr int NV = A::NVAR;
    const int lane = threadIdx.x & 31;
    const int nx = gp.n[0], ny = gp.n[1];
    const int x = seg * SEG - 1 + lane;
    const int y0 = chunk * gp.chunk;
    const int y1 = min(y0 + gp.chunk, ny);
    const bool out_col = (lane >= 1) && (lane <= SEG) && (x < nx);
    const bool xface_valid = (lane <= SEG) && (x < nx);
    const bool perx = gp.bc_lo[0] == BC_PERIODIC, pery = gp.bc_lo[1] == BC_PERIODIC;
    unsigned *st = (STAGE == STAGE_1 && out_col) ? &status : nullptr;

    SideSrc<A, 2> cur;
    double Fylo[NV], Fyhi[NV], Fxlo[NV], Fxhi[NV], acc[NV];
    {
        CellRecV<1, NV> below, ym;
        {
            SideSrc<A, 2> bl;
            load_src<A, 2>(gp, state, S, x, y0 - 1, 0, bl);
            side_of<A, 2>(bl, 1, 1, below, nullptr);
        }
        load_src<A, 2>(gp, state, S, x, y0, 0, cur);
        side_of<A, 2>(cur, 1, 0, ym, nullptr);
        const double l = side_face<A>(below, ym, Fylo);
        if (out_col) lmax = max_nonneg(lmax, l);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) Fyhi[k] = 0.0;
#pragma unroll 4
    for (int y = y0; y < y1; ++y) {
        {
            CellRecV<1, NV> xp, xm;
            side_of<A, 2>(cur, 0, 1, xp, st);
            side_of<A, 2>(cur, 0, 0, xm, nullptr);
            const double lx = xfaces_o2<A>(xp, xm, Fxlo, Fxhi);
            if (STAGE <= STAGE_1 && xface_valid) lmax = max_nonneg(lmax, lx);
        }
        accumulate_pair<A, true>(acc, Fxlo, Fxhi, gp.area, perx && x == nx - 1);
        {
            CellRecV<1, NV> yp, ym;
            side_of<A, 2>(cur, 1, 1, yp, st);
            load_src<A, 2>(gp, state, S, x, y + 1, 0, cur);
            if (out_col) {   // the halo lanes only provide x-face states
                side_of<A, 2>(cur, 1, 0, ym, nullptr);
                const double ly = side_face<A>(yp, ym, Fyhi);
                if (STAGE <= STAGE_1) lmax = max_nonneg(lmax, ly);
            }
        }
        if (out_col) {
            accumulate_pair<A, false>(acc, Fylo, Fyhi, gp.area, pery && y == ny - 1);
            store_output_o2<A, STAGE>(sa, gp, sc, state, (long long)x + (long long)nx * y, acc);
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) Fylo[k] = Fyhi[k];
    }
}

template <class A, int STAGE>
__global__ void __launch_bounds__(128) stage2d_o2_kernel(GridParams gp, StageArgs sa, const double *state,
                                                         const double *S)
{
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (warp >= gp.nseg * gp.nchunk) return;
    const StepScalars sc = step_scalars<A, STAGE>(gp, sa.ctrl);
    if (gp.bookkeep && blockIdx.x == 0 && threadIdx.x == 0) step_bookkeeping<STAGE>(sa.ctrl, sc);
    if (!sc.active) return;
    double lmax = 0.0;
    unsigned status = 0;
    march2d_o2<A, STAGE>(gp, sa, state, S, sc, warp % gp.nseg, gp.chunk0 + warp / gp.nseg, lmax, status);
    publish_reductions<STAGE>(lmax, status, sa.ctrl, sa.rhs_maxeig);
}

// ---------------------------------------------------------------- 3D, order 2
// The 3D kernel's rows are 32 output columns wide (every lane an output
// cell, so 256 columns take 8 rows exactly); the face sides of the columns
// left and right of a row come from the block's two halo warps.
constexpr int SEG3D_O2 = 32;

template <int BY, int NV>
struct Smem3DO2 {
    double c[BY][NV][32];
    double f[BY][NV][32];
    double lam[BY][32];
    double F[BY][NV][32];
    // x-halo face sides per row: [0] the +x side of the column left of the
    // block, [1] the -x side of the column right of it
    double xc[2][NV][BY], xf[2][NV][BY], xlam[2][BY];
};

// Registers: the next plane is kept as its state and slopes (SideSrc), and
// each face-side record is evaluated where its face is, so that the kernel
// fits 128 registers: one block of 16 warps (or two of 8) per SM.
template <class A, int BY> struct O2Stage3DMinBlocks { static constexpr int value = 1; };
template <int BY> struct O2Stage3DMinBlocks<FastArithT<5>, BY> { static constexpr int value = BY <= 8 ? 2 : 1; };

template <class A, int STAGE, int BY>
__global__ void __launch_bounds__(BY * 32, O2Stage3DMinBlocks<A, BY>::value)
    stage3d_o2_kernel(GridParams gp, StageArgs sa, const double *state, const double *S)
{
    constexpr int NV = A::NVAR;
    __shared__ Smem3DO2<BY, NV> sm;
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const StepScalars sc = step_scalars<A, STAGE>(gp, sa.ctrl);
    if (gp.bookkeep && blockIdx.x == 0 && threadIdx.x == 0) step_bookkeeping<STAGE>(sa.ctrl, sc);
    if (!sc.active) return;

    const int nx = gp.n[0], ny = gp.n[1], nz = gp.n[2];
    int b = blockIdx.x;
    const int seg = b % gp.nseg; b /= gp.nseg;
    const int rb = b % gp.nrowblk; b /= gp.nrowblk;
    const int chunk = gp.chunk0 + b;
    const int x0 = seg * SEG3D_O2;
    const int x = x0 + lane;
    const int y = rb * (BY - 2) - 1 + w;
    const int z0 = chunk * gp.chunk;
    const int z1 = min(z0 + gp.chunk, nz);
    const bool halo_lo = (w == 0), halo_hi = (w == BY - 1);
    const bool out_row = !halo_lo && !halo_hi && (y < ny);
    const bool out_col = x < nx;
    const bool out = out_row && out_col;
    const bool perx = gp.bc_lo[0] == BC_PERIODIC, pery = gp.bc_lo[1] == BC_PERIODIC,
               perz = gp.bc_lo[2] == BC_PERIODIC;
    // rows past the one beyond the grid's last row (the overhang of the last
    // row block) only take part in the block's barriers
    const bool idle = y > ny;
    unsigned status = 0;
    unsigned *st = (STAGE == STAGE_1 && out) ? &status : nullptr;
    double lmax = 0.0;

    // The x-halo face sides of the output rows of plane zz, by the halo
    // warps: lane r of the low one the +x side of the cell left of row r, of
    // the high one the -x side of the cell right of it.  Written for plane
    // z + 1 between the second and third barriers of plane z, read before the
    // first barrier of plane z + 1.
    auto x_halo = [&](int zz) {
        const int yr = rb * (BY - 2) - 1 + lane;
        if (lane >= 1 && lane <= BY - 2 && yr < ny) {
            const int side = halo_lo ? 0 : 1;
            CellRecV<1, NV> xr;
            {
                SideSrc<A, 3> h;
                load_src<A, 3>(gp, state, S, halo_lo ? x0 - 1 : x0 + SEG3D_O2, yr, zz, h);
                side_of<A, 3>(h, 0, halo_lo ? 1 : 0, xr, nullptr);
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) { sm.xc[side][k][lane] = xr.c[k]; sm.xf[side][k][lane] = xr.f[0][k]; }
            sm.xlam[side][lane] = xr.lam[0];
        }
    };

    SideSrc<A, 3> cur;
    double Fzlo[NV], Fzhi[NV], Fa[NV], Fb[NV], acc[NV];
    if (halo_lo || halo_hi) x_halo(z0);
    __syncthreads();
    if (!halo_lo && !halo_hi && !idle) {
        CellRecV<1, NV> below, zm;
        {
            SideSrc<A, 3> bl;
            load_src<A, 3>(gp, state, S, x, y, z0 - 1, bl);
            side_of<A, 3>(bl, 2, 1, below, nullptr);
        }
        load_src<A, 3>(gp, state, S, x, y, z0, cur);
        side_of<A, 3>(cur, 2, 0, zm, nullptr);
        const double l = side_face<A>(below, zm, Fzlo);
        if (out) lmax = max_nonneg(lmax, l);
    }
    for (int z = z0; z < z1; ++z) {
        if (idle) {   // the three barriers of a plane (an idle high halo warp still makes the x halo)
            __syncthreads();
            __syncthreads();
            if (halo_hi && z + 1 < z1) x_halo(z + 1);
            __syncthreads();
            continue;
        }
        if (halo_lo || halo_hi) {
            // the face side this halo row shows to the block: +y for the row below, -y above
            CellRecV<1, NV> hr;
            {
                SideSrc<A, 3> h;
                load_src<A, 3>(gp, state, S, x, y, z, h);
                side_of<A, 3>(h, 1, halo_lo ? 1 : 0, hr, nullptr);
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) { sm.c[w][k][lane] = hr.c[k]; sm.f[w][k][lane] = hr.f[0][k]; }
            sm.lam[w][lane] = hr.lam[0];
            __syncthreads();
            if (halo_hi) {
                CellRecV<1, NV> L;
#pragma unroll
                for (int k = 0; k < NV; ++k) { L.c[k] = sm.c[w - 1][k][lane]; L.f[0][k] = sm.f[w - 1][k][lane]; }
                L.lam[0] = sm.lam[w - 1][lane];
                const double ly = side_face<A>(L, hr, Fa);
#pragma unroll
                for (int k = 0; k < NV; ++k) sm.F[w][k][lane] = Fa[k];
                if (STAGE <= STAGE_1 && out_col && y - 1 < ny) lmax = max_nonneg(lmax, ly);
            }
            __syncthreads();
            if (z + 1 < z1) x_halo(z + 1);   // read after the next plane's start
            __syncthreads();
            continue;
        }
        // x faces: the right one with the next lane's -x side (lane 31: the
        // right halo column's), the left one the previous lane's right face
        // (lane 0: evaluated with the left halo column's +x side)
        {
            CellRecV<1, NV> xp, xm, R;
            side_of<A, 3>(cur, 0, 1, xp, st);
            side_of<A, 3>(cur, 0, 0, xm, nullptr);
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double c = shfl_down(xm.c[k], 1), f = shfl_down(xm.f[0][k], 1);
                R.c[k] = lane == 31 ? sm.xc[1][k][w] : c;
                R.f[0][k] = lane == 31 ? sm.xf[1][k][w] : f;
            }
            const double lr = shfl_down(xm.lam[0], 1);
            R.lam[0] = lane == 31 ? sm.xlam[1][w] : lr;
            const double lx = side_face<A>(xp, R, Fb);
            if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, lx);
#pragma unroll
            for (int k = 0; k < NV; ++k) Fa[k] = shfl_up(Fb[k], 1);
            if (lane == 0) {
                CellRecV<1, NV> L;
#pragma unroll
                for (int k = 0; k < NV; ++k) { L.c[k] = sm.xc[0][k][w]; L.f[0][k] = sm.xf[0][k][w]; }
                L.lam[0] = sm.xlam[0][w];
                const double ll = side_face<A>(L, xm, Fa);
                if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, ll);
            }
        }
        accumulate_pair<A, true>(acc, Fa, Fb, gp.area, perx && x == nx - 1);
        // y faces: rows publish their +y side, each row evaluates the face below it
        {
            CellRecV<1, NV> yp;
            side_of<A, 3>(cur, 1, 1, yp, st);
#pragma unroll
            for (int k = 0; k < NV; ++k) { sm.c[w][k][lane] = yp.c[k]; sm.f[w][k][lane] = yp.f[0][k]; }
            sm.lam[w][lane] = yp.lam[0];
        }
        __syncthreads();
        {
            CellRecV<1, NV> L, ym;
            side_of<A, 3>(cur, 1, 0, ym, nullptr);
#pragma unroll
            for (int k = 0; k < NV; ++k) { L.c[k] = sm.c[w - 1][k][lane]; L.f[0][k] = sm.f[w - 1][k][lane]; }
            L.lam[0] = sm.lam[w - 1][lane];
            const double ly = side_face<A>(L, ym, Fa);
#pragma unroll
            for (int k = 0; k < NV; ++k) sm.F[w][k][lane] = Fa[k];
            if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, ly);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NV; ++k) Fb[k] = sm.F[w + 1][k][lane];
        accumulate_pair<A, false>(acc, Fa, Fb, gp.area, pery && y == ny - 1);
        // z face above: this plane's +z side, the next plane's -z side
        {
            CellRecV<1, NV> zp, zm;
            side_of<A, 3>(cur, 2, 1, zp, st);
            load_src<A, 3>(gp, state, S, x, y, z + 1, cur);
            side_of<A, 3>(cur, 2, 0, zm, nullptr);
            const double lz = side_face<A>(zp, zm, Fzhi);
            if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, lz);
        }
        if (out) {
            accumulate_pair<A, false>(acc, Fzlo, Fzhi, gp.area, perz && z == nz - 1);
            store_output_o2<A, STAGE>(sa, gp, sc, state,
                                      (long long)x + (long long)nx * ((long long)y + (long long)ny * z), acc);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NV; ++k) Fzlo[k] = Fzhi[k];
    }
    if (STAGE <= STAGE_1) {
        lmax = warp_max(lmax);
        if (lane == 0) {
            unsigned long long *dst = (STAGE == STAGE_RHS) ? (unsigned long long *)sa.rhs_maxeig
                                                           : &sa.ctrl->maxeig_bits;
            atomicMax(dst, (unsigned long long)dbits(lmax));
        }
        if (STAGE == STAGE_1) {
            status = __reduce_or_sync(0xffffffffu, status);
            if (lane == 0 && status) atomicOr(&sa.ctrl->status, status);
        }
    }
}

} // namespace mmf
