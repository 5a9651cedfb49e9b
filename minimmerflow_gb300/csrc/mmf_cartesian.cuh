// mmf_cartesian.cuh -- fused SSP-RK3 stage kernels on a uniform Cartesian grid
// (order-1 reconstruction), FP64, structure-of-arrays state.
//
// One launch per Runge-Kutta stage computes, for every cell it owns, the
// residual of euler::computeRHS (euler.cpp:127-249) and applies the stage
// combination of main.cpp:409-495, so the residual never round-trips HBM
// except between stage 1 and stage 2 (dt is only known after stage 1's
// maxEig reduction):
//   stage 1:  R1 = RHS(U);                       maxEig -> ctrl (atomicMax)
//   stage 2:  W1 = U + dt R1 / V (recomputed on the fly, halo included)
//             W2 = 3/4 U + 1/4 (W1 + dt RHS(W1) / V)
//   stage 3:  U  = 1/3 U + 2/3 (W2 + dt RHS(W2) / V)      (in place)
// 320 bytes of HBM traffic per cell and step (8 reads/writes x 5 fields x 8 B).
//
// Work decomposition.  A warp owns 30 consecutive cells of a grid row and
// evaluates 32 (one halo cell each side), so x-face states move between lanes
// by shuffles.  In 2D the warp marches up the rows of a chunk and carries the
// previous row's record and y-face flux in registers; in 3D a block stacks
// BY warps in y (halo rows at both ends exchange through shared memory) and
// marches along z.  Each face flux is evaluated once per owning warp.
//
// Per-cell accumulation order is the reference's: for each direction, the
// low face then the high face (the interface list is x-faces, y-faces,
// z-faces), except that a periodic wrap face comes first for the last cell
// of the line.  Border faces are evaluated as split(ghost, U, +e_d), which
// is the exact negation of the reference's split(U, ghost, -e_d).
#pragma once

#include "mmf_physics.cuh"

namespace mmf {

struct Ctrl {
    double t;
    double t_end;
    double dt;
    double cfl_h;                   // 0.9 * cfl * minCellSize   (main.cpp:398)
    unsigned long long maxeig_bits; // stage-1 max eigenvalue (non-negative double bits)
    long long step;
    long long max_steps;
    int active;                     // this step runs (t < t_end and step < max_steps)
    unsigned status;                // bit0 rho<0, bit1 p<0, bit2 NaN
    double last_maxeig;             // stage-1 maxEig of the last step (log)
    double *log;                    // optional step log: per step (maxEig, dt, t after the step)
    long long log_cap;              // entries of the log ring (step % log_cap)
};

struct GridParams {
    int dim;
    int n[3];
    int bc_lo[3], bc_hi[3];
    double dir_cons[NF];   // Dirichlet ghost state (conservative, dirichlet_conservatives)
    double area, vol;
    double half_area_per_vol;   // 0.5 area / vol: the fast arithmetic's stage scale per unit dt
    int chunk;      // rows (2D) / planes (3D) per marching chunk
    int nseg;       // x segments of 30 cells
    int nrowblk;    // 3D: row blocks in y
    int nchunk;     // chunks covered by one launch
    int chunk0;     // first chunk of the launch (a launch may cover a band of the grid)
    int bookkeep;   // this launch updates the control block (exactly one launch per stage)
    int wpb;        // 2D: warps per block
    int tile3d;     // 3D order 1: 0 = row-block kernel, 1 = 32 x 8 tile kernel with one block per tile and
                    // chunk, 2 = the tile kernel on at most one block per resident slot
    int unit;       // tile3d 2: planes per (column, unit) work unit (a band launch keeps the whole grid's)
    long long plane;  // cells per field plane
};

struct StageArgs {
    const double *U;     // state at the start of the step
    const double *R;     // stage-1 residual
    const double *W;     // stage-2 result
    double *out;         // this stage's output
    Ctrl *ctrl;
    double *rhs_maxeig;  // stage 0 (residual only): max eigenvalue output
};

constexpr int SEG = 30;   // output cells per warp row

// Grid coordinates of cell g (x fastest).  Grids of fewer than 2^32 cells
// take 32-bit unsigned division: a 64-bit integer division by a run-time
// divisor is a sequence of FP64 reciprocal steps, dear on this GPU.
__device__ __forceinline__ void cell_coords(const GridParams &gp, long long g, int &x, int &y, int &z)
{
    if (gp.plane <= 0xffffffffll) {
        const unsigned u = (unsigned)g, nx = (unsigned)gp.n[0], ny = (unsigned)gp.n[1];
        const unsigned q = u / nx;
        x = (int)(u - q * nx);
        y = (int)(q % ny);
        z = (int)(q / ny);
    } else {
        const long long q = g / gp.n[0];
        x = (int)(g - q * gp.n[0]);
        y = (int)(q % gp.n[1]);
        z = (int)(q / gp.n[1]);
    }
}

enum { STAGE_RHS = 0, STAGE_1 = 1, STAGE_2 = 2, STAGE_3 = 3 };

template <class A> struct IsExact { static constexpr bool value = false; };
template <> struct IsExact<ExactArith> { static constexpr bool value = true; };

template <class A, int DIM>
using RecOf = CellRecV<DIM, A::NVAR>;

__device__ __forceinline__ double shfl_down(double v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
__device__ __forceinline__ double shfl_up(double v, int d) { return __shfl_up_sync(0xffffffffu, v, d); }

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Per-launch step scalars.
struct StepScalars {
    double dt;     // time step (stages 2, 3)
    double s;      // stage scale: exact dt (then / V), fast 0.5*A*dt/V
    bool active;
};

template <class A, int STAGE>
__device__ __forceinline__ StepScalars step_scalars(const GridParams &gp, const Ctrl *ctrl)
{
    StepScalars sc;
    sc.dt = 0.0;
    sc.s = 0.0;
    if (STAGE == STAGE_RHS) { sc.active = true; return sc; }
    if (STAGE == STAGE_1) {
        sc.active = (ctrl->t < ctrl->t_end) && (ctrl->step < ctrl->max_steps);
        return sc;
    }
    sc.active = ctrl->active != 0;
    if (STAGE == STAGE_2) {
        // main.cpp:398-402
        double maxEig = bitsd((long long)ctrl->maxeig_bits);
        double dt = ctrl->cfl_h / maxEig;
        if (ctrl->t + dt > ctrl->t_end) dt = ctrl->t_end - ctrl->t;
        sc.dt = dt;
    } else {
        sc.dt = ctrl->dt;
    }
    sc.s = IsExact<A>::value ? sc.dt : sc.dt * gp.half_area_per_vol;
    return sc;
}

// Control-block updates made once per launch by thread 0 of block 0.  No
// other block of the same launch reads the fields written here: stage 2 and
// stage 3 read only 'active' and 'dt' (stage 2 recomputes dt from maxEig).
template <int STAGE>
__device__ __forceinline__ void step_bookkeeping(Ctrl *ctrl, const StepScalars &sc)
{
    if (STAGE == STAGE_1) ctrl->active = sc.active ? 1 : 0;
    if (!sc.active) return;
    if (STAGE == STAGE_2) ctrl->dt = sc.dt;
    if (STAGE == STAGE_3) {
        // main.cpp:399-404: the step's maxEig, dt and new time, as the reference logs them
        if (ctrl->log) {
            double *e = ctrl->log + 3 * (ctrl->step % ctrl->log_cap);
            e[0] = bitsd((long long)ctrl->maxeig_bits);
            e[1] = sc.dt;
            e[2] = ctrl->t + sc.dt;
        }
        // main.cpp:505-506; the stage-1 reduction slot is cleared for the next step
        ctrl->last_maxeig = bitsd((long long)ctrl->maxeig_bits);
        ctrl->t += sc.dt;
        ctrl->step += 1;
        ctrl->maxeig_bits = 0ull;
    }
}

// Stage input state of grid cell g.
template <class A, int STAGE>
__device__ __forceinline__ void load_state(const StageArgs &sa, const GridParams &gp, const StepScalars &sc,
                                           long long g, double *c)
{
#pragma unroll
    for (int k = 0; k < A::NVAR; ++k) {
        const long long o = (long long)A::field(k) * gp.plane + g;
        if (STAGE == STAGE_2) {
            const double u = __ldg(sa.U + o), r = __ldg(sa.R + o);
            if (IsExact<A>::value) c[k] = u + sc.dt * r / gp.vol;   // main.cpp:421
            else c[k] = fma(sc.s, r, u);
        } else if (STAGE == STAGE_3) {
            c[k] = __ldg(sa.W + o);
        } else {
            c[k] = __ldg(sa.U + o);
        }
    }
}

// Stage output of grid cell g from its residual accumulator and stage state.
// Fast stage 2 uses W2 = 3/4 U + 1/4 (W1 + s R2) = U + s/4 (R1 + R2), which
// is the same combination with W1 = U + s R1 substituted.
template <class A, int STAGE>
__device__ __forceinline__ void store_output(const StageArgs &sa, const GridParams &gp, const StepScalars &sc,
                                             long long g, const double *acc, const double *cstate)
{
#pragma unroll
    for (int k = 0; k < A::NVAR; ++k) {
        const long long o = (long long)A::field(k) * gp.plane + g;
        double v;
        if (STAGE == STAGE_RHS || STAGE == STAGE_1) {
            v = acc[k];
        } else if (STAGE == STAGE_2) {
            const double u = __ldg(sa.U + o);
            if (IsExact<A>::value) v = 0.75 * u + 0.25 * (cstate[k] + sc.dt * acc[k] / gp.vol); // main.cpp:457
            else v = fma(0.25 * sc.s, __ldg(sa.R + o) + acc[k], u);
        } else {
            const double u = sa.out[o];   // in place: U
            if (IsExact<A>::value) v = (1. / 3) * u + (2. / 3) * (cstate[k] + sc.dt * acc[k] / gp.vol); // main.cpp:493
            else v = fma(2.0 / 3.0, fma(sc.s, acc[k], cstate[k]), u * (1.0 / 3.0));
        }
        sa.out[o] = v;
    }
}

// Adds the two faces of direction d to the accumulator in reference order.
// The first pair of a cell starts the accumulator: the reference starts from
// 0.0 (euler.cpp:142-148), which the reference arithmetic keeps so that signed
// zeros match too; the fast arithmetic starts from the first difference.
template <class A, bool FIRST>
__device__ __forceinline__ void accumulate_pair(double *acc, const double *Flo, const double *Fhi, double area,
                                                bool hi_first)
{
#pragma unroll
    for (int k = 0; k < A::NVAR; ++k) {
        if (IsExact<A>::value) {
            if (FIRST) acc[k] = 0.0;
            if (hi_first) { acc[k] = acc[k] - area * Fhi[k]; acc[k] = acc[k] + area * Flo[k]; }
            else { acc[k] = acc[k] + area * Flo[k]; acc[k] = acc[k] - area * Fhi[k]; }
        } else {
            if (FIRST) acc[k] = Flo[k] - Fhi[k];
            else acc[k] += Flo[k] - Fhi[k];
        }
    }
}

// Column (or row) index along one direction with border handling:
// returns the interior index to load and sets ghost = -1/+1 for a border ghost.
__device__ __forceinline__ int resolve_index(int i, int n, bool periodic, int &ghost)
{
    ghost = 0;
    if (i < 0) {
        if (periodic) return n - 1;
        ghost = -1;
        return 0;
    }
    if (i >= n) {
        if (periodic) return (i - n < n) ? i - n : n - 1;
        if (i == n) ghost = 1;
        return n - 1;
    }
    return i;
}

// Record of the cell at (x, y, z) (may be a ghost) for this stage.
template <class A, int STAGE, int DIM>
__device__ __forceinline__ void load_record(const StageArgs &sa, const GridParams &gp, const StepScalars &sc,
                                            int x, int y, int z, RecOf<A, DIM> &r, unsigned *status)
{
    int gx, gy, gz = 0;
    const int ix = resolve_index(x, gp.n[0], gp.bc_lo[0] == BC_PERIODIC, gx);
    const int iy = resolve_index(y, gp.n[1], gp.bc_lo[1] == BC_PERIODIC, gy);
    const int iz = (DIM == 3) ? resolve_index(z, gp.n[2], gp.bc_lo[2] == BC_PERIODIC, gz) : 0;
    const long long g = (long long)ix + (long long)gp.n[0] * ((long long)iy + (long long)gp.n[1] * iz);
    load_state<A, STAGE>(sa, gp, sc, g, r.c);
    const bool ghost = (gx | gy | gz) != 0;
    if (ghost) {
        if (gx) ghost_in_place<A>(gx < 0 ? gp.bc_lo[0] : gp.bc_hi[0], 0, gx, r.c, gp.dir_cons);
        if (gy) ghost_in_place<A>(gy < 0 ? gp.bc_lo[1] : gp.bc_hi[1], 1, gy, r.c, gp.dir_cons);
        if (DIM == 3 && gz) ghost_in_place<A>(gz < 0 ? gp.bc_lo[2] : gp.bc_hi[2], 2, gz, r.c, gp.dir_cons);
    }
    A::template record<DIM>(r, ghost ? nullptr : status);
}

// Face between record L (this lane) and record R along direction d.
template <class A, int DIM>
__device__ __forceinline__ double face_dir(const RecOf<A, DIM> &L, const RecOf<A, DIM> &R, int d, double *F)
{
    return A::face(L.c, L.f[d], L.lam[d], R.c, R.f[d], R.lam[d], F);
}

// x-faces of a warp row: Fhi = face(lane, lane+1), Flo = face(lane-1, lane).
template <class A, int DIM>
__device__ __forceinline__ double xfaces(const RecOf<A, DIM> &r, double *Flo, double *Fhi)
{
    constexpr int NV = A::NVAR;
    double cR[NV], fR[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) { cR[k] = shfl_down(r.c[k], 1); fR[k] = shfl_down(r.f[0][k], 1); }
    const double lamR = shfl_down(r.lam[0], 1);
    const double lam = A::face(r.c, r.f[0], r.lam[0], cR, fR, lamR, Fhi);
#pragma unroll
    for (int k = 0; k < NV; ++k) Flo[k] = shfl_up(Fhi[k], 1);
    return lam;
}

// ---------------------------------------------------------------- 2D kernel
// One warp's work item: 30 output columns (segment 'seg') over the rows of
// chunk 'chunk' of the grid described by gp; sa holds the grid's planes
// (field stride gp.plane).  Returns the item's maximum face eigenvalue (stage
// 1 / residual only) and its status bits.
template <class A, int STAGE>
__device__ __forceinline__ void march2d(const GridParams &gp, const StageArgs &sa, const StepScalars &sc, int seg,
                                        int chunk, double &lmax, unsigned &status)
{
    const int lane = threadIdx.x & 31;
    const int nx = gp.n[0], ny = gp.n[1];
    const int x = seg * SEG - 1 + lane;
    const int y0 = chunk * gp.chunk;
    const int y1 = min(y0 + gp.chunk, ny);
    const bool out_col = (lane >= 1) && (lane <= SEG) && (x < nx);
    const bool xface_valid = (lane <= SEG) && (x < nx);
    const bool perx = gp.bc_lo[0] == BC_PERIODIC, pery = gp.bc_lo[1] == BC_PERIODIC;
    unsigned *st = (STAGE == STAGE_1 && out_col) ? &status : nullptr;

    constexpr int NV = A::NVAR;
    RecOf<A, 2> cur, abv;
    double Fylo[NV], Fyhi[NV], Fxlo[NV], Fxhi[NV], acc[NV];
    load_record<A, STAGE, 2>(sa, gp, sc, x, y0 - 1, 0, abv, nullptr);
    load_record<A, STAGE, 2>(sa, gp, sc, x, y0, 0, cur, st);
    {
        const double l = face_dir<A, 2>(abv, cur, 1, Fylo);
        if (out_col) lmax = max_nonneg(lmax, l);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) Fyhi[k] = 0.0;
    // unrolled so that the FP64 work of consecutive rows interleaves (the
    // fast unit is built without implicit contraction, so the bits do not
    // depend on the unrolling)
#pragma unroll 4
    for (int y = y0; y < y1; ++y) {
        // x faces of row y (the cell's x pair opens the accumulator)
        const double lx = xfaces<A, 2>(cur, Fxlo, Fxhi);
        if (STAGE <= STAGE_1 && xface_valid) lmax = max_nonneg(lmax, lx);
        accumulate_pair<A, true>(acc, Fxlo, Fxhi, gp.area, perx && x == nx - 1);
        // row y+1 and the y face between y and y+1 (output lanes only: the
        // halo lanes only provide x-face states)
        load_record<A, STAGE, 2>(sa, gp, sc, x, y + 1, 0, abv, (y + 1 < y1) ? st : nullptr);
        if (out_col) {
            const double ly = face_dir<A, 2>(cur, abv, 1, Fyhi);
            if (STAGE <= STAGE_1) lmax = max_nonneg(lmax, ly);
            accumulate_pair<A, false>(acc, Fylo, Fyhi, gp.area, pery && y == ny - 1);
            store_output<A, STAGE>(sa, gp, sc, (long long)x + (long long)nx * y, acc, cur.c);
        }
        cur = abv;
#pragma unroll
        for (int k = 0; k < NV; ++k) Fylo[k] = Fyhi[k];
    }
}

// Warp-level publication of an item's max eigenvalue and status bits.
template <int STAGE>
__device__ __forceinline__ void publish_reductions(double lmax, unsigned status, Ctrl *ctrl, double *rhs_maxeig)
{
    if (STAGE > STAGE_1) return;
    const int lane = threadIdx.x & 31;
    lmax = warp_max(lmax);
    if (lane == 0) {
        unsigned long long *dst = (STAGE == STAGE_RHS) ? (unsigned long long *)rhs_maxeig : &ctrl->maxeig_bits;
        atomicMax(dst, (unsigned long long)dbits(lmax));
    }
    if (STAGE == STAGE_1) {
        status = __reduce_or_sync(0xffffffffu, status);
        if (lane == 0 && status) atomicOr(&ctrl->status, status);
    }
}

template <class A, int STAGE>
__global__ void __launch_bounds__(128) stage2d_kernel(GridParams gp, StageArgs sa)
{
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (warp >= gp.nseg * gp.nchunk) return;
    const StepScalars sc = step_scalars<A, STAGE>(gp, sa.ctrl);
    if (gp.bookkeep && blockIdx.x == 0 && threadIdx.x == 0) step_bookkeeping<STAGE>(sa.ctrl, sc);
    if (!sc.active) return;
    double lmax = 0.0;
    unsigned status = 0;
    march2d<A, STAGE>(gp, sa, sc, warp % gp.nseg, gp.chunk0 + warp / gp.nseg, lmax, status);
    publish_reductions<STAGE>(lmax, status, sa.ctrl, sa.rhs_maxeig);
}

// ---------------------------------------------------------------- 3D kernel
// Block = BY warps stacked in y, rows y0-1 .. y0+BY-2, marching along z.
// Warp 0 and warp BY-1 are halo rows: they only provide the y-face state of
// their row (and warp BY-1 evaluates the y face below it); warps 1..BY-2
// own the output rows.  Per plane: x faces (shuffles), y faces (shared
// memory), then the next plane's record and the z face.
template <int BY, int NV>
struct Smem3D {
    double c[BY][NV][32];
    double f[BY][NV][32];
    double lam[BY][32];
    double F[BY][NV][32];   // F[w] = face between rows w-1 and w
};

template <class A, int STAGE, int BY>
__global__ void __launch_bounds__(BY * 32) stage3d_kernel(GridParams gp, StageArgs sa)
{
    constexpr int NV = A::NVAR;
    __shared__ Smem3D<BY, NV> sm;
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
    const int x = seg * SEG - 1 + lane;
    const int y = rb * (BY - 2) - 1 + w;
    const int z0 = chunk * gp.chunk;
    const int z1 = min(z0 + gp.chunk, nz);
    const bool halo_lo = (w == 0), halo_hi = (w == BY - 1);
    const bool out_row = !halo_lo && !halo_hi && (y < ny);
    const bool out_col = (lane >= 1) && (lane <= SEG) && (x < nx);
    const bool out = out_row && out_col;
    const bool perx = gp.bc_lo[0] == BC_PERIODIC, pery = gp.bc_lo[1] == BC_PERIODIC,
               perz = gp.bc_lo[2] == BC_PERIODIC;
    // rows past the one beyond the grid's last row (the overhang of the last
    // row block) only take part in the block's barriers
    const bool idle = y > ny;
    unsigned status = 0;
    unsigned *st = (STAGE == STAGE_1 && out) ? &status : nullptr;
    double lmax = 0.0;

    RecOf<A, 3> cur, abv;
    double Fzlo[NV], Fzhi[NV], Fa[NV], Fb[NV], acc[NV];
    if (!halo_lo && !halo_hi && !idle) {
        load_record<A, STAGE, 3>(sa, gp, sc, x, y, z0 - 1, abv, nullptr);
        load_record<A, STAGE, 3>(sa, gp, sc, x, y, z0, cur, st);
        const double l = face_dir<A, 3>(abv, cur, 2, Fzlo);
        if (out) lmax = max_nonneg(lmax, l);
    }
    for (int z = z0; z < z1; ++z) {
        if (idle) {   // the three barriers of a plane
            __syncthreads();
            __syncthreads();
            __syncthreads();
            continue;
        }
        if (halo_lo || halo_hi) {
            // halo row: y-face state only (the compiler drops the unused fluxes)
            RecOf<A, 3> h;
            load_record<A, STAGE, 3>(sa, gp, sc, x, y, z, h, nullptr);
#pragma unroll
            for (int k = 0; k < NV; ++k) { sm.c[w][k][lane] = h.c[k]; sm.f[w][k][lane] = h.f[1][k]; }
            sm.lam[w][lane] = h.lam[1];
            __syncthreads();
            if (halo_hi) {
                double cL[NV], fL[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) { cL[k] = sm.c[w - 1][k][lane]; fL[k] = sm.f[w - 1][k][lane]; }
                const double ly = A::face(cL, fL, sm.lam[w - 1][lane], h.c, h.f[1], h.lam[1], Fa);
#pragma unroll
                for (int k = 0; k < NV; ++k) sm.F[w][k][lane] = Fa[k];
                if (STAGE <= STAGE_1 && out_col && y - 1 < ny) lmax = max_nonneg(lmax, ly);
            }
            __syncthreads();
            __syncthreads();
            continue;
        }
        // x faces of plane z
        const double lx = xfaces<A, 3>(cur, Fa, Fb);
        if (STAGE <= STAGE_1 && out_row && lane <= SEG && x < nx) lmax = max_nonneg(lmax, lx);
        accumulate_pair<A, true>(acc, Fa, Fb, gp.area, perx && x == nx - 1);
        // y faces through shared memory: this warp evaluates the face below its row
#pragma unroll
        for (int k = 0; k < NV; ++k) { sm.c[w][k][lane] = cur.c[k]; sm.f[w][k][lane] = cur.f[1][k]; }
        sm.lam[w][lane] = cur.lam[1];
        __syncthreads();
        {
            double cL[NV], fL[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) { cL[k] = sm.c[w - 1][k][lane]; fL[k] = sm.f[w - 1][k][lane]; }
            const double ly = A::face(cL, fL, sm.lam[w - 1][lane], cur.c, cur.f[1], cur.lam[1], Fa);
#pragma unroll
            for (int k = 0; k < NV; ++k) sm.F[w][k][lane] = Fa[k];
            if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, ly);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < NV; ++k) Fb[k] = sm.F[w + 1][k][lane];
        accumulate_pair<A, false>(acc, Fa, Fb, gp.area, pery && y == ny - 1);
        // plane z+1 and the z face
        load_record<A, STAGE, 3>(sa, gp, sc, x, y, z + 1, abv, (z + 1 < z1) ? st : nullptr);
        const double lz = face_dir<A, 3>(cur, abv, 2, Fzhi);
        if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, lz);
        if (out) {
            accumulate_pair<A, false>(acc, Fzlo, Fzhi, gp.area, perz && z == nz - 1);
            store_output<A, STAGE>(sa, gp, sc, (long long)x + (long long)nx * ((long long)y + (long long)ny * z),
                                   acc, cur.c);
        }
        __syncthreads();
        cur = abv;
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

// ---------------------------------------------------------- 3D tile kernel
// Block = 8 warps over a tile of 32 x 8 cells (x = lane, y = warp) that
// marches along z, two blocks per SM (128 registers a thread), so that one
// block computes while the other waits at a barrier; one block of 16 warps
// over 32 x 16 cells per SM, with half the halo records per cell, ran the
// 256^3 vortex 3% slower.  Every lane and warp owns an output cell, so tiles
// divide 256-cell grid lines exactly.  The records the tile's faces need from the
// four neighbouring lines (the column left and right of the tile, the row
// below and above it) are evaluated once per plane by three warps in one
// extra pass each (x or y part only), and the faces on the tile's left,
// right and bottom edges by two more warps; every other face is evaluated
// once, by the cell on its low side: x faces move between lanes by shuffles,
// y faces go through shared memory, z faces stay in registers along the march.
//
// Two barriers per plane: (A) the plane's records are in shared memory,
// (B) its faces are.  The next plane's records and halo records are written
// after (B), during the update of this plane: every read of the record slots
// happens between (A) and (B), and every read of the face slots between (B)
// and the next (A), so no third barrier is needed.  The extra passes sit on
// different SM sub-partitions (warp w runs on sub-partition w % 4): the halo
// records on 1, 2 and 3 (between (B) and (A)), the edge faces on 0 and 3
// (between (A) and (B)).
constexpr int TILE_X = 32, TILE_Y = 8;
static_assert(TILE_Y == 8 || TILE_Y == 16, "tile rows: 8 (two blocks per SM) or 16 (one)");
constexpr int TILE_MIN_BLOCKS = TILE_Y == 8 ? 2 : 1;   // blocks per SM the register cap is for
constexpr int TW_TOP = 5, TW_BOT = 6, TW_SIDE = 7;   // warps of the halo-record passes
constexpr int TW_BOTF = 4, TW_LEFTF = 3;             // warps of the edge-face passes

template <int NV>
struct SmemTile {
    double yc[TILE_Y + 1][NV][32];   // y-face side (state, y flux, y speed) of the rows and the top halo row
    double yf[TILE_Y + 1][NV][32];
    double ylam[TILE_Y + 1][32];
    double bc[NV][32], bf[NV][32], blam[32];                        // bottom halo row
    double xc[2][NV][TILE_Y], xf[2][NV][TILE_Y], xlam[2][TILE_Y];    // left [0] / right [1] halo column
    double c0[NV][TILE_Y], f0[NV][TILE_Y], lam0[TILE_Y];            // column 0 of the tile (x side)
    double c31[NV][TILE_Y], f31[NV][TILE_Y], lam31[TILE_Y];         // column 31 of the tile (x side)
    double Fy[TILE_Y][NV][32];       // y face above row w
    double Fl[NV][TILE_Y];           // x face on the tile's left edge, row w
    double Fr[NV][TILE_Y];           // x face on the tile's right edge, row w
    double Fb[NV][32];               // y face on the tile's bottom edge, column l
};

// The halo records of plane z (the x or y part their faces use), by the
// three halo warps.
template <class A, int STAGE>
__device__ __forceinline__ void tile_halo_records(const StageArgs &sa, const GridParams &gp, const StepScalars &sc,
                                                  SmemTile<A::NVAR> &sm, int w, int l, int x0, int y0, int z)
{
    constexpr int NV = A::NVAR;
    if (w == TW_TOP || w == TW_BOT) {
        RecOf<A, 3> h;
        load_record<A, STAGE, 3>(sa, gp, sc, x0 + l, w == TW_TOP ? y0 + TILE_Y : y0 - 1, z, h, nullptr);
        if (w == TW_TOP) {
#pragma unroll
            for (int k = 0; k < NV; ++k) { sm.yc[TILE_Y][k][l] = h.c[k]; sm.yf[TILE_Y][k][l] = h.f[1][k]; }
            sm.ylam[TILE_Y][l] = h.lam[1];
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) { sm.bc[k][l] = h.c[k]; sm.bf[k][l] = h.f[1][k]; }
            sm.blam[l] = h.lam[1];
        }
    } else if (w == TW_SIDE && l < 2 * TILE_Y) {
        const int side = l / TILE_Y, r = l % TILE_Y;
        RecOf<A, 3> h;
        load_record<A, STAGE, 3>(sa, gp, sc, side ? x0 + TILE_X : x0 - 1, y0 + r, z, h, nullptr);
#pragma unroll
        for (int k = 0; k < NV; ++k) { sm.xc[side][k][r] = h.c[k]; sm.xf[side][k][r] = h.f[0][k]; }
        sm.xlam[side][r] = h.lam[0];
    }
}

// This row's y side, and the x side of columns 0 and 31, of record r.
template <int NV>
__device__ __forceinline__ void tile_publish(SmemTile<NV> &sm, const CellRecV<3, NV> &r, int w, int l)
{
#pragma unroll
    for (int k = 0; k < NV; ++k) { sm.yc[w][k][l] = r.c[k]; sm.yf[w][k][l] = r.f[1][k]; }
    sm.ylam[w][l] = r.lam[1];
    if (l == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) { sm.c0[k][w] = r.c[k]; sm.f0[k][w] = r.f[0][k]; }
        sm.lam0[w] = r.lam[0];
    } else if (l == 31) {
#pragma unroll
        for (int k = 0; k < NV; ++k) { sm.c31[k][w] = r.c[k]; sm.f31[k][w] = r.f[0][k]; }
        sm.lam31[w] = r.lam[0];
    }
}

template <class A, int STAGE>
__global__ void __launch_bounds__(TILE_X * TILE_Y, TILE_MIN_BLOCKS) stage3d_tile_kernel(GridParams gp, StageArgs sa)
{
    constexpr int NV = A::NVAR;
    __shared__ SmemTile<NV> sm;
    const int l = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const StepScalars sc = step_scalars<A, STAGE>(gp, sa.ctrl);
    if (gp.bookkeep && blockIdx.x == 0 && threadIdx.x == 0) step_bookkeeping<STAGE>(sa.ctrl, sc);
    if (!sc.active) return;

    const int nx = gp.n[0], ny = gp.n[1], nz = gp.n[2];
    const int ntx = (nx + TILE_X - 1) / TILE_X, nty = (ny + TILE_Y - 1) / TILE_Y;
    const bool perx = gp.bc_lo[0] == BC_PERIODIC, pery = gp.bc_lo[1] == BC_PERIODIC,
               perz = gp.bc_lo[2] == BC_PERIODIC;
    // The launch covers planes [zlo, zlo + nzr) of every tile column, as
    // units of one column and L planes, columns fastest.  With G blocks, the
    // whole rounds of G units go one unit per block (block b: units b, b + G,
    // ...), so the blocks running together march neighbouring columns over
    // the same planes and their halo rows and columns are read from L2; the
    // units of the last, partial round are split evenly over all G blocks as
    // (column, plane) pairs, unit after unit.  One block per chunk-long unit
    // (G = units) is the plain one-chunk-per-block decomposition.
    const int ntiles = ntx * nty, G = gridDim.x;
    const int zlo = gp.chunk0 * gp.chunk;
    const int nzr = min(nz, zlo + gp.nchunk * gp.chunk) - zlo;
    const int L = (gp.tile3d == 2 && gp.unit > 0) ? gp.unit : gp.chunk;
    const int nunit = (nzr + L - 1) / L;                     // units per column
    const int units = ntiles * nunit;
    const int full = units / G * G;
    const int last_len = nzr - (nunit - 1) * L;              // planes of a column's last unit
    const int ub = (nunit - 1) * ntiles;                     // first unit of the columns' last units
    const int na = max(0, ub - full);                        // tail units of L planes
    const int nb = units - max(full, ub);                    // tail units of last_len planes
    const long long npair = (long long)na * L + (long long)nb * last_len;
    int q = (int)(npair * blockIdx.x / G);
    const int q1 = (int)(npair * (blockIdx.x + 1) / G);
    int u = blockIdx.x;
    unsigned status = 0;
    double lmax = 0.0;
    for (;;) {
        int col, z0, z1;
        if (u < full) {
            col = u % ntiles;
            z0 = zlo + (u / ntiles) * L;
            z1 = min(z0 + L, zlo + nzr);
            u += G;
        } else if (q < q1) {
            const bool a = q < na * L;
            const int len = a ? L : last_len;
            const int qq = a ? q : q - na * L;
            const int uu = (a ? full : max(full, ub)) + qq / len;
            const int off = qq - (qq / len) * len;
            col = uu % ntiles;
            z0 = zlo + (uu / ntiles) * L + off;
            z1 = z0 + min(len - off, q1 - q);
            q += z1 - z0;
        } else {
            break;
        }
        const int x0 = (col % ntx) * TILE_X, y0 = (col / ntx) * TILE_Y;
        const int x = x0 + l, y = y0 + w;
        const bool out = (x < nx) && (y < ny);
        unsigned *st = (STAGE == STAGE_1 && out) ? &status : nullptr;

        RecOf<A, 3> cur, nxt;
        double Fzlo[NV], Fzhi[NV], Fxl[NV], Fxr[NV], Fyb[NV], Fyt[NV], acc[NV];
        load_record<A, STAGE, 3>(sa, gp, sc, x, y, z0 - 1, nxt, nullptr);
        load_record<A, STAGE, 3>(sa, gp, sc, x, y, z0, cur, st);
        {
            const double lz = face_dir<A, 3>(nxt, cur, 2, Fzlo);
            if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, lz);
        }
        tile_halo_records<A, STAGE>(sa, gp, sc, sm, w, l, x0, y0, z0);
        tile_publish<NV>(sm, cur, w, l);
        for (int z = z0; z < z1; ++z) {
            __syncthreads();   // (A) records of plane z
            // x face on the right: the next lane (lane 31's, on the tile's right
            // edge, comes from the edge pass; its value here is replaced)
            {
                double cR[NV], fR[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) { cR[k] = shfl_down(cur.c[k], 1); fR[k] = shfl_down(cur.f[0][k], 1); }
                const double lamR = shfl_down(cur.lam[0], 1);
                const double lx = A::face(cur.c, cur.f[0], cur.lam[0], cR, fR, lamR, Fxr);
                if (STAGE <= STAGE_1 && out && l < 31) lmax = max_nonneg(lmax, lx);
            }
            // y face above: the next row, or the top halo row
            {
                double cU[NV], fU[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) { cU[k] = sm.yc[w + 1][k][l]; fU[k] = sm.yf[w + 1][k][l]; }
                const double ly = A::face(cur.c, cur.f[1], cur.lam[1], cU, fU, sm.ylam[w + 1][l], Fyt);
                if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, ly);
#pragma unroll
                for (int k = 0; k < NV; ++k) sm.Fy[w][k][l] = Fyt[k];
            }
            // faces on the tile's left edge (lanes 0..TILE_Y-1: rows), right
            // edge (the next TILE_Y lanes: rows) and bottom edge (lanes: columns)
            if (w == TW_LEFTF && l < 2 * TILE_Y) {
                const int r = l % TILE_Y;
                const bool right = l >= TILE_Y;
                double cL[NV], fL[NV], cR[NV], fR[NV], F[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    cL[k] = right ? sm.c31[k][r] : sm.xc[0][k][r];
                    fL[k] = right ? sm.f31[k][r] : sm.xf[0][k][r];
                    cR[k] = right ? sm.xc[1][k][r] : sm.c0[k][r];
                    fR[k] = right ? sm.xf[1][k][r] : sm.f0[k][r];
                }
                const double le = A::face(cL, fL, right ? sm.lam31[r] : sm.xlam[0][r], cR, fR,
                                          right ? sm.xlam[1][r] : sm.lam0[r], F);
                if (right) {
#pragma unroll
                    for (int k = 0; k < NV; ++k) sm.Fr[k][r] = F[k];
                    if (STAGE <= STAGE_1 && x0 + TILE_X - 1 < nx && y0 + r < ny) lmax = max_nonneg(lmax, le);
                } else {
#pragma unroll
                    for (int k = 0; k < NV; ++k) sm.Fl[k][r] = F[k];
                    if (STAGE <= STAGE_1 && x0 < nx && y0 + r < ny) lmax = max_nonneg(lmax, le);
                }
            } else if (w == TW_BOTF) {
                double cL[NV], fL[NV], cR[NV], fR[NV], F[NV];
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    cL[k] = sm.bc[k][l]; fL[k] = sm.bf[k][l]; cR[k] = sm.yc[0][k][l]; fR[k] = sm.yf[0][k][l];
                }
                const double le = A::face(cL, fL, sm.blam[l], cR, fR, sm.ylam[0][l], F);
#pragma unroll
                for (int k = 0; k < NV; ++k) sm.Fb[k][l] = F[k];
                if (STAGE <= STAGE_1 && x < nx && y0 < ny) lmax = max_nonneg(lmax, le);
            }
            __syncthreads();   // (B) faces of plane z
            // the faces below and on the left: the previous lane / row, or the tile edge
            const int wb = (w > 0) ? w - 1 : 0;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const double fl = shfl_up(Fxr[k], 1);
                Fxl[k] = (l == 0) ? sm.Fl[k][w] : fl;
                Fxr[k] = (l == 31) ? sm.Fr[k][w] : Fxr[k];
                Fyb[k] = (w == 0) ? sm.Fb[k][l] : sm.Fy[wb][k][l];
            }
            accumulate_pair<A, true>(acc, Fxl, Fxr, gp.area, perx && x == nx - 1);
            accumulate_pair<A, false>(acc, Fyb, Fyt, gp.area, pery && y == ny - 1);
            // plane z+1 and the z face
            load_record<A, STAGE, 3>(sa, gp, sc, x, y, z + 1, nxt, (z + 1 < z1) ? st : nullptr);
            const double lz = face_dir<A, 3>(cur, nxt, 2, Fzhi);
            if (STAGE <= STAGE_1 && out) lmax = max_nonneg(lmax, lz);
            if (out) {
                accumulate_pair<A, false>(acc, Fzlo, Fzhi, gp.area, perz && z == nz - 1);
                store_output<A, STAGE>(sa, gp, sc, (long long)x + (long long)nx * ((long long)y + (long long)ny * z),
                                       acc, cur.c);
            }
            // records of plane z+1 for the next (A)
            if (z + 1 < z1) {
                tile_halo_records<A, STAGE>(sa, gp, sc, sm, w, l, x0, y0, z + 1);
                tile_publish<NV>(sm, nxt, w, l);
            }
            cur = nxt;
#pragma unroll
            for (int k = 0; k < NV; ++k) Fzlo[k] = Fzhi[k];
        }
    }
    publish_reductions<STAGE>(lmax, status, sa.ctrl, sa.rhs_maxeig);
}

} // namespace mmf
