/*
 * mmf_gb300.h -- C ABI of the GB300 (sm_103a) finite-volume Euler step that
 * replaces the hot path of optimad/minimmerflow: face reconstruction
 * (src/reconstruction.cpp), interface fluxes and residual accumulation
 * (src/euler.cpp), the SSP-RK3 stage update and the CFL time step (inline in
 * src/main.cpp:377-506).
 *
 * Conventions (mirroring the reference boundary, src/euler.hpp:37-48):
 *  - The caller owns every host buffer; the library writes results into
 *    caller storage and never calls exit().
 *  - Cell state crosses the ABI as the reference's PiercedStorage raw layout:
 *    AoS double[n_raw][5] in raw-id order, fields (rho, rho u, rho v, rho w,
 *    rho E) = FID_RHO..FID_RHO_E (src/constants.hpp:43-47).  A raw-id -> grid
 *    cell map (mmf_set_cell_map) lets it follow bitpit's octree (Morton) order.
 *  - Every function returns an int status: MMF_OK (0) or a negative code;
 *    mmf_last_error() describes the last failure of the calling thread.
 *  - One context = one GPU, one CUDA stream; calls on a context are ordered
 *    and not thread-safe (the reference is single-threaded per rank).
 *  - No CPU fallback: without a usable CUDA device mmf_create fails.
 */
#ifndef MMF_GB300_H
#define MMF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MMF_ABI_VERSION 1

/* status codes */
#define MMF_OK 0
#define MMF_ERR_ARG (-1)          /* invalid argument */
#define MMF_ERR_CUDA (-2)         /* CUDA runtime error (no device, launch failure, ...) */
#define MMF_ERR_STATE (-3)        /* non-physical state seen (rho < 0, p < 0, NaN) */
#define MMF_ERR_UNSUPPORTED (-4)  /* unsupported order / configuration */
#define MMF_ERR_NOMEM (-5)        /* device allocation failed */

/* border conditions: src/constants.hpp:58-62; MMF_BC_PERIODIC has no
 * reference counterpart (periodic wrap of the two opposite borders). */
#define MMF_BC_NONE (-1)
#define MMF_BC_FREE_FLOW 0
#define MMF_BC_REFLECTING 1
#define MMF_BC_WALL 2
#define MMF_BC_DIRICHLET 3
#define MMF_BC_PERIODIC 16

/* arithmetic of the fused step */
#define MMF_ARITH_REFERENCE 0   /* reference operation order, bit-identical results */
#define MMF_ARITH_FAST 1        /* one division + one sqrt per cell, FMA; round-off level agreement */

/* status bits reported by mmf_get_status (src/euler.cpp:93-101 logs the first two) */
#define MMF_STATUS_NEG_DENSITY 1u
#define MMF_STATUS_NEG_PRESSURE 2u
#define MMF_STATUS_NAN 4u

typedef struct mmf_ctx mmf_ctx;

/* Uniform Cartesian mesh, the mesh VolOctree builds with uniform refinement
 * (src/main.cpp:146-155).  Cell (i,j,k) has centroid origin + (i+1/2, j+1/2,
 * k+1/2) h, volume h^dim, faces of area h^(dim-1). */
typedef struct {
    int dim;                   /* 2 or 3 */
    int n[3];                  /* cells per direction (n[2] = 1 in 2D) */
    double origin[3];
    double h;                  /* cell edge = minCellSize (src/main.cpp:351-356) */
    int bc_lo[3], bc_hi[3];    /* border condition per side (MMF_BC_*) */
    double dirichlet_prim[5];  /* (p,u,v,w,T) behind MMF_BC_DIRICHLET borders (src/problem.cpp:458-468) */
    int order;                 /* reconstruction order: 1 (src/reconstruction.cpp:67-79), or 2 (MC-limited
                                  MUSCL on the computePolynomials hook; no reference implementation) */
    int arith;                 /* MMF_ARITH_* */
    int chunk;                 /* marching chunk (rows 2D / planes 3D); 0 = default */
} mmf_grid;

/* ---- context --------------------------------------------------------- */
int mmf_create(const mmf_grid *grid, int device, mmf_ctx **out);
int mmf_destroy(mmf_ctx *ctx);
const char *mmf_last_error(void);
int mmf_abi_version(void);
/* Number of kernel launches issued by this context since creation. */
int64_t mmf_launch_count(const mmf_ctx *ctx);

/* Raw-id -> grid-cell map (grid index = i + n0 (j + n1 k)); n_raw must equal
 * the cell count.  Default: identity (row-major raw order).  Replaces the
 * id -> raw-position lookups of src/euler.cpp:158-178. */
int mmf_set_cell_map(mmf_ctx *ctx, int64_t n_raw, const int64_t *raw_to_cell);

/* ---- state transfer (PiercedStorage AoS raw layout <-> device SoA) --- */
int mmf_upload_state(mmf_ctx *ctx, const double *aos, int64_t n_raw);
int mmf_download_state(mmf_ctx *ctx, double *aos, int64_t n_raw);
/* Same with device pointers (AoS [n_raw][5] already in device memory). */
int mmf_upload_state_device(mmf_ctx *ctx, const double *d_aos, int64_t n_raw);
int mmf_download_state_device(mmf_ctx *ctx, double *d_aos, int64_t n_raw);

/* ---- reference entry points ------------------------------------------ */
/* euler::computeRHS (src/euler.hpp:41-43): residual of every cell (not
 * divided by the volume) and the maximum face eigenvalue, for the state
 * 'cons' (host AoS raw layout).  Always uses the reference arithmetic. */
int mmf_compute_rhs(mmf_ctx *ctx, const double *cons, double *rhs, double *max_eig, int64_t n_raw);
/* reconstruction::computePolynomials (src/reconstruction.hpp:41-42) of the
 * state 'cons' (host AoS raw layout): a no-op at order 1.  At order 2 it
 * computes the limited slopes (returned as AoS [n_raw][3][5] when 'slopes' is
 * not NULL, direction-major) and the cells where the limiter changed a slope
 * ('limiter_active', one byte per raw id, when not NULL). */
int mmf_compute_polynomials(mmf_ctx *ctx, const double *cons, double *slopes, unsigned char *limiter_active,
                            int64_t n_raw);
/* Order-2 limiter selection: MMF_LIMIT_ALL (every cell), MMF_LIMIT_NONE
 * (central slopes), MMF_LIMIT_FLAGGED (cells whose byte in 'flags', raw order,
 * is non-zero; flags may be NULL to keep the uploaded ones). */
#define MMF_LIMIT_ALL 0
#define MMF_LIMIT_NONE 1
#define MMF_LIMIT_FLAGGED 2
int mmf_set_limiter(mmf_ctx *ctx, int mode, const unsigned char *flags, int64_t n_raw);
/* Flags already on the device, one byte per grid cell (grid order); selects MMF_LIMIT_FLAGGED. */
int mmf_set_limiter_flags_device(mmf_ctx *ctx, const unsigned char *d_flags_grid);
/* Where the limiter changed a slope at stage 1 of the last step (or the last
 * mmf_compute_polynomials call): one byte per raw id. */
int mmf_get_limiter_activity(mmf_ctx *ctx, unsigned char *active, int64_t n_raw);

/* ---- time loop (src/main.cpp:377-506) on the uploaded state ----------- */
/* Sets t, t_end (INFINITY allowed with max_steps >= 0), CFL; minCellSize = h. */
int mmf_time_setup(mmf_ctx *ctx, double cfl, double t, double t_end, int64_t max_steps);
/* Runs up to n_steps SSP-RK3 steps (stopping at t_end / max_steps), device
 * resident, replayed from a CUDA graph; returns the time and steps done. */
int mmf_advance(mmf_ctx *ctx, int64_t n_steps, double *t_out, int64_t *steps_done);
/* Enqueues n_steps graph-replayed steps without waiting (no host sync); the
 * time and step count are read later with mmf_time_info. */
int mmf_advance_async(mmf_ctx *ctx, int64_t n_steps);
/* Current time and steps done since mmf_time_setup (synchronises). */
int mmf_time_info(mmf_ctx *ctx, double *t, int64_t *step);
/* The CUDA stream (cudaStream_t) all work of this context is ordered on. */
void *mmf_get_stream(mmf_ctx *ctx);
/* Host-buffer form: uploads 'aos', advances n_steps, downloads into 'aos'. */
/* Chooses the work decomposition of the stage kernels by timing a few steps
 * of each candidate from the current state (2D: rows per marching chunk x
 * warps per block; 3D: planes per chunk x, at order 1, the 3D kernel: row
 * blocks or 32 x 8 tiles, the tiles with one block per tile and chunk or
 * one block per resident slot); restores the state and the time control
 * afterwards.  Results are bitwise independent of the choice.  Needs
 * mmf_time_setup.  warps_per_block receives the warps per block in 2D, and
 * in 3D minus the variant of mmf_set_shape (0 row blocks, -1 tiles with one
 * block per tile and chunk, -2 tiles with one block per resident slot).  No
 * reference counterpart. */
int mmf_autotune(mmf_ctx *ctx, int trial_steps, int *chunk, int *warps_per_block);
/* Sets the work decomposition directly: rows (2D) or planes (3D) per
 * marching chunk, and 'variant' = warps per block in 2D (1..4), the 3D
 * kernel in 3D (0 = row blocks; 1 = 32 x 8 tiles, one block per tile and
 * chunk; 2 = 32 x 8 tiles on at most one block per resident slot (two per
 * SM): whole rounds of (tile column, 'chunk'-plane) units, the last round
 * split evenly by planes; the default; 1 and 2 are order 1 only).  Results
 * are bitwise independent of the choice.  No reference counterpart. */
int mmf_set_shape(mmf_ctx *ctx, int chunk, int variant);
/* Per-step log, the values the reference prints each step (src/main.cpp:
 * 399-404): maxEig, the dt used and the time after the step.  The device
 * keeps the last 'capacity' steps in a ring (0 switches the log off).
 * mmf_get_step_log copies up to max_entries of the most recent steps, oldest
 * first, as out[3 * i + {0, 1, 2}] = {maxEig, dt, t}, with the index of the
 * first one.  No reference counterpart (the reference writes a text log). */
int mmf_set_step_log(mmf_ctx *ctx, int64_t capacity);
int mmf_get_step_log(mmf_ctx *ctx, double *out, int64_t max_entries, int64_t *first_step, int64_t *n_entries);
/* Upload the AoS state, advance up to n_steps steps, download into the same
 * buffer.  With a page-locked buffer (and no raw-id map or learned indicator)
 * the copies run in bands overlapped with the stages; the bits are those of
 * the sequential round trip. */
int mmf_advance_host(mmf_ctx *ctx, double *aos, int64_t n_raw, int64_t n_steps, double *t_out);
/* Last step's dt and stage-1 maxEig (the reference logs both, main.cpp:399). */
int mmf_last_step_info(mmf_ctx *ctx, double *dt, double *max_eig);
/* Status bits accumulated since the last call (cleared on read). */
int mmf_get_status(mmf_ctx *ctx, unsigned *status);
/* Blocks until queued work is done. */
int mmf_synchronize(mmf_ctx *ctx);

/* Single stages, for drivers that keep the reference loop structure:
 * stage 1 = computeRHS(U) + maxEig; 2 = W update (needs dt); 3 = close. */
int mmf_rk_stage(mmf_ctx *ctx, int stage);

/* ---- unit-level functions, batched over n items (host AoS buffers) ---- */
/* utils::conservative2primitive / primitive2conservative (src/utils.hpp:34-35) */
int mmf_cons2prim(int64_t n, const double *cons, double *prim);
int mmf_prim2cons(int64_t n, const double *prim, double *cons);
/* euler::evalFluxes (src/euler.hpp:39): cons[n][5], prim[n][5], normal[n][3] */
int mmf_eval_fluxes(int64_t n, const double *cons, const double *prim, const double *normal, double *flux);
/* euler::evalSplitting (src/euler.hpp:37) */
int mmf_eval_splitting(int64_t n, const double *cons_l, const double *cons_r, const double *normal,
                       double *flux, double *lambda);
/* euler::evalInterfaceBCValues (src/euler.hpp:45-48); dirichlet_prim may be NULL */
int mmf_eval_bc_values(int64_t n, int bc_type, const double *normal, const double *cons,
                       const double *dirichlet_prim, double *cons_bc);

/* ---- initial states, errors, output, checkpoints ------------------------ */
/* Problem types (src/problem.hpp:33-42) and the parameters the reference
 * hard-codes (vortex strength 5, Sod radius 1 and states 1/1 inside,
 * 0.125/0.1 outside; src/problem.cpp:257-262, 336-342). */
#define MMF_VORTEX_XY 0
#define MMF_VORTEX_ZX 1
#define MMF_VORTEX_YZ 2
#define MMF_RADSOD 3
#define MMF_SOD_X 4
#define MMF_SOD_Y 5
#define MMF_SOD_Z 6
#define MMF_FFSTEP 7
typedef struct {
    int problem;
    double vortex_beta;
    double sod_radius, sod_rho_in, sod_p_in, sod_rho_out, sod_p_out;
    int periodic_exact;   /* translated vortex wrapped into the domain (periodic borders) */
} mmf_problem;
/* Initial conservative state at every cell centroid, on the device
 * (src/main.cpp:335-344 with src/problem.cpp:247-392). */
int mmf_init_state(mmf_ctx *ctx, const mmf_problem *problem);
/* sum over cells of |rho - rho_exact(t)| V on the device (src/main.cpp:550-567). */
int mmf_l1_density_error(mmf_ctx *ctx, const mmf_problem *problem, double t, double *error);
/* VTK XML ImageData file (raw appended data, grid order) with the cell
 * fields of the reference's writer (src/main.cpp:289-298,
 * src/solver_writer.cpp:56-119): solved, velocity, pressure, temperature,
 * density and residualC/MX/MY/MZ/E.  The residuals are computeRHS of the
 * written state with the reference arithmetic (the reference writes the
 * residual of its last stage's input, which the fused step does not keep). */
int mmf_write_vtk(mmf_ctx *ctx, const char *path);
/* Raw checkpoint of the state and the time control (t, step, dt, ...) and
 * its restore; mmf_advance continues the run where it stopped. */
int mmf_save_checkpoint(mmf_ctx *ctx, const char *path);
int mmf_load_checkpoint(mmf_ctx *ctx, const char *path);

/* ---- general face lists ------------------------------------------------ */
/* The Euler step on any mesh given as MeshGeometricalInfo-like arrays
 * (src/mesh_info.hpp:31-105): per raw cell volume, size and solved flag
 * (cellSolvedFlag), per interface owner / neighbour raw ids (neighbour -1 on a
 * border), area, normal [n_faces][3] (owner -> neighbour) and border
 * condition (interfaceBCs; MMF_BC_NONE inside, MMF_BC_WALL between fluid and
 * solid cells, src/main.cpp:251-277).  The residual keeps the reference's face
 * order (src/euler.cpp:153-248) through an atomic-free per-cell gather, so the
 * reference arithmetic is bit-identical on any mesh: refined octrees,
 * immersed bodies, the forward-facing step.  Order 1. */
typedef struct {
    int dim;
    int64_t n_cells, n_faces;
    const double *cell_volume, *cell_size;
    const unsigned char *solved;    /* NULL = every cell solved */
    const int64_t *owner, *neigh;
    const double *area, *normal;
    const int *bc;
    double dirichlet_prim[5];       /* (p,u,v,w,T) behind MMF_BC_DIRICHLET faces */
    int arith;
} mmf_umesh_desc;
typedef struct mmf_umesh mmf_umesh;
int mmf_umesh_create(const mmf_umesh_desc *desc, int device, mmf_umesh **out);
int mmf_umesh_destroy(mmf_umesh *u);
int64_t mmf_umesh_launch_count(const mmf_umesh *u);
int mmf_umesh_upload(mmf_umesh *u, const double *aos, int64_t n_cells);
int mmf_umesh_download(mmf_umesh *u, double *aos, int64_t n_cells);
/* euler::computeRHS on the face list (residual not divided by the volume). */
int mmf_umesh_compute_rhs(mmf_umesh *u, const double *cons, double *rhs, double *max_eig, int64_t n_cells);
int mmf_umesh_time_setup(mmf_umesh *u, double cfl, double t, double t_end, int64_t max_steps);
int mmf_umesh_advance(mmf_umesh *u, int64_t n_steps, double *t_out, int64_t *steps_done);

/* ---- batched cases ------------------------------------------------------ */
/* Many independent 2D cases of uneven size advanced together: one
 * persistent launch per RK stage walks a list of (case, segment, row chunk)
 * work items, each case keeps its own t, CFL dt (per-case maxEig reduction),
 * step count and status, and the step sequence replays from a CUDA graph.
 * Each case gets exactly the result of its own single-case context.  No
 * reference counterpart (the reference runs one case per process).  Order 1
 * or order 2 (all cases alike). */
typedef struct mmf_batch mmf_batch;
int mmf_batch_create(int ncases, const mmf_grid *grids, int device, mmf_batch **out);
int mmf_batch_destroy(mmf_batch *batch);
int64_t mmf_batch_cell_count(const mmf_batch *batch);
int64_t mmf_batch_launch_count(const mmf_batch *batch);
void *mmf_batch_get_stream(mmf_batch *batch);
/* all cases' states, AoS [total][5], case after case, each row-major */
int mmf_batch_upload(mmf_batch *batch, const double *aos, int64_t total);
int mmf_batch_download(mmf_batch *batch, double *aos, int64_t total);
/* per-case CFL and end time (t_end NULL = no end time, then max_steps >= 0) */
int mmf_batch_time_setup(mmf_batch *batch, const double *cfl, const double *t_end, int64_t max_steps);
int mmf_batch_advance_async(mmf_batch *batch, int64_t n_steps);
int mmf_batch_synchronize(mmf_batch *batch);
int mmf_batch_case_info(mmf_batch *batch, int c, double *t, int64_t *steps, unsigned *status);
/* Order-2 batches: limiter mode for every case (MMF_LIMIT_*), and the learned
 * indicator (a 2D mmf_mlp) run at the start of every step over all cases. */
typedef struct mmf_mlp mmf_mlp;
int mmf_batch_set_limiter(mmf_batch *batch, int mode);
int mmf_batch_set_indicator(mmf_batch *batch, mmf_mlp *mlp, float threshold);
/* mmf_set_indicator_period for a batch (one counter for all its cases). */
int mmf_batch_set_indicator_period(mmf_batch *batch, int period);
/* Decomposition: rows per work item and resident blocks per SM (0 = occupancy maximum). */
int mmf_batch_set_shape(mmf_batch *batch, int chunk, int blocks_per_sm);
int mmf_batch_get_shape(mmf_batch *batch, int *chunk, int *blocks_per_sm);
/* Times trial_steps steps per candidate shape (chunk in {8,16,32,64} x up to
 * three block counts), keeps the fastest, restores the state; results are
 * cached per workload signature for the process. */
int mmf_batch_autotune(mmf_batch *batch, int trial_steps, int *chunk, int *blocks_per_sm);

/* ---- learned troubled-cell indicator (order 2) --------------------------- */
/* A small MLP predicts, from the normalised primitive variables of a cell's
 * 3^dim stencil (dim 2: 45 inputs padded to 48; dim 3: 135 padded to 144),
 * whether the order-2 limiter would change one of the cell's slopes; cells
 * predicted smooth take central slopes and skip the limiter.  135 -> 64 ->
 * 64 -> 1, GELU, sigmoid; BF16 operands, FP32 accumulation.  Training and
 * inference run on the GPU (mma.sync BF16 training kernels, a fused tcgen05
 * inference kernel).  No reference counterpart (the reference has no limiter). */
typedef struct mmf_mlp mmf_mlp;
int mmf_mlp_create(int dim, uint64_t seed, int device, mmf_mlp **out);
int mmf_mlp_destroy(mmf_mlp *mlp);
int64_t mmf_mlp_num_params(const mmf_mlp *mlp);
/* Feature width KPAD of one sample (48 in 2D, 144 in 3D). */
int mmf_mlp_input_width(const mmf_mlp *mlp);
/* FP32 parameters W1 [64][KPAD], b1 [64], W2 [64][64], b2 [64], w3 [64], b3 */
int mmf_mlp_get_params(mmf_mlp *mlp, float *params, int64_t n);
int mmf_mlp_set_params(mmf_mlp *mlp, const float *params, int64_t n);
/* Gradients of the mean binary cross-entropy over a batch (device features
 * d_X: BF16 [B][KPAD]; d_y: labels 0/1; B a multiple of 16), to host memory. */
int mmf_mlp_gradients(mmf_mlp *mlp, const void *d_X, const unsigned char *d_y, int64_t B, float *grad, float *loss);
/* One Adam step on a batch. */
int mmf_mlp_train_batch(mmf_mlp *mlp, const void *d_X, const unsigned char *d_y, int64_t B, float lr, float *loss);
/* Iteration limits of the tcgen05 kernels' mbarrier waits (default 2^22
 * and 0).  Every wait of the inference and training kernels on the weights'
 * bulk copies and on the MMA completions gives up after wait_limit polls: the
 * kernel then sets its error flag, frees its tensor memory and returns, and
 * the entry point that launched it returns MMF_ERR_CUDA.  probe_limit > 0
 * makes every CTA of the inference kernel first wait on a barrier that
 * nothing completes, before any copy or MMA is issued: a test of that path
 * with nothing in flight.  No reference counterpart (the reference only logs
 * bad states, src/euler.cpp:94-101). */
int mmf_mlp_set_wait_limits(mmf_mlp *mlp, int64_t wait_limit, int64_t probe_limit);
/* Probabilities of n stored samples (device in, device out). */
int mmf_mlp_predict(mmf_mlp *mlp, const void *d_X, int64_t n, float *d_prob);
/* Features of every cell of the uploaded state, grid order, into device
 * memory d_X (BF16 [n][KPAD]). */
int mmf_features(mmf_ctx *ctx, void *d_X);
/* Training labels of the uploaded state: 1 where the order-2 limiter (every
 * cell limited, reference arithmetic) changes a slope, grid order, device memory. */
int mmf_limiter_labels(mmf_ctx *ctx, unsigned char *d_labels);
/* Runs the indicator on the uploaded state: the limiter becomes
 * MMF_LIMIT_FLAGGED with flag = (probability > threshold).  prob / flags
 * (host, raw order, nullable) receive the probabilities and flags. */
int mmf_indicator(mmf_ctx *ctx, mmf_mlp *mlp, float threshold, float *prob, unsigned char *flags);
/* From the next step on, every step starts with the indicator on U (inside
 * the step's CUDA graph); mlp = NULL switches it off (limiter back to ALL). */
int mmf_set_indicator(mmf_ctx *ctx, mmf_mlp *mlp, float threshold);
/* The indicator runs every 'period' steps (1, the default, or 2).  With 2,
 * its flags are dilated by one cell (a cell is limited where any cell of its
 * 3^dim neighbourhood is flagged) and serve the step after as well: at
 * CFL <= 0.5 a wave moves at most one cell in two steps.  The counter starts
 * again, so that the next step runs the indicator, whenever the state or the
 * time control is set (upload, checkpoint, mmf_time_setup, mmf_autotune).
 * mmf_indicator returns the dilated flags when the period is 2.  No reference
 * counterpart. */
int mmf_set_indicator_period(mmf_ctx *ctx, int period);

/* ---- residual without device allocation ------------------------------- */
/* Largest mesh accepted by mmf_compute_rhs_noalloc. */
#define MMF_NOALLOC_MAX_CELLS 65536
/* euler::computeRHS for callers that cannot call cudaMalloc (for example code
 * running while another library captures a CUDA graph, real-time loops that
 * cannot take the synchronisation an allocation implies, or processes whose
 * device memory is held by a pool allocator).  No counterpart in the
 * reference.  Inputs and outputs are device pointers: d_cons and d_rhs are
 * AoS double[n][5] in raw order, d_max_eig one double, d_raw_to_cell an
 * optional raw -> grid-cell map (NULL = row-major).  The grid is checked as
 * mmf_create checks it; order 1 and MMF_ARITH_REFERENCE only (anything else is
 * MMF_ERR_UNSUPPORTED).  Work is queued on 'stream' (a cudaStream_t, NULL =
 * the default stream) on the current device and the call returns without
 * waiting.  The working set lives in a static device array of
 * 2*5*MMF_NOALLOC_MAX_CELLS + 32 + MMF_NOALLOC_MAX_CELLS/2 doubles (about
 * 5.5 MB) that every GPU which loads the library holds until exit; meshes with
 * more cells are rejected with MMF_ERR_ARG.  The map must be a permutation of
 * 0..n-1: the GPU checks it, and when it is not, every row of d_rhs and
 * *d_max_eig are set to NaN (the call has returned by then, so no error code
 * can report it).  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress), so make it before any stream capture.  All
 * calls share the array: calls that overlap on the GPU race.  Reference
 * arithmetic: the result equals mmf_compute_rhs bit for bit. */
int mmf_compute_rhs_noalloc(const mmf_grid *grid, const double *d_cons, double *d_rhs, double *d_max_eig,
                            const int64_t *d_raw_to_cell, void *stream);

/* Measured FP64 instruction rate of a GPU, in thread-level instructions per
 * second: out[0] for DFMA whose multiplier and addend stay in the same
 * registers (the pipe's best case), out[1] for DADD, DMUL and DFMA whose
 * operands change from one instruction to the next (the stage kernels' mix).
 * The roofline denominator of the FP64-bound stage kernels; no reference
 * counterpart.  Takes about 0.2 s. */
int mmf_fp64_rate(int device, double out[2]);

/* Self-test of the reciprocal and square root of MMF_ARITH_FAST (Newton
 * iterations on the hardware approximations): rcp[i] ~ 1/x[i], sqrt[i] ~ sqrt(x[i])
 * for positive x.  No reference counterpart; used to check the error bound. */
int mmf_newton_selftest(int64_t n, const double *x, double *rcp, double *sqrt_out);

/* Self-test of the FP32 screen of the order-2 positivity fallback: for each of
 * n cells (uc [n][nv] stored fields, sig [n][dim][nv] slopes), dec[i] = 1 (every
 * face state U -+ sigma/2 has rho > 0 and p > 0), 0 (some has not) or -1
 * (undecided in FP32), and ref[i] = the FP64 test of the same arithmetic.
 * nv = 4 is the 2D four-field layout (rho, rho u, rho v, rho E) of
 * MMF_ARITH_FAST.  No reference counterpart; a decided dec must equal ref. */
int mmf_o2_screen_selftest(int arith, int nv, int dim, int64_t n, const double *uc, const double *sig, int *dec,
                           unsigned char *ref);

#ifdef __cplusplus
}
#endif
#endif
