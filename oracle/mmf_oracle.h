/*
 * mmf_oracle.h -- CPU oracle for the minimmerflow finite-volume Euler step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (optimad/minimmerflow src/utils.cpp, src/euler.cpp,
 * src/reconstruction.cpp, src/problem.cpp and the time loop of src/main.cpp).
 * Only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark may load it, and only as the reference results the GPU path is
 * compared with, or as the timed CPU baseline.
 * The product path (minimmerflow_gb300) never calls into it.
 *
 * Parity is pinned: the five reference regression goldens
 * (test/<case>/CMakeLists.txt:33) are reproduced by this code, and the
 * reference sources themselves, compiled against a minimal bitpit shim
 * (oracle/ref_shim, built into oracle/_ref), agree with it bit for bit.
 *
 * Project extensions that have no reference counterpart (periodic borders,
 * step-count termination, the parametrised radial Sod / vortex of the
 * benchmark configurations, order-2 limited reconstruction) are marked
 * "EXTENSION" and are pinned only by this restatement.
 *
 * Build: gcc -O2 -ffp-contract=off (no FMA contraction: the reference is
 * compiled with plain -O2 on x86-64, which emits no FMA).
 */
#ifndef MMF_ORACLE_H
#define MMF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* constants.hpp:35-62 */
#define ORC_N_FIELDS 5
#define ORC_BC_NONE (-1)
#define ORC_BC_FREE_FLOW 0
#define ORC_BC_REFLECTING 1
#define ORC_BC_WALL 2
#define ORC_BC_DIRICHLET 3
/* EXTENSION: periodic border (no reference counterpart) */
#define ORC_BC_PERIODIC 16

/* problem.hpp:33-42 */
enum {
    ORC_VORTEX_XY = 0, ORC_VORTEX_ZX = 1, ORC_VORTEX_YZ = 2, ORC_RADSOD = 3,
    ORC_SOD_X = 4, ORC_SOD_Y = 5, ORC_SOD_Z = 6, ORC_FFSTEP = 7
};

/* Problem parameters.  Defaults (orc_params_default) are the constants the
 * reference hard-codes (problem.cpp:257-262, 336-342). EXTENSION: other
 * values drive the parametrised benchmark configurations. */
typedef struct {
    double vortex_beta;                 /* 5.0 */
    double sod_radius;                  /* 1.0 */
    double sod_rho_in, sod_p_in;        /* 1.0, 1.0 */
    double sod_rho_out, sod_p_out;      /* 0.125, 0.1 */
    int    periodic_exact;              /* wrap the translated vortex (EXTENSION) */
    double domain_origin[3];            /* used by periodic_exact */
    double domain_length;
} orc_params;

void orc_params_default(orc_params *p);

/* utils.cpp:37-83 */
double orc_normal_velocity(const double *prim, const double *n);
void orc_cons2prim(const double *c, double *p);
void orc_prim2cons(const double *p, double *c);

/* euler.cpp:42-113 */
void orc_eval_fluxes(const double *c, const double *p, const double *n, double *f);
void orc_eval_splitting(const double *cl, const double *cr, const double *n, double *f, double *lambda);

/* euler.cpp:261-376 with problem.cpp:450-477 (border info) */
void orc_eval_bc(int problem, int bc, const double *point, const double *n,
                 const double *c, double *c_bc);

/* problem.cpp:247-392 */
void orc_exact_conservatives(int problem, int dim, const orc_params *prm,
                             const double *point, double t, double *c);
/* problem.cpp:404-438 */
int orc_border_bc_type(int problem, const double *face_centroid);

/* ---- mesh: the subset of MeshGeometricalInfo (mesh_info.hpp:31-105) the path
 * reads, for a uniform Cartesian grid as VolOctree builds it with uniform
 * refinement.  Interfaces are listed x-faces first, then y-faces, then
 * z-faces, each block in (k, j, i) order of the face index; owner is the
 * lower cell, border faces are owned by the interior cell with the outward
 * normal.  Cell raw order is row-major (x fastest) or Morton. */
typedef struct {
    int dim;
    int64_t n[3];
    double origin[3];
    double h;
    int bc_lo[3], bc_hi[3];     /* border BC code per side (ORC_BC_PERIODIC wraps) */
    int cell_order;             /* 0 row-major, 1 Morton */

    int64_t ncells;
    int64_t *raw_of_grid;       /* grid linear index (x fastest) -> raw id */
    int64_t *grid_of_raw;
    double *cell_volume, *cell_size, *cell_centroid; /* per raw id; centroid [3] */
    unsigned char *solved;      /* cellSolvedFlag per raw id */

    int64_t nfaces;
    int64_t *owner, *neigh;     /* raw ids; neigh < 0 on a border */
    double *area, *normal, *fcentroid; /* normal/centroid [3] per face */
    int *bc;                    /* ORC_BC_NONE for interior faces */
    int *fdir;                  /* face direction 0..2 */
} orc_mesh;

/* Builds the mesh.  'length' is the domain edge (VolOctree ctor, main.cpp:149),
 * h = length / n[0] for every direction of the cube.  bc_lo/bc_hi may be NULL:
 * then orc_border_bc_type(problem, ...) decides (main.cpp:251-277). */
int orc_mesh_build(orc_mesh *m, int problem, int dim, const int64_t *n, const double *origin,
                   double length, const int *bc_lo, const int *bc_hi, int cell_order);
void orc_mesh_free(orc_mesh *m);

/* ---- reconstruction (reconstruction.cpp:47-97).  Order 1 is the reference
 * (copy of the mean).  EXTENSION: order 2 = MUSCL slopes per direction with
 * the monotonised-central (MC) limiter; 'limiter_mode' 0 = limit every cell,
 * 1 = never limit (central slopes), 2 = limit only cells with flag[c] != 0
 * (the others take central slopes but keep the positivity fallback).
 * 'active' (nullable) receives 1 where the limiter changed a slope by more
 * than 1e-6 (|rho| + |rho E|) of the cell, or fell back to order 1. */
void orc_compute_polynomials(const orc_mesh *m, int problem, int order, const double *U,
                             double *slopes, int limiter_mode, const unsigned char *flag,
                             unsigned char *active);
void orc_reconstruction_eval(const orc_mesh *m, int order, int64_t raw, const double *point,
                             const double *means, const double *slopes, double *values);

/* euler.cpp:127-249 */
void orc_compute_rhs(const orc_mesh *m, int problem, int order, const double *U,
                     const double *slopes, double *rhs, double *max_eig);

/* ---- time loop: main.cpp:335-506 (SSP-RK3 + CFL dt), minus VTK and MPI.
 * Runs while t < t_end; EXTENSION: also stops after max_steps (<0 = no
 * limit).  U (raw order, AoS [ncells][5]) is the initial state on entry and
 * the final state on exit.  Returns the number of steps; *t_out = final t. */
typedef struct {
    int problem;
    int order;
    double cfl;
    double t_start, t_end;
    int64_t max_steps;
    int limiter_mode;
    const unsigned char *limiter_flag;
    double *dt_log;        /* nullable: dt per step */
    double *maxeig_log;    /* nullable: stage-1 maxEig per step */
} orc_run_cfg;

int64_t orc_run(const orc_mesh *m, const orc_run_cfg *cfg, double *U, double *t_out);

/* main.cpp:335-344: IC at every cell centroid. */
void orc_initial_state(const orc_mesh *m, int problem, const orc_params *prm, double *U);
/* main.cpp:550-561: sum over internal cells of |rho - rho_exact(t)| * V. */
double orc_l1_density_error(const orc_mesh *m, int problem, const orc_params *prm,
                            const double *U, double t);

/* Wall-clock helper for the CPU baseline (steady clock, seconds). */
double orc_now(void);

#ifdef __cplusplus
}
#endif
#endif
