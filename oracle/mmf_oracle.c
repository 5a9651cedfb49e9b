/*
 * mmf_oracle.c -- CPU oracle (test infrastructure; see mmf_oracle.h).
 *
 * Each function restates the reference function cited beside it with the
 * same floating-point operation order, so that a build with
 * -ffp-contract=off reproduces the reference's arithmetic bit for bit.
 */
#include "mmf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define NF ORC_N_FIELDS
static const double GAMMA = 1.4;   /* constants.hpp:55 */

/* FID_* (constants.hpp:37-53) */
enum { FID_P = 0, FID_U = 1, FID_V = 2, FID_W = 3, FID_T = 4 };
enum { FID_RHO = 0, FID_RHO_U = 1, FID_RHO_V = 2, FID_RHO_W = 3, FID_RHO_E = 4 };

static double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max(a, b) */

void orc_params_default(orc_params *p)
{
    p->vortex_beta = 5.0;
    p->sod_radius = 1.0;
    p->sod_rho_in = 1.0;  p->sod_p_in = 1.0;
    p->sod_rho_out = 0.125; p->sod_p_out = 0.1;
    p->periodic_exact = 0;
    p->domain_origin[0] = p->domain_origin[1] = p->domain_origin[2] = 0.0;
    p->domain_length = 0.0;
}

double orc_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* utils.cpp:37-40 */
double orc_normal_velocity(const double *f, const double *n)
{
    return (f[FID_U] * n[0] + f[FID_V] * n[1] + f[FID_W] * n[2]);
}

/* utils.cpp:48-63 */
void orc_cons2prim(const double *c, double *p)
{
    double K = (c[FID_RHO_U] * c[FID_RHO_U] + c[FID_RHO_V] * c[FID_RHO_V] + c[FID_RHO_W] * c[FID_RHO_W])
               / (c[FID_RHO] * c[FID_RHO]);
    p[FID_T] = (2.0 * c[FID_RHO_E] / c[FID_RHO] - K) / (2.0 / (GAMMA - 1.0));
    p[FID_U] = c[FID_RHO_U] / c[FID_RHO];
    p[FID_V] = c[FID_RHO_V] / c[FID_RHO];
    p[FID_W] = c[FID_RHO_W] / c[FID_RHO];
    p[FID_P] = c[FID_RHO] * p[FID_T];
}

/* utils.cpp:71-83 */
void orc_prim2cons(const double *p, double *c)
{
    c[FID_RHO] = p[FID_P] / p[FID_T];
    c[FID_RHO_U] = c[FID_RHO] * p[FID_U];
    c[FID_RHO_V] = c[FID_RHO] * p[FID_V];
    c[FID_RHO_W] = c[FID_RHO] * p[FID_W];
    c[FID_RHO_E] = c[FID_RHO] * p[FID_T] / (GAMMA - 1.0)
                   + 0.5 * c[FID_RHO] * (p[FID_U] * p[FID_U] + p[FID_V] * p[FID_V] + p[FID_W] * p[FID_W]);
}

/* euler.cpp:83-113 (the negative p / rho log lines are not restated) */
void orc_eval_fluxes(const double *c, const double *p, const double *n, double *f)
{
    double u = p[FID_U], v = p[FID_V], w = p[FID_W];
    double vel2 = u * u + v * v + w * w;
    double un = orc_normal_velocity(p, n);
    double pr = p[FID_P];
    double rho = c[FID_RHO];
    double eto = pr / (GAMMA - 1.) + 0.5 * rho * vel2;
    double massFlux = rho * un;
    f[0] = massFlux;
    f[1] = massFlux * u + pr * n[0];
    f[2] = massFlux * v + pr * n[1];
    f[3] = massFlux * w + pr * n[2];
    f[4] = un * (eto + pr);
}

/* euler.cpp:42-73 */
void orc_eval_splitting(const double *cl, const double *cr, const double *n, double *f, double *lambda)
{
    double pl[NF], pr[NF], fl[NF], fr[NF];
    orc_cons2prim(cl, pl);
    orc_cons2prim(cr, pr);
    orc_eval_fluxes(cl, pl, n, fl);
    orc_eval_fluxes(cr, pr, n, fr);
    double unL = orc_normal_velocity(pl, n);
    double aL = sqrt(GAMMA * pl[FID_T]);
    double lambdaL = fabs(unL) + aL;
    double unR = orc_normal_velocity(pr, n);
    double aR = sqrt(GAMMA * pr[FID_T]);
    double lambdaR = fabs(unR) + aR;
    *lambda = dmax(lambdaR, lambdaL);
    for (int k = 0; k < NF; ++k)
        f[k] = 0.5 * ((fr[k] + fl[k]) - (*lambda) * (cr[k] - cl[k]));
}

/* problem.cpp:450-477 */
static void border_bc_info(int problem, int bc, double *info)
{
    if (problem == ORC_FFSTEP && bc == ORC_BC_DIRICHLET) {
        info[FID_U] = 3.0; info[FID_V] = 0.; info[FID_W] = 0.;
        info[FID_P] = 1.;  info[FID_T] = 1. / 1.4;
    }
}

/* euler.cpp:318-337 */
static void reflecting_bc(const double *n, const double *c, double *c_bc)
{
    double prim[NF];
    orc_cons2prim(c, prim);
    double u[3] = {prim[FID_U], prim[FID_V], prim[FID_W]};
    double un = orc_normal_velocity(prim, n);
    double u_n[3] = {un * n[0], un * n[1], un * n[2]};
    prim[FID_U] = u[0] - 2 * u_n[0];
    prim[FID_V] = u[1] - 2 * u_n[1];
    prim[FID_W] = u[2] - 2 * u_n[2];
    orc_prim2cons(prim, c_bc);
}

/* euler.cpp:261-288, 298-308, 347-376 */
void orc_eval_bc(int problem, int bc, const double *point, const double *n, const double *c, double *c_bc)
{
    (void)point;
    double info[NF] = {0, 0, 0, 0, 0};
    border_bc_info(problem, bc, info);
    switch (bc) {
    case ORC_BC_FREE_FLOW: memcpy(c_bc, c, NF * sizeof(double)); break;
    case ORC_BC_REFLECTING:
    case ORC_BC_WALL: reflecting_bc(n, c, c_bc); break;
    case ORC_BC_DIRICHLET: orc_prim2cons(info, c_bc); break;
    default: break;
    }
}

/* problem.cpp:247-392 */
void orc_exact_conservatives(int problem, int dim, const orc_params *prm, const double *point_in,
                             double t, double *c)
{
    double prim[NF] = {0, 0, 0, 0, 0};
    double point[3] = {point_in[0], point_in[1], point_in[2]};
    switch (problem) {
    case ORC_VORTEX_XY:
    case ORC_VORTEX_ZX:
    case ORC_VORTEX_YZ: {
        const double VORTEX_BETA = prm->vortex_beta;
        const double VORTEX_P_INF = 1.0;
        const double VORTEX_T_INF = 1.0;
        double VORTEX_U_INF = 1.0, VORTEX_V_INF = 1.0, VORTEX_W_INF = 1.0;
        if (problem == ORC_VORTEX_XY) VORTEX_W_INF = 0.;
        else if (problem == ORC_VORTEX_ZX) VORTEX_V_INF = 0.;
        else VORTEX_U_INF = 0.;
        point[0] -= t * VORTEX_U_INF;
        point[1] -= t * VORTEX_V_INF;
        point[2] -= t * VORTEX_W_INF;
        if (prm->periodic_exact) {
            /* EXTENSION: nearest periodic image, only for points that left the box */
            for (int d = 0; d < dim; ++d) {
                const double o = prm->domain_origin[d], L = prm->domain_length;
                while (point[d] < o) point[d] += L;
                while (point[d] >= o + L) point[d] -= L;
            }
        }
        double csi = 0., eta = 0.;
        if (problem == ORC_VORTEX_XY) { csi = point[0]; eta = point[1]; }
        else if (problem == ORC_VORTEX_ZX) { csi = point[2]; eta = point[0]; }
        else { csi = point[1]; eta = point[2]; }
        double r = sqrt(csi * csi + eta * eta);
        double shape = VORTEX_BETA / (2 * M_PI) * exp(0.5 * (1 - r * r));
        double du = 0., dv = 0., dw = 0.;
        if (problem == ORC_VORTEX_XY) { du = -eta * shape; dv = csi * shape; dw = 0.; }
        else if (problem == ORC_VORTEX_ZX) { dw = -eta * shape; du = csi * shape; dv = 0.; }
        else { dv = -eta * shape; dw = csi * shape; du = 0.; }
        const double dT = -(GAMMA - 1.0) / (2 * GAMMA) * shape * shape;
        const double dp = pow(VORTEX_T_INF + dT, GAMMA / (GAMMA - 1.0)) - 1.0;
        prim[FID_P] = VORTEX_P_INF + dp;
        prim[FID_U] = VORTEX_U_INF + du;
        prim[FID_V] = VORTEX_V_INF + dv;
        prim[FID_W] = (dim == 3) ? VORTEX_W_INF + dw : 0;
        prim[FID_T] = VORTEX_T_INF + dT;
        break;
    }
    case ORC_RADSOD: {
        double r = sqrt(point[0] * point[0] + point[1] * point[1] + point[2] * point[2]);
        prim[FID_U] = 0.0; prim[FID_V] = 0.0; prim[FID_W] = 0.0;
        if (r < prm->sod_radius) {
            prim[FID_P] = prm->sod_p_in;
            prim[FID_T] = prm->sod_p_in / prm->sod_rho_in;
        } else {
            prim[FID_P] = prm->sod_p_out;
            prim[FID_T] = prm->sod_p_out / prm->sod_rho_out;
        }
        break;
    }
    case ORC_SOD_X:
    case ORC_SOD_Y:
    case ORC_SOD_Z: {
        prim[FID_U] = 0.0; prim[FID_V] = 0.0; prim[FID_W] = 0.0;
        double r = (problem == ORC_SOD_X) ? point[0] : (problem == ORC_SOD_Y) ? point[1] : point[2];
        if (r < 0.) { prim[FID_P] = 1.0; prim[FID_T] = 1.0 / 1.0; }
        else { prim[FID_P] = 0.1; prim[FID_T] = 0.1 / 0.125; }
        break;
    }
    case ORC_FFSTEP:
        prim[FID_U] = 3.0; prim[FID_V] = 0.0; prim[FID_W] = 0.0;
        prim[FID_P] = 1.0; prim[FID_T] = 1.0 / 1.4;
        break;
    default: break;
    }
    orc_prim2cons(prim, c);
}

/* problem.cpp:404-438 */
int orc_border_bc_type(int problem, const double *fc)
{
    switch (problem) {
    case ORC_VORTEX_XY: case ORC_VORTEX_ZX: case ORC_VORTEX_YZ:
    case ORC_SOD_X: case ORC_SOD_Y: case ORC_SOD_Z:
        return ORC_BC_FREE_FLOW;
    case ORC_RADSOD:
        return ORC_BC_REFLECTING;
    case ORC_FFSTEP:
        if (fc[0] < 1e-10) return ORC_BC_DIRICHLET;
        else if (fc[0] > 3.2 - 1e-10) return ORC_BC_FREE_FLOW;
        return ORC_BC_REFLECTING;
    default: return ORC_BC_FREE_FLOW;
    }
}

/* ------------------------------------------------------------------ mesh */

static uint64_t spread_bits(uint64_t x, int dim)
{
    uint64_t r = 0;
    for (int b = 0; b < 21; ++b)
        if (x & (1ull << b)) r |= 1ull << (b * dim);
    return r;
}

static int64_t *g_sort_keys;
static int cmp_by_key(const void *a, const void *b)
{
    int64_t ka = g_sort_keys[*(const int64_t *)a], kb = g_sort_keys[*(const int64_t *)b];
    return (ka > kb) - (ka < kb);
}

int orc_mesh_build(orc_mesh *m, int problem, int dim, const int64_t *n, const double *origin,
                   double length, const int *bc_lo, const int *bc_hi, int cell_order)
{
    memset(m, 0, sizeof(*m));
    m->dim = dim;
    m->n[0] = n[0]; m->n[1] = n[1]; m->n[2] = (dim == 3) ? n[2] : 1;
    for (int d = 0; d < 3; ++d) m->origin[d] = origin[d];
    m->h = length / (double)n[0];
    m->cell_order = cell_order;
    const double h = m->h;
    const int64_t nx = m->n[0], ny = m->n[1], nz = m->n[2];
    const int64_t nc = nx * ny * nz;
    m->ncells = nc;
    m->raw_of_grid = malloc(nc * sizeof(int64_t));
    m->grid_of_raw = malloc(nc * sizeof(int64_t));
    if (cell_order == 1) {
        int64_t *keys = malloc(nc * sizeof(int64_t));
        for (int64_t g = 0; g < nc; ++g) {
            int64_t i = g % nx, j = (g / nx) % ny, k = g / (nx * ny);
            keys[g] = (int64_t)(spread_bits(i, dim) | (spread_bits(j, dim) << 1) |
                                (dim == 3 ? spread_bits(k, dim) << 2 : 0));
            m->grid_of_raw[g] = g;
        }
        g_sort_keys = keys;
        qsort(m->grid_of_raw, nc, sizeof(int64_t), cmp_by_key);
        free(keys);
        for (int64_t r = 0; r < nc; ++r) m->raw_of_grid[m->grid_of_raw[r]] = r;
    } else {
        for (int64_t g = 0; g < nc; ++g) m->raw_of_grid[g] = m->grid_of_raw[g] = g;
    }
    m->cell_volume = malloc(nc * sizeof(double));
    m->cell_size = malloc(nc * sizeof(double));
    m->cell_centroid = malloc(3 * nc * sizeof(double));
    m->solved = malloc(nc);
    const double vol = (dim == 3) ? h * h * h : h * h;
    for (int64_t g = 0; g < nc; ++g) {
        int64_t i = g % nx, j = (g / nx) % ny, k = g / (nx * ny);
        int64_t r = m->raw_of_grid[g];
        m->cell_volume[r] = vol;
        m->cell_size[r] = h;
        m->cell_centroid[3 * r + 0] = origin[0] + ((double)i + 0.5) * h;
        m->cell_centroid[3 * r + 1] = origin[1] + ((double)j + 0.5) * h;
        m->cell_centroid[3 * r + 2] = (dim == 3) ? origin[2] + ((double)k + 0.5) * h : origin[2];
        m->solved[r] = 1;
    }
    for (int d = 0; d < 3; ++d) {
        m->bc_lo[d] = bc_lo ? bc_lo[d] : -100;
        m->bc_hi[d] = bc_hi ? bc_hi[d] : -100;
    }
    /* count faces */
    int64_t nf = 0;
    for (int d = 0; d < dim; ++d) {
        int per = (m->bc_lo[d] == ORC_BC_PERIODIC);
        int64_t cnt[3] = {nx, ny, nz};
        cnt[d] += per ? 0 : 1;
        nf += cnt[0] * cnt[1] * cnt[2];
    }
    m->nfaces = nf;
    m->owner = malloc(nf * sizeof(int64_t));
    m->neigh = malloc(nf * sizeof(int64_t));
    m->area = malloc(nf * sizeof(double));
    m->normal = malloc(3 * nf * sizeof(double));
    m->fcentroid = malloc(3 * nf * sizeof(double));
    m->bc = malloc(nf * sizeof(int));
    m->fdir = malloc(nf * sizeof(int));
    const double area = (dim == 3) ? h * h : h;
    /* border condition of each side as the faces resolve it (the ghost cells of
     * the order-2 slopes use it) */
    int side_bc_lo[3] = {-100, -100, -100}, side_bc_hi[3] = {-100, -100, -100};
    int64_t f = 0;
    for (int d = 0; d < dim; ++d) {
        int per = (m->bc_lo[d] == ORC_BC_PERIODIC);
        int64_t cnt[3] = {nx, ny, nz};
        cnt[d] += per ? 0 : 1;
        for (int64_t k = 0; k < cnt[2]; ++k)
            for (int64_t j = 0; j < cnt[1]; ++j)
                for (int64_t i = 0; i < cnt[0]; ++i, ++f) {
                    int64_t idx[3] = {i, j, k};
                    int64_t lo[3] = {i, j, k}, hi[3] = {i, j, k};
                    const int64_t nd = m->n[d];
                    double nrm[3] = {0.0, 0.0, 0.0};
                    double fc[3];
                    fc[0] = origin[0] + ((double)i + 0.5) * h;
                    fc[1] = origin[1] + ((double)j + 0.5) * h;
                    fc[2] = (dim == 3) ? origin[2] + ((double)k + 0.5) * h : origin[2];
                    fc[d] = origin[d] + (double)idx[d] * h;
                    m->area[f] = area;
                    m->fdir[f] = d;
                    lo[d] = idx[d] - 1;
                    hi[d] = idx[d];
                    if (per && idx[d] == 0) lo[d] = nd - 1;
                    int64_t glo = lo[0] + nx * (lo[1] + ny * lo[2]);
                    int64_t ghi = hi[0] + nx * (hi[1] + ny * hi[2]);
                    if (!per && idx[d] == 0) {
                        nrm[d] = -1.0;
                        m->owner[f] = m->raw_of_grid[ghi];
                        m->neigh[f] = -1;
                        m->bc[f] = (m->bc_lo[d] >= 0) ? m->bc_lo[d] : orc_border_bc_type(problem, fc);
                        if (side_bc_lo[d] == -100) side_bc_lo[d] = m->bc[f];
                    } else if (!per && idx[d] == nd) {
                        nrm[d] = 1.0;
                        m->owner[f] = m->raw_of_grid[glo];
                        m->neigh[f] = -1;
                        m->bc[f] = (m->bc_hi[d] >= 0) ? m->bc_hi[d] : orc_border_bc_type(problem, fc);
                        if (side_bc_hi[d] == -100) side_bc_hi[d] = m->bc[f];
                    } else {
                        nrm[d] = 1.0;
                        m->owner[f] = m->raw_of_grid[glo];
                        m->neigh[f] = m->raw_of_grid[ghi];
                        m->bc[f] = ORC_BC_NONE;
                    }
                    for (int q = 0; q < 3; ++q) {
                        m->normal[3 * f + q] = nrm[q];
                        m->fcentroid[3 * f + q] = fc[q];
                    }
                }
    }
    /* record the resolved border BCs */
    for (int d = 0; d < 3; ++d) {
        if (m->bc_lo[d] < 0) m->bc_lo[d] = (d < dim && side_bc_lo[d] != -100) ? side_bc_lo[d] : -1;
        if (m->bc_hi[d] < 0) m->bc_hi[d] = (d < dim && side_bc_hi[d] != -100) ? side_bc_hi[d] : -1;
    }
    return 0;
}

void orc_mesh_free(orc_mesh *m)
{
    free(m->raw_of_grid); free(m->grid_of_raw);
    free(m->cell_volume); free(m->cell_size); free(m->cell_centroid); free(m->solved);
    free(m->owner); free(m->neigh); free(m->area); free(m->normal); free(m->fcentroid);
    free(m->bc); free(m->fdir);
    memset(m, 0, sizeof(*m));
}

/* -------------------------------------------------------- reconstruction */

/* raw id of the neighbour of cell 'raw' across its side (d, s), s = -1 / +1;
 * -1 on a non-periodic border. */
static int64_t cell_neighbour(const orc_mesh *m, int64_t raw, int d, int s)
{
    int64_t g = m->grid_of_raw[raw];
    int64_t idx[3] = {g % m->n[0], (g / m->n[0]) % m->n[1], g / (m->n[0] * m->n[1])};
    int64_t q = idx[d] + s;
    if (q < 0 || q >= m->n[d]) {
        int bc = (s < 0) ? m->bc_lo[d] : m->bc_hi[d];
        if (bc != ORC_BC_PERIODIC) return -1;
        q = (q < 0) ? m->n[d] - 1 : 0;
    }
    idx[d] = q;
    return m->raw_of_grid[idx[0] + m->n[0] * (idx[1] + m->n[1] * idx[2])];
}

/* EXTENSION: division-free positivity test of a conservative state:
 * rho > 0 and 2 rho E > |m|^2 (i.e. p > 0). */
static int state_admissible(const double *c)
{
    if (!(c[0] > 0.0)) return 0;
    double m2 = c[1] * c[1] + c[2] * c[2] + c[3] * c[3];
    return (2.0 * c[0] * c[4] - m2) > 0.0;
}

/* reconstruction.cpp:47-55 is an empty hook for order 1; EXTENSION for
 * order 2: MC-limited MUSCL slopes (per direction, per conservative field),
 * stored as slopes[(raw * 3 + d) * 5 + k]. */
void orc_compute_polynomials(const orc_mesh *m, int problem, int order, const double *U,
                             double *slopes, int limiter_mode, const unsigned char *flag,
                             unsigned char *active)
{
    if (order != 2) return;
    for (int64_t c = 0; c < m->ncells; ++c) {
        const double *uc = U + NF * c;
        int limit = (limiter_mode == 0) || (limiter_mode == 2 && flag && flag[c]);
        int act = 0;
        for (int d = 0; d < 3; ++d) {
            double *sd = slopes + (c * 3 + d) * NF;
            if (d >= m->dim) { for (int k = 0; k < NF; ++k) sd[k] = 0.0; continue; }
            double gl[NF], gr[NF];
            const double *ul, *ur;
            int64_t nl = cell_neighbour(m, c, d, -1), nr = cell_neighbour(m, c, d, +1);
            double nrm[3] = {0.0, 0.0, 0.0};
            if (nl >= 0) ul = U + NF * nl;
            else {
                nrm[d] = -1.0;
                orc_eval_bc(problem, m->bc_lo[d], m->cell_centroid + 3 * c, nrm, uc, gl);
                ul = gl;
            }
            if (nr >= 0) ur = U + NF * nr;
            else {
                nrm[d] = 1.0;
                orc_eval_bc(problem, m->bc_hi[d], m->cell_centroid + 3 * c, nrm, uc, gr);
                ur = gr;
            }
            for (int k = 0; k < NF; ++k) {
                double a = uc[k] - ul[k];
                double b = ur[k] - uc[k];
                double central = 0.5 * (ur[k] - ul[k]);   /* one difference: (U+ - U-) / 2 */
                double s = central;
                if (limit) {
                    if (a * b <= 0.0) s = 0.0;
                    else {
                        double lim = fmin(2.0 * fabs(a), 2.0 * fabs(b));
                        double mag = fmin(lim, fabs(central));
                        s = (a > 0.0) ? mag : -mag;
                    }
                    /* activation counts where the slope change is significant
                     * (round-off level sign flips in flat regions do not) */
                    if (fabs(s - central) > 1e-6 * (fabs(uc[0]) + fabs(uc[4]))) act = 1;
                }
                sd[k] = s;
            }
        }
        if (limit || limiter_mode == 2) {
            /* positivity fallback: every face state must stay admissible (also
             * for the cells a flag leaves on central slopes) */
            int ok = 1;
            for (int d = 0; d < m->dim && ok; ++d) {
                const double *sd = slopes + (c * 3 + d) * NF;
                double fm[NF], fp[NF];
                for (int k = 0; k < NF; ++k) { fm[k] = uc[k] - 0.5 * sd[k]; fp[k] = uc[k] + 0.5 * sd[k]; }
                ok = state_admissible(fm) && state_admissible(fp);
            }
            if (!ok) {
                memset(slopes + c * 3 * NF, 0, 3 * NF * sizeof(double));
                act = 1;
            }
        }
        if (active) active[c] = (unsigned char)act;
    }
}

/* face value of cell 'raw' on its side s (-1/+1) of direction d */
static void eval_side(int order, int64_t raw, int d, int s, const double *means, const double *slopes,
                      double *values)
{
    if (order == 1) { memcpy(values, means, NF * sizeof(double)); return; } /* reconstruction.cpp:90-97 */
    const double *sd = slopes + (raw * 3 + d) * NF;
    const double off = (s > 0) ? 0.5 : -0.5;
    for (int k = 0; k < NF; ++k) values[k] = means[k] + off * sd[k];
}

/* reconstruction.cpp:67-79: point-based evaluation (the face is the nearest
 * axis side of the cell; periodic wrap is resolved by distance) */
void orc_reconstruction_eval(const orc_mesh *m, int order, int64_t raw, const double *point,
                             const double *means, const double *slopes, double *values)
{
    if (order == 1) { memcpy(values, means, NF * sizeof(double)); return; }
    const double *xc = m->cell_centroid + 3 * raw;
    int best = 0; double bestv = 0.0;
    for (int d = 0; d < m->dim; ++d) {
        double o = point[d] - xc[d];
        if (fabs(o) > fabs(bestv)) { bestv = o; best = d; }
    }
    int s = (bestv > 0.0) ? 1 : -1;
    if (fabs(bestv) > m->h) s = -s; /* periodic wrap face */
    eval_side(order, raw, best, s, means, slopes, values);
}

/* euler.cpp:127-249 */
void orc_compute_rhs(const orc_mesh *m, int problem, int order, const double *U, const double *slopes,
                     double *rhs, double *max_eig)
{
    for (int64_t c = 0; c < m->ncells; ++c)
        for (int k = 0; k < NF; ++k) rhs[NF * c + k] = 0.;
    *max_eig = 0.0;
    for (int64_t f = 0; f < m->nfaces; ++f) {
        const int64_t o = m->owner[f], nb = m->neigh[f];
        const double *ownerMean = U + NF * o;
        double *ownerRHS = rhs + NF * o;
        int ownerSolved = m->solved[o];
        const double *neighMean = NULL;
        double *neighRHS = NULL;
        int neighSolved = 0;
        if (nb >= 0) {
            neighMean = U + NF * nb;
            neighRHS = rhs + NF * nb;
            neighSolved = m->solved[nb];
        }
        if (!ownerSolved && !neighSolved) continue;
        const int bc = m->bc[f];
        const double A = m->area[f];
        const double *nrm = m->normal + 3 * f;
        const double *fc = m->fcentroid + 3 * f;
        const int d = m->fdir[f];
        /* side of the face seen from the owner: -1 only for a low border face */
        const int ownerSide = (nrm[d] < 0.0) ? -1 : 1;
        double ownerRec[NF], neighRec[NF];
        if (bc == ORC_BC_NONE) {
            eval_side(order, o, d, ownerSide, ownerMean, slopes, ownerRec);
            eval_side(order, nb, d, -1, neighMean, slopes, neighRec);
        } else {
            double n2[3] = {nrm[0], nrm[1], nrm[2]};
            double *fluidRec, *virtualRec;
            if (ownerSolved) {
                fluidRec = ownerRec; virtualRec = neighRec;
                eval_side(order, o, d, ownerSide, ownerMean, slopes, fluidRec);
            } else {
                for (int q = 0; q < 3; ++q) n2[q] = -1. * n2[q];
                fluidRec = neighRec; virtualRec = ownerRec;
                eval_side(order, nb, d, -1, neighMean, slopes, fluidRec);
            }
            orc_eval_bc(problem, bc, fc, n2, fluidRec, virtualRec);
        }
        double F[NF], faceMaxEig;
        orc_eval_splitting(ownerRec, neighRec, nrm, F, &faceMaxEig);
        *max_eig = dmax(faceMaxEig, *max_eig);
        if (ownerSolved)
            for (int k = 0; k < NF; ++k) ownerRHS[k] -= A * F[k];
        if (neighSolved)
            for (int k = 0; k < NF; ++k) neighRHS[k] += A * F[k];
    }
}

/* ------------------------------------------------------------- time loop */

/* main.cpp:335-344 */
void orc_initial_state(const orc_mesh *m, int problem, const orc_params *prm, double *U)
{
    for (int64_t c = 0; c < m->ncells; ++c)
        orc_exact_conservatives(problem, m->dim, prm, m->cell_centroid + 3 * c, 0.0, U + NF * c);
}

/* main.cpp:550-561 */
double orc_l1_density_error(const orc_mesh *m, int problem, const orc_params *prm, const double *U, double t)
{
    double error = 0.;
    double ex[NF];
    for (int64_t c = 0; c < m->ncells; ++c) {
        orc_exact_conservatives(problem, m->dim, prm, m->cell_centroid + 3 * c, t, ex);
        error += fabs(U[NF * c + 0] - ex[0]) * m->cell_volume[c];
    }
    return error;
}

/* main.cpp:351-356, 377-506 */
int64_t orc_run(const orc_mesh *m, const orc_run_cfg *cfg, double *U, double *t_out)
{
    const int64_t nc = m->ncells;
    double *W = malloc(NF * nc * sizeof(double));
    double *R = malloc(NF * nc * sizeof(double));
    double *S = (cfg->order == 2) ? malloc(3 * NF * nc * sizeof(double)) : NULL;
    memset(W, 0, NF * nc * sizeof(double));
    double minCellSize = 1.79769313486231570815e+308;
    for (int64_t c = 0; c < nc; ++c) minCellSize = fmin(m->cell_size[c], minCellSize);
    const double cfl = cfg->cfl, tMax = cfg->t_end;
    int64_t step = 0;
    double t = cfg->t_start;
    while (t < tMax && (cfg->max_steps < 0 || step < cfg->max_steps)) {
        double maxEig;
        orc_compute_polynomials(m, cfg->problem, cfg->order, U, S, cfg->limiter_mode, cfg->limiter_flag, NULL);
        orc_compute_rhs(m, cfg->problem, cfg->order, U, S, R, &maxEig);
        double dt = 0.9 * cfl * minCellSize / maxEig;
        if (t + dt > tMax) dt = tMax - t;
        if (cfg->dt_log) cfg->dt_log[step] = dt;
        if (cfg->maxeig_log) cfg->maxeig_log[step] = maxEig;
        for (int64_t c = 0; c < nc; ++c) {
            if (!m->solved[c]) continue;
            const double V = m->cell_volume[c];
            for (int k = 0; k < NF; ++k) W[NF * c + k] = U[NF * c + k] + dt * R[NF * c + k] / V;
        }
        orc_compute_polynomials(m, cfg->problem, cfg->order, W, S, cfg->limiter_mode, cfg->limiter_flag, NULL);
        orc_compute_rhs(m, cfg->problem, cfg->order, W, S, R, &maxEig);
        for (int64_t c = 0; c < nc; ++c) {
            if (!m->solved[c]) continue;
            const double V = m->cell_volume[c];
            for (int k = 0; k < NF; ++k)
                W[NF * c + k] = 0.75 * U[NF * c + k] + 0.25 * (W[NF * c + k] + dt * R[NF * c + k] / V);
        }
        orc_compute_polynomials(m, cfg->problem, cfg->order, W, S, cfg->limiter_mode, cfg->limiter_flag, NULL);
        orc_compute_rhs(m, cfg->problem, cfg->order, W, S, R, &maxEig);
        for (int64_t c = 0; c < nc; ++c) {
            if (!m->solved[c]) continue;
            const double V = m->cell_volume[c];
            for (int k = 0; k < NF; ++k)
                U[NF * c + k] = (1. / 3) * U[NF * c + k] + (2. / 3) * (W[NF * c + k] + dt * R[NF * c + k] / V);
        }
        t += dt;
        step++;
    }
    free(W); free(R); free(S);
    if (t_out) *t_out = t;
    return step;
}
