/*
 * Oracle (TEST INFRASTRUCTURE ONLY) -- CPU FP64 restatement of the reference
 * pressure-Poisson multigrid path.  See mg_oracle.h for the scope, the array
 * conventions and the parity pin.  Every routine cites the reference routine
 * (file:line) whose steps it restates; loop orders and floating-point
 * evaluation orders follow the reference so that a sweep here and a sweep
 * there produce the same bits.  Compile with -ffp-contract=off so that the
 * results are the same on x86-64 and aarch64 hosts.
 *
 * Documented choices where the reference is undefined or out of scope:
 *  - Periodic velocity BCs are rejected: the reference's MG reads
 *    var(nxc,...) on coarse arrays (IBM/CORE_MG.F90:1958-1961), out of bounds.
 *  - Coarse z-level ghost metrics (zc_MG(0,n), zc_MG(m+1,n), dz_MG(0,n),
 *    dz_MG(m+1,n)) are left uninitialised by the reference
 *    (IBM/CORE_MG.F90:254-266); they are computed here the same way as the
 *    x and y levels (:186-205).  They only enter through a Dirichlet
 *    pressure BC on a z face.
 *  - fresh_cell is 0 (stationary bodies); pot_flag is 0 (viscous flow).
 *  - nlw (the MG extra term, IBM/CORE_MG.F90:1968) is 0, as in a standalone
 *    solve (IBM/MAIN.F90:2266).
 */
#include "mg_oracle.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum { BC_DIRICHLET = 1, BC_ZERO_GRADIENT = 2, BC_PERIODIC = 5 };
enum { PBC_DIRICHLET = 1, PBC_NEUMANN = 2 };
enum { GCM_METHOD = 2, DIM_2D = 2, DIM_3D = 3 };

typedef struct { int8_t *a; int sx, sy; } i8v;

struct or_ctx {
    fsi_mg_params p;
    int nx, ny, nz, nxc, nyc, nzc;
    int n[3], nc[3];
    /* fine grid, (0:n+1) */
    double *x[3], *xc[3], *dx[3], *dxinv[3], *dxc[3], *dxcinv[3];
    /* MG grid per level: a[i + (n+2)*(lev-1)] */
    int nlev[3];
    int *mgrid[3];
    double *x_MG[3], *xc_MG[3], *dx_MG[3], *dxinv_MG[3], *dxc_MG[3], *dxcinv_MG[3];
    /* fine flags (0:nx+1)^3 */
    int8_t *iblank, *ghost, *fl[6];
    int8_t *fresh;   /* fresh_cell (0:nx+1)^3 or NULL (no fresh cells) */
    int8_t *flMG[6];
    int *ghostMG;
    int8_t **cib[3];    /* coarse iblank per direction, index n-1 (n>=2) */
    double *nlw, *nlw0;
    double *pgrad[6];
    int pg_sx[6];
    int nGhost;
    int32_t *gi[6];
    double *coeff, *probe;
    double *pPrime_mod;
    i8v ibMG;
    int gs_last_iters;
    int ghost_nonconv;
    int geometry_set;
    /* ghost-cell velocities (GCM_vel_set_bc_internal) */
    double *vg_coeff, *vg_bi;   /* coeffGCMD (8,nGhost); uBI, vBI, wBI (3 x nGhost) or NULL */
    double vg_bw, vg_iw;
    int vg_on, vg_last_iters;
    /* implicit momentum coefficients amx_ad, apx_ad, amy_ad, apy_ad, amz_ad, apz_ad (or_set_solve_ad) */
    double *ad[6];
};

static const int incI[8] = {0, 0, 1, 1, 0, 0, 1, 1};   /* IBM/GCM_MEMORY_ALLOCATE.F90:494-518 */
static const int incJ[8] = {0, 1, 1, 0, 0, 1, 1, 0};
static const int incK[8] = {0, 0, 0, 0, 1, 1, 1, 1};

#define FI(c, i, j, k) ((size_t)(i) + (size_t)((c)->nx + 2) * ((size_t)(j) + (size_t)((c)->ny + 2) * (size_t)(k)))
#define VI(sx, sy, i, j, k) ((size_t)(i) + (size_t)(sx) * ((size_t)(j) + (size_t)(sy) * (size_t)(k)))
#define IBV(v, i, j, k) ((v).a[VI((v).sx, (v).sy, i, j, k)])
#define MG1(c, d, arr, i, lev) ((c)->arr[d][(size_t)(i) + (size_t)((c)->n[d] + 2) * (size_t)((lev) - 1)])

static void *zalloc(size_t n) { return calloc(n ? n : 1, 1); }
static inline double sq_inv(double t) { return 1.0 / (t * t); }

/* ---------------------------------------------------------------- tdma ---- */
/* IBM/CORE_TDMA.F90:10-34: Thomas algorithm, no pivoting; a(n1), c(n2) unused.
 * gam is caller-provided work space of length n2+1 (the reference's automatic array). */
static void tdma_w(const double *a, const double *b, const double *c_, const double *r,
                   double *u, double *gam, int n1, int n2)
{
    double binv = 1.0 / b[n1];
    u[n1] = r[n1] * binv;
    for (int j = n1 + 1; j <= n2; ++j) {
        gam[j] = c_[j - 1] * binv;
        binv = 1.0 / (b[j] - a[j] * gam[j]);
        u[j] = (r[j] - a[j] * u[j - 1]) * binv;
    }
    for (int j = n2 - 1; j >= n1; --j) u[j] = u[j] - gam[j + 1] * u[j + 1];
}

void or_tdma(const double *a, const double *b, const double *c_, const double *r,
             double *u, int n1, int n2)
{
    double *gam = (double *)zalloc(sizeof(double) * (size_t)(n2 + 1));
    tdma_w(a, b, c_, r, u, gam, n1, n2);
    free(gam);
}

/* ------------------------------------------------------------ MG_initial -- */
/* IBM/CORE_MG.F90:31-278 */
static int auto_levels(int cells)
{
    const int nCoarseGrids = 4, MG_LEVEL_MAX = 10;
    int ii = cells, nLevel;
    for (nLevel = 1; nLevel <= MG_LEVEL_MAX; ++nLevel) {
        ii = ii / 2;
        if (ii >= nCoarseGrids) continue;
        break;
    }
    if (nLevel > MG_LEVEL_MAX) nLevel = MG_LEVEL_MAX; /* Fortran DO exit value is MAX+1; never reached for <=1M cells */
    return nLevel;
}

static void mg_initial(or_ctx *c)
{
    for (int d = 0; d < 3; ++d) {
        int N = c->n[d];
        int cells = (d == 2) ? (c->nz - 1) : c->nc[d];
        int nl = c->p.mgLevels[d];
        if (nl == 0) nl = auto_levels(cells);
        if (d == 2 && c->p.ndim == DIM_2D) nl = (c->p.mgLevels[2] == 0) ? auto_levels(c->nz - 1) : c->p.mgLevels[2];
        c->nlev[d] = nl;
        c->mgrid[d] = (int *)zalloc(sizeof(int) * (size_t)(nl + 2));
        c->mgrid[d][1] = c->nc[d];
        for (int l = 2; l <= nl; ++l) {
            int m = c->mgrid[d][l - 1];
            c->mgrid[d][l] = (m % 2 == 0) ? m / 2 : (m - 1) / 2;
        }
        size_t sz = sizeof(double) * (size_t)(N + 2) * (size_t)nl;
        c->x_MG[d] = zalloc(sz); c->xc_MG[d] = zalloc(sz); c->dx_MG[d] = zalloc(sz);
        c->dxinv_MG[d] = zalloc(sz); c->dxc_MG[d] = zalloc(sz); c->dxcinv_MG[d] = zalloc(sz);
        for (int i = 0; i <= N; ++i) {           /* :148-176 */
            MG1(c, d, dxc_MG, i, 1) = c->dxc[d][i];
            MG1(c, d, dx_MG, i, 1) = c->dx[d][i];
            MG1(c, d, dxcinv_MG, i, 1) = c->dxcinv[d][i];
            MG1(c, d, dxinv_MG, i, 1) = c->dxinv[d][i];
            MG1(c, d, xc_MG, i, 1) = c->xc[d][i];
        }
        for (int i = 0; i <= N + 1; ++i) MG1(c, d, x_MG, i, 1) = c->x[d][i]; /* :178-188 */
        if (d == 2 && c->p.ndim != DIM_3D) continue;
        for (int l = 2; l <= nl; ++l) {          /* :190-205 (x), :212-231 (y), :234-266 (z) */
            int m = c->mgrid[d][l];
            for (int i = 1; i <= m + 1; ++i) MG1(c, d, x_MG, i, l) = MG1(c, d, x_MG, 2 * i - 1, l - 1);
            MG1(c, d, x_MG, 0, l) = -MG1(c, d, x_MG, 2, l);
            MG1(c, d, x_MG, m + 2, l) = 2.0 * MG1(c, d, x_MG, m + 1, l) - MG1(c, d, x_MG, m, l);
            for (int i = 0; i <= m + 1; ++i) {
                MG1(c, d, dx_MG, i, l) = MG1(c, d, x_MG, i + 1, l) - MG1(c, d, x_MG, i, l);
                MG1(c, d, dxinv_MG, i, l) = 1.0 / MG1(c, d, dx_MG, i, l);
            }
            for (int i = 0; i <= m + 1; ++i)
                MG1(c, d, xc_MG, i, l) = 0.5 * (MG1(c, d, x_MG, i, l) + MG1(c, d, x_MG, i + 1, l));
            for (int i = 1; i <= m + 1; ++i) {
                MG1(c, d, dxc_MG, i, l) = MG1(c, d, xc_MG, i, l) - MG1(c, d, xc_MG, i - 1, l);
                MG1(c, d, dxcinv_MG, i, l) = 1.0 / MG1(c, d, dxc_MG, i, l);
            }
        }
    }
}

/* ------------------------------------------------------------ create ------ */
or_ctx *or_create(const fsi_mg_params *p, const double *x, const double *y, const double *z)
{
    if (!p || !x || !y || !z) return NULL;
    if (p->ndim != DIM_2D && p->ndim != DIM_3D) return NULL;
    if (p->nx < 3 || p->ny < 3 || p->nz < 2) return NULL;
    if (p->ndim == DIM_2D && p->nz != 2) return NULL;
    for (int s = 0; s < 6; ++s) if (p->bc[s] == BC_PERIODIC) return NULL;
    or_ctx *c = (or_ctx *)zalloc(sizeof(or_ctx));
    c->p = *p;
    c->nx = p->nx; c->ny = p->ny; c->nz = p->nz;
    c->nxc = p->nx - 1; c->nyc = p->ny - 1; c->nzc = p->nz - 1;
    c->n[0] = c->nx; c->n[1] = c->ny; c->n[2] = c->nz;
    c->nc[0] = c->nxc; c->nc[1] = c->nyc; c->nc[2] = c->nzc;
    const double *xs[3] = {x, y, z};
    /* IBM/CORE_GRID.F90:96-139 (metrics of the given nodes x(0:n+1)) */
    for (int d = 0; d < 3; ++d) {
        int N = c->n[d];
        size_t sz = sizeof(double) * (size_t)(N + 2);
        c->x[d] = zalloc(sz); c->xc[d] = zalloc(sz); c->dx[d] = zalloc(sz);
        c->dxinv[d] = zalloc(sz); c->dxc[d] = zalloc(sz); c->dxcinv[d] = zalloc(sz);
        memcpy(c->x[d], xs[d], sz);
        for (int i = 0; i <= N; ++i) {
            c->xc[d][i] = 0.5 * (c->x[d][i + 1] + c->x[d][i]);
            c->dx[d][i] = c->x[d][i + 1] - c->x[d][i];
            c->dxinv[d][i] = 1.0 / c->dx[d][i];
        }
        c->xc[d][N + 1] = c->x[d][N + 1];
        for (int i = 1; i <= N; ++i) {
            c->dxc[d][i] = c->xc[d][i] - c->xc[d][i - 1];
            c->dxcinv[d][i] = 1.0 / c->dxc[d][i];
        }
    }
    mg_initial(c);
    size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    c->iblank = zalloc(nf); c->ghost = zalloc(nf);
    for (int s = 0; s < 6; ++s) { c->fl[s] = zalloc(nf); c->flMG[s] = zalloc(nf); }
    c->ghostMG = zalloc(nf * sizeof(int));
    c->nlw = zalloc(nf * sizeof(double));
    c->nlw0 = zalloc(nf * sizeof(double));
    int pgs[6][2] = {{c->ny + 2, c->nz + 2}, {c->ny + 2, c->nz + 2}, {c->nx + 2, c->nz + 2},
                     {c->nx + 2, c->nz + 2}, {c->nx + 2, c->ny + 2}, {c->nx + 2, c->ny + 2}};
    for (int s = 0; s < 6; ++s) {
        c->pg_sx[s] = pgs[s][0];
        c->pgrad[s] = zalloc(sizeof(double) * (size_t)pgs[s][0] * (size_t)pgs[s][1]);
    }
    for (int d = 0; d < 3; ++d) {
        c->cib[d] = (int8_t **)zalloc(sizeof(int8_t *) * (size_t)(c->nlev[d] + 1));
        for (int l = 2; l <= c->nlev[d]; ++l) {
            size_t e[3] = {(size_t)c->nx + 1, (size_t)c->ny + 1, (size_t)c->nz + 1};
            e[d] = (size_t)c->mgrid[d][l] + 2;
            c->cib[d][l] = zalloc(e[0] * e[1] * e[2]);
        }
    }
    /* default flags: set_outer_iup (IBM/BOUNDARY_SET.F90:54-80) */
    for (int j = 1; j <= c->ny; ++j) for (int k = 1; k <= c->nz; ++k) {
        c->fl[0][FI(c, 1, j, k)] = 1; c->fl[1][FI(c, c->nxc, j, k)] = 1; }
    for (int i = 1; i <= c->nx; ++i) for (int k = 1; k <= c->nz; ++k) {
        c->fl[2][FI(c, i, 1, k)] = 1; c->fl[3][FI(c, i, c->nyc, k)] = 1; }
    if (c->p.ndim == DIM_3D)
        for (int i = 1; i <= c->nx; ++i) for (int j = 1; j <= c->ny; ++j) {
            c->fl[4][FI(c, i, j, 1)] = 1; c->fl[5][FI(c, i, j, c->nzc)] = 1; }
    return c;
}

void or_destroy(or_ctx *c)
{
    if (!c) return;
    free(c->vg_coeff); free(c->vg_bi);
    for (int q = 0; q < 6; ++q) free(c->ad[q]);
    free(c->fresh);
    for (int d = 0; d < 3; ++d) {
        free(c->x[d]); free(c->xc[d]); free(c->dx[d]); free(c->dxinv[d]); free(c->dxc[d]); free(c->dxcinv[d]);
        free(c->x_MG[d]); free(c->xc_MG[d]); free(c->dx_MG[d]); free(c->dxinv_MG[d]);
        free(c->dxc_MG[d]); free(c->dxcinv_MG[d]); free(c->mgrid[d]);
        if (c->cib[d]) for (int l = 2; l <= c->nlev[d]; ++l) free(c->cib[d][l]);
        free(c->cib[d]);
    }
    free(c->iblank); free(c->ghost); free(c->ghostMG); free(c->nlw); free(c->nlw0);
    for (int s = 0; s < 6; ++s) { free(c->fl[s]); free(c->flMG[s]); free(c->pgrad[s]); free(c->gi[s]); }
    free(c->coeff); free(c->probe);
    free(c);
}

int or_set_geometry(or_ctx *c, const int8_t *iblank, const int8_t *ghost,
                    const int8_t *ium, const int8_t *iup, const int8_t *jum,
                    const int8_t *jup, const int8_t *kum, const int8_t *kup,
                    int nGhost, const int32_t *iG, const int32_t *jG, const int32_t *kG,
                    const int32_t *iCI, const int32_t *jCI, const int32_t *kCI,
                    const double *coeffGCMN, const double *probeLength, const double *pgrad)
{
    size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    if (iblank) memcpy(c->iblank, iblank, nf);
    if (ghost) memcpy(c->ghost, ghost, nf);
    const int8_t *f[6] = {ium, iup, jum, jup, kum, kup};
    for (int s = 0; s < 6; ++s) if (f[s]) memcpy(c->fl[s], f[s], nf);
    for (int s = 0; s < 6; ++s) { free(c->gi[s]); c->gi[s] = NULL; }
    free(c->coeff); free(c->probe); c->coeff = c->probe = NULL;
    c->nGhost = nGhost;
    if (nGhost > 0) {
        const int32_t *g[6] = {iG, jG, kG, iCI, jCI, kCI};
        for (int s = 0; s < 6; ++s) {
            c->gi[s] = zalloc(sizeof(int32_t) * (size_t)nGhost);
            memcpy(c->gi[s], g[s], sizeof(int32_t) * (size_t)nGhost);
        }
        c->coeff = zalloc(sizeof(double) * 8 * (size_t)nGhost);
        memcpy(c->coeff, coeffGCMN, sizeof(double) * 8 * (size_t)nGhost);
        c->probe = zalloc(sizeof(double) * (size_t)nGhost);
        memcpy(c->probe, probeLength, sizeof(double) * (size_t)nGhost);
        for (int n = 0; n < nGhost; ++n)
            for (int r = 0; r < 8; ++r) {
                int ii = iCI[n] + incI[r], jj = jCI[n] + incJ[r], kk = kCI[n] + incK[r];
                if (ii < 0 || ii > c->nx || jj < 0 || jj > c->ny || kk < 0 || kk > c->nz) return -3;
            }
    }
    if (pgrad) {
        size_t off = 0;
        for (int s = 0; s < 6; ++s) {
            int sy = (s < 2) ? c->nz + 2 : (s < 4 ? c->nz + 2 : c->ny + 2);
            size_t cnt = (size_t)c->pg_sx[s] * (size_t)sy;
            memcpy(c->pgrad[s], pgrad + off, sizeof(double) * cnt);
            off += cnt;
        }
    }
    c->geometry_set = 1;
    return 0;
}

void or_get_pgrad(or_ctx *c, double *pgrad)
{
    size_t off = 0;
    for (int s = 0; s < 6; ++s) {
        int sy = (s < 4) ? c->nz + 2 : c->ny + 2;
        size_t cnt = (size_t)c->pg_sx[s] * (size_t)sy;
        memcpy(pgrad + off, c->pgrad[s], sizeof(double) * cnt);
        off += cnt;
    }
}

/* ------------------------------------------------ outer ghost / ghost rows */
/* IBM/CORE_SET_OUTER_GHOST.F90:66-213; pres is (0:mx,0:my,0:mz), loops use nx,ny,nz. */
static void set_outer_ghost_pres(or_ctx *c, double *pres, int mx, int my)
{
    int nx = c->nx, ny = c->ny, nz = c->nz;
    int sx = mx + 1, sy = my + 1;
#define P(i, j, k) pres[VI(sx, sy, i, j, k)]
    const int *pbc = c->p.pbc;
    for (int k = 0; k <= nz; ++k) for (int j = 0; j <= ny; ++j)
        P(0, j, k) = (pbc[0] == PBC_NEUMANN) ? P(1, j, k) : -P(1, j, k);
    for (int k = 0; k <= nz; ++k) for (int j = 0; j <= ny; ++j)
        P(nx, j, k) = (pbc[1] == PBC_NEUMANN) ? P(nx - 1, j, k) : -P(nx - 1, j, k);
    for (int k = 0; k <= nz; ++k) for (int i = 0; i <= nx; ++i)
        P(i, 0, k) = (pbc[2] == PBC_NEUMANN) ? P(i, 1, k) : -P(i, 1, k);
    for (int k = 0; k <= nz; ++k) for (int i = 0; i <= nx; ++i)
        P(i, ny, k) = (pbc[3] == PBC_NEUMANN) ? P(i, ny - 1, k) : -P(i, ny - 1, k);
    if (c->p.ndim == DIM_3D)
        for (int j = 0; j <= ny; ++j) for (int i = 0; i <= nx; ++i) {
            P(i, j, 0) = P(i, j, 1);
            P(i, j, nz) = P(i, j, nz - 1);
        }
    for (int j = 0; j <= ny; ++j) for (int i = 0; i <= nx; ++i)
        P(i, j, 0) = (pbc[4] == PBC_NEUMANN) ? P(i, j, 1) : -P(i, j, 1);
    for (int j = 0; j <= ny; ++j) for (int i = 0; i <= nx; ++i)
        P(i, j, nz) = (pbc[5] == PBC_NEUMANN) ? P(i, j, nz - 1) : -P(i, j, nz - 1);
#undef P
}

/* IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:250-384 (viscous: uNormal = 0).
 * Gauss-Seidel over the ordered ghost list until max|dp| <= restol_ad. */
static void gcm_p_set_bc_internal(or_ctx *c, double *pres, int mx, int my)
{
    int sx = mx + 1, sy = my + 1;
    int iterGC = 0;
    double resPresMax = 1.0e10;
    const double uNormal = 0.0;
    while (iterGC < c->p.iterMax_ad && resPresMax > c->p.restol_ad) {
        resPresMax = 0.0;
        for (int n = 0; n < c->nGhost; ++n) {
            int iG = c->gi[0][n], jG = c->gi[1][n], kG = c->gi[2][n];
            double pIP = 0.0;
            for (int r = 0; r < 8; ++r) {
                int ii = c->gi[3][n] + incI[r], jj = c->gi[4][n] + incJ[r], kk = c->gi[5][n] + incK[r];
                if (ii == iG && jj == jG && kk == kG) pIP = pIP + c->coeff[8 * (size_t)n + r] * uNormal;
                else pIP = pIP + c->coeff[8 * (size_t)n + r] * pres[VI(sx, sy, ii, jj, kk)];
            }
            size_t g = VI(sx, sy, iG, jG, kG);
            double pPrev = pres[g];
            pres[g] = pIP + c->probe[n] * uNormal;
            double resPres = fabs(pres[g] - pPrev);
            if (resPres > resPresMax) resPresMax = resPres;
        }
        iterGC = iterGC + 1;
    }
    c->gs_last_iters = iterGC;
    if (iterGC == c->p.iterMax_ad && resPresMax > c->p.restol_ad) c->ghost_nonconv = 1;
}

void or_ghost_update(or_ctx *c, double *var, int mx, int my, int mz, int *iters, double *resmax)
{
    (void)mz;
    c->ghost_nonconv = 0;
    gcm_p_set_bc_internal(c, var, mx, my);
    if (iters) *iters = c->gs_last_iters;
    if (resmax) *resmax = (double)c->ghost_nonconv;
}

int or_nghost_gs_last(or_ctx *c) { return c->gs_last_iters; }

/* set_outer_ghost_pres on an MG-layout (0:nx,0:ny,0:nz) array. */
void or_outer_ghost(or_ctx *c, double *var) { set_outer_ghost_pres(c, var, c->nx, c->ny); }

/* IBM/GCM_GLOBAL_MASS_CONSERVE.F90:260-394 (non-periodic branch). */
static void gcm_enforce_p_compatibility(or_ctx *c, const double *pres, int mx, int my)
{
    const int *bc = c->p.bc;
    int active = 0;
    for (int s = 0; s < 6; ++s) if (bc[s] == BC_ZERO_GRADIENT) active = 1;
    if (!active) return;
    int sx = mx + 1, sy = my + 1;
#define P(i, j, k) pres[VI(sx, sy, i, j, k)]
#define PG(s, a, b) c->pgrad[s][(size_t)(a) + (size_t)c->pg_sx[s] * (size_t)(b)]
    double pgradflux = 0.0;
    double *dxcinv = c->dxcinv[0], *dycinv = c->dxcinv[1], *dzcinv = c->dxcinv[2];
    double *dx = c->dx[0], *dy = c->dx[1], *dz = c->dx[2];
    for (int k = 1; k <= c->nz - 1; ++k)
        for (int j = 1; j <= c->ny - 1; ++j)
            for (int i = 1; i <= c->nx - 1; ++i) {
                size_t f = FI(c, i, j, k);
                int ium = c->fl[0][f], iup = c->fl[1][f], jum = c->fl[2][f];
                int jup = c->fl[3][f], kum = c->fl[4][f], kup = c->fl[5][f];
                double pgxw = PG(0, j, k) * ium + ((double)(1 - ium) * (P(i, j, k) - P(i - 1, j, k))) * dxcinv[i];
                double pgxe = PG(1, j, k) * iup + ((double)(1 - iup) * (P(i + 1, j, k) - P(i, j, k))) * dxcinv[i + 1];
                double pgys = PG(2, i, k) * jum + ((double)(1 - jum) * (P(i, j, k) - P(i, j - 1, k))) * dycinv[j];
                double pgyn = PG(3, i, k) * jup + ((double)(1 - jup) * (P(i, j + 1, k) - P(i, j, k))) * dycinv[j + 1];
                double pgzb = PG(4, i, j) * kum + ((double)(1 - kum) * (P(i, j, k) - P(i, j, k - 1))) * dzcinv[k];
                double pgzf = PG(5, i, j) * kup + ((double)(1 - kup) * (P(i, j, k + 1) - P(i, j, k))) * dzcinv[k + 1];
                pgradflux = pgradflux +
                    (-(pgxw * dy[j] * dz[k]) + pgxe * dy[j] * dz[k] - pgys * dx[i] * dz[k] +
                     pgyn * dx[i] * dz[k] - pgzb * dx[i] * dy[j] + pgzf * dx[i] * dy[j]) *
                    (double)(1 - c->iblank[f]);
            }
    double corr = -pgradflux / c->p.outflow_area;
    for (int k = 0; k <= c->nz; ++k) for (int j = 0; j <= c->ny; ++j) {
        if (bc[0] == BC_ZERO_GRADIENT) PG(0, j, k) = PG(0, j, k) - corr;
        if (bc[1] == BC_ZERO_GRADIENT) PG(1, j, k) = PG(1, j, k) + corr;
    }
    for (int k = 0; k <= c->nz; ++k) for (int i = 0; i <= c->nx; ++i) {
        if (bc[2] == BC_ZERO_GRADIENT) PG(2, i, k) = PG(2, i, k) - corr;
        if (bc[3] == BC_ZERO_GRADIENT) PG(3, i, k) = PG(3, i, k) + corr;
    }
    for (int j = 0; j <= c->ny; ++j) for (int i = 0; i <= c->nx; ++i) {
        if (bc[4] == BC_ZERO_GRADIENT) PG(4, i, j) = PG(4, i, j) - corr;
        if (bc[5] == BC_ZERO_GRADIENT) PG(5, i, j) = PG(5, i, j) + corr;
    }
#undef P
#undef PG
}

/* IBM/CORE_POISSON.F90:1794-1823 on a full (0:nx+1)^3 array. */
void or_gcm_correct_pressure(or_ctx *c, double *p)
{
    set_outer_ghost_pres(c, p, c->nx + 1, c->ny + 1);
    gcm_p_set_bc_internal(c, p, c->nx + 1, c->ny + 1);
    gcm_enforce_p_compatibility(c, p, c->nx + 1, c->ny + 1);
#define PG(s, a, b) c->pgrad[s][(size_t)(a) + (size_t)c->pg_sx[s] * (size_t)(b)]
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                size_t f = FI(c, i, j, k);
                const double pot = 0.0;
                c->nlw0[f] = -(c->dxinv[0][i] * (c->fl[1][f] * PG(1, j, k) - c->fl[0][f] * PG(0, j, k)) * (1.0 - pot))
                             - c->dxinv[1][j] * (c->fl[3][f] * PG(3, i, k) - c->fl[2][f] * PG(2, i, k)) * (1.0 - pot)
                             - c->dxinv[2][k] * (c->fl[5][f] * PG(5, i, j) - c->fl[4][f] * PG(4, i, j)) * (1.0 - pot);
            }
#undef PG
}

/* ---------------------------------------------------- MG bookkeeping ---- */
/* IBM/CORE_MG.F90:699-822 MG_Prepare_Iblank (also zeroes coarse ghost marks without a body). */
static void mg_prepare_iblank(or_ctx *c, int d)
{
    for (int l = 2; l <= c->nlev[d]; ++l) {
        size_t e[3] = {(size_t)c->nx + 1, (size_t)c->ny + 1, (size_t)c->nz + 1};
        e[d] = (size_t)c->mgrid[d][l] + 2;
        memset(c->cib[d][l], 0, e[0] * e[1] * e[2]);
    }
    int ext[3] = {c->nxc, c->nyc, c->nzc};
    for (int l = 2; l <= c->nlev[d]; ++l) {
        int sx = (d == 0) ? c->mgrid[0][l] + 2 : c->nx + 1;
        int sy = (d == 1) ? c->mgrid[1][l] + 2 : c->ny + 1;
        int e[3] = {ext[0], ext[1], ext[2]};
        e[d] = c->mgrid[d][l];
        if (c->p.internal_boundary_present == 1) {
            int psx = (l > 2) ? ((d == 0) ? c->mgrid[0][l - 1] + 2 : c->nx + 1) : c->nx + 2;
            int psy = (l > 2) ? ((d == 1) ? c->mgrid[1][l - 1] + 2 : c->ny + 1) : c->ny + 2;
            const int8_t *prev = (l > 2) ? c->cib[d][l - 1] : c->iblank;
            for (int k = 1; k <= e[2]; ++k)
                for (int j = 1; j <= e[1]; ++j)
                    for (int i = 1; i <= e[0]; ++i) {
                        int a[3] = {i, j, k}, b[3] = {i, j, k};
                        a[d] = 2 * a[d] - 1; b[d] = 2 * b[d];
                        c->cib[d][l][VI(sx, sy, i, j, k)] =
                            (int8_t)(prev[VI(psx, psy, a[0], a[1], a[2])] * prev[VI(psx, psy, b[0], b[1], b[2])]);
                    }
        } else {
            for (int k = 1; k <= e[2]; ++k)
                for (int j = 1; j <= e[1]; ++j)
                    for (int i = 1; i <= e[0]; ++i) c->ghostMG[FI(c, i, j, k)] = 0;
        }
    }
}

static i8v ib_view(or_ctx *c, int d, int l)
{
    i8v v;
    if (l <= 1) { v.a = c->iblank; v.sx = c->nx + 2; v.sy = c->ny + 2; return v; }
    v.a = c->cib[d][l];
    v.sx = (d == 0) ? c->mgrid[0][l] + 2 : c->nx + 1;
    v.sy = (d == 1) ? c->mgrid[1][l] + 2 : c->ny + 1;
    return v;
}

static void gcm_pressure(or_ctx *c, double *var, double *rhs);

/* IBM/CORE_MG.F90:1667-1713 MG_Prepare_BC */
static void mg_prepare_bc(or_ctx *c, int l)
{
    size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    if (l == 1) {
        for (int s = 0; s < 6; ++s) memcpy(c->flMG[s], c->fl[s], nf);
        if (c->p.internal_boundary_present == 1)
            for (size_t q = 0; q < nf; ++q) c->ghostMG[q] = c->ghost[q];
        if (c->p.boundary_formulation == GCM_METHOD) {
            /* GCM_correct_pressure acts on the module pPrime, not on the MG copy */
            if (c->pPrime_mod) or_gcm_correct_pressure(c, c->pPrime_mod);
        } else {
            memset(c->nlw, 0, nf * sizeof(double));
        }
    } else if (c->p.internal_boundary_present == 1) {
        memset(c->ghostMG, 0, nf * sizeof(int));
        memset(c->nlw, 0, nf * sizeof(double));
    }
}

/* IBM/CORE_MG.F90:1716-1879 MG_Prepare(nlev, mx, my, mz) with mx.. = cell counts. */
static void mg_prepare(or_ctx *c, int mx, int my, int mz)
{
    i8v ib = c->ibMG;
#define FL(s, i, j, k) c->flMG[s][FI(c, i, j, k)]
#define UPF(a, b) ((int8_t)(int)((double)((int)(a) - (int)(b)) / 2.0 + 0.5))
    if (c->p.internal_boundary_present == 1 || c->p.coarse_flag_mode == 1) {
        for (int k = 1; k <= mz; ++k) {
            for (int j = 1; j <= my; ++j) {
                for (int i = 1; i <= mx - 1; ++i) FL(1, i, j, k) = UPF(IBV(ib, i + 1, j, k), IBV(ib, i, j, k));
                for (int i = 2; i <= mx; ++i) FL(0, i, j, k) = UPF(IBV(ib, i - 1, j, k), IBV(ib, i, j, k));
            }
            for (int j = 1; j <= my - 1; ++j)
                for (int i = 1; i <= mx; ++i) FL(3, i, j, k) = UPF(IBV(ib, i, j + 1, k), IBV(ib, i, j, k));
            for (int j = 2; j <= my; ++j)
                for (int i = 1; i <= mx; ++i) FL(2, i, j, k) = UPF(IBV(ib, i, j - 1, k), IBV(ib, i, j, k));
        }
        for (int j = 1; j <= my; ++j)
            for (int i = 1; i <= mx; ++i) {
                for (int k = 1; k <= mz - 1; ++k) FL(5, i, j, k) = UPF(IBV(ib, i, j, k + 1), IBV(ib, i, j, k));
                for (int k = 2; k <= mz; ++k) FL(4, i, j, k) = UPF(IBV(ib, i, j, k - 1), IBV(ib, i, j, k));
            }
    }
    const int *pbc = c->p.pbc;
    for (int k = 1; k <= mz; ++k) for (int j = 1; j <= my; ++j) {
        FL(0, 1, j, k) = (pbc[0] == PBC_DIRICHLET) ? -1 : 1;
        FL(1, mx, j, k) = (pbc[1] == PBC_DIRICHLET) ? -1 : 1;
    }
    for (int k = 1; k <= mz; ++k) for (int i = 1; i <= mx; ++i) {
        FL(2, i, 1, k) = (pbc[2] == PBC_DIRICHLET) ? -1 : 1;
        FL(3, i, my, k) = (pbc[3] == PBC_DIRICHLET) ? -1 : 1;
    }
    for (int j = 1; j <= my; ++j) for (int i = 1; i <= mx; ++i) {
        FL(4, i, j, 1) = (pbc[4] == PBC_DIRICHLET) ? -1 : 1;
        FL(5, i, j, mz) = (pbc[5] == PBC_DIRICHLET) ? -1 : 1;
    }
#undef FL
#undef UPF
}

/* --------------------------------------------------------- MG_itsolv ---- */
/* IBM/CORE_MG.F90:1883-2270.  Coefficients for cell (i,j,k) at levels (lx,ly,lz). */
typedef struct { double amx, apx, acx, amy, apy, acy, amz, apz, acz; } coefs9;

static inline coefs9 cell_coefs(or_ctx *c, int i, int j, int k, int lx, int ly, int lz)
{
    coefs9 q;
    size_t f = FI(c, i, j, k);
    double d2 = (double)(c->p.ndim - DIM_2D);
    q.amx = MG1(c, 0, dxcinv_MG, i, lx) * MG1(c, 0, dxinv_MG, i, lx) * (1.0 - (double)c->flMG[0][f]);
    q.apx = MG1(c, 0, dxcinv_MG, i + 1, lx) * MG1(c, 0, dxinv_MG, i, lx) * (1.0 - (double)c->flMG[1][f]);
    q.acx = -(q.amx + q.apx);
    q.amy = MG1(c, 1, dxcinv_MG, j, ly) * MG1(c, 1, dxinv_MG, j, ly) * (1.0 - (double)c->flMG[2][f]);
    q.apy = MG1(c, 1, dxcinv_MG, j + 1, ly) * MG1(c, 1, dxinv_MG, j, ly) * (1.0 - (double)c->flMG[3][f]);
    q.acy = -(q.amy + q.apy);
    q.amz = MG1(c, 2, dxcinv_MG, k, lz) * MG1(c, 2, dxinv_MG, k, lz) * (1.0 - (double)c->flMG[4][f]) * d2;
    q.apz = MG1(c, 2, dxcinv_MG, k + 1, lz) * MG1(c, 2, dxinv_MG, k, lz) * (1.0 - (double)c->flMG[5][f]) * d2;
    q.acz = -(q.amz + q.apz);
    return q;
}

static int line_active(or_ctx *c, int dir, int colour, int a, int b)
{
    /* colour schedule; returns 1 when the line indexed (a,b) is visited in pass `colour` */
    int rb = c->p.iRedBlack;
    int nd = c->p.ndim;
    if (rb == 3) return ((a + b) & 1) == (colour == 0 ? 0 : 1);
    if (rb == 0) return colour == 0;
    /* reference colour loops, IBM/MAIN.F90:548-571 and IBM/CORE_MG.F90:1921-1923,2043-2046,2165-2168 */
    int TNx = 2, TNy = (rb == 1) ? 1 : 2, TNz = (rb == 1) ? 1 : 2;
    int iStep = (rb == 1) ? 1 : 2, jStep = 2, kStep = (nd - DIM_2D) + 1;
    int Ncolor = colour + 1;
    if (dir == 0) {           /* a = j, b = k */
        if (Ncolor > TNx) return 0;
        int kinit = (Ncolor - 1) * (nd - DIM_2D) + 1, jinit = Ncolor;
        return b >= kinit && (b - kinit) % kStep == 0 && a >= jinit && (a - jinit) % jStep == 0;
    } else if (dir == 1) {    /* a = i, b = k */
        if (Ncolor > TNy) return 0;
        int kinit = (Ncolor - 1) * (nd - DIM_2D) + 1, iinit = Ncolor;
        return b >= kinit && (b - kinit) % kStep == 0 && a >= iinit && (a - iinit) % iStep == 0;
    } else {                  /* a = i, b = j */
        if (Ncolor > TNz) return 0;
        int jinit = Ncolor, iinit = Ncolor;
        return b >= jinit && (b - jinit) % jStep == 0 && a >= iinit && (a - iinit) % iStep == 0;
    }
}

static void mg_itsolv(or_ctx *c, double *var, const double *R, int lx, int ly, int lz, int mx, int my, int mz)
{
    int sx = mx + 1, sy = my + 1;
    int nmax = mx > my ? mx : my; if (mz > nmax) nmax = mz;
    double *am = zalloc(sizeof(double) * (size_t)(nmax + 2)), *ac = zalloc(sizeof(double) * (size_t)(nmax + 2));
    double *ap = zalloc(sizeof(double) * (size_t)(nmax + 2)), *rhs = zalloc(sizeof(double) * (size_t)(nmax + 2));
    double *sol = zalloc(sizeof(double) * (size_t)(nmax + 2));
    double *gam = zalloc(sizeof(double) * (size_t)(nmax + 2));
    i8v ib = c->ibMG;
    const double om = c->p.omega;
    const int finest = (lx * ly * lz == 1);
    const int *pbc = c->p.pbc;
    const double *ppp = c->p.ppp;
    const double tiny = (double)1.0e-12f;
#define V(i, j, k) var[VI(sx, sy, i, j, k)]
    int ncol = (c->p.iRedBlack == 0) ? 1 : 2;
    /* x-lines */
    for (int col = 0; col < ncol; ++col)
        for (int k = 1; k <= mz - 1; ++k)
            for (int j = 1; j <= my - 1; ++j) {
                if (!line_active(c, 0, col, j, k)) continue;
                for (int i = 1; i <= mx - 1; ++i) {
                    coefs9 q = cell_coefs(c, i, j, k, lx, ly, lz);
                    size_t f = FI(c, i, j, k);
                    double r = R[VI(sx, sy, i, j, k)] - V(i, j - 1, k) * q.amy - V(i, j + 1, k) * q.apy -
                               V(i, j, k - 1) * q.amz - V(i, j, k + 1) * q.apz + c->nlw[f];
                    double b = (double)IBV(ib, i, j, k);
                    am[i] = q.amx * (1.0 - b);
                    ap[i] = q.apx * (1.0 - b);
                    ac[i] = (q.acx + q.acy + q.acz) * (1.0 - b) + b;
                    rhs[i] = r * (1.0 - b) + (double)c->ghostMG[f] * V(i, j, k);
                    if (fabs(ac[i]) < tiny) { am[i] = 0.0; ap[i] = 0.0; ac[i] = 1.0; rhs[i] = V(i, j, k); }
                }
                if (pbc[0] == PBC_DIRICHLET && finest) rhs[1] = rhs[1] - ppp[0] * am[1];
                if (pbc[1] == PBC_DIRICHLET && finest) rhs[mx - 1] = rhs[mx - 1] - ppp[1] * ap[mx - 1];
                tdma_w(am, ac, ap, rhs, sol, gam, 1, mx - 1);
                for (int i = 1; i <= mx - 1; ++i) V(i, j, k) = V(i, j, k) * (1.0 - om) + om * sol[i];
                if (pbc[0] == PBC_DIRICHLET && finest) V(0, j, k) = ppp[0];
                if (pbc[1] == PBC_DIRICHLET && finest) V(mx, j, k) = ppp[1];
            }
    /* y-lines */
    for (int col = 0; col < ncol; ++col)
        for (int k = 1; k <= mz - 1; ++k)
            for (int i = 1; i <= mx - 1; ++i) {
                if (!line_active(c, 1, col, i, k)) continue;
                for (int j = 1; j <= my - 1; ++j) {
                    coefs9 q = cell_coefs(c, i, j, k, lx, ly, lz);
                    size_t f = FI(c, i, j, k);
                    double r = R[VI(sx, sy, i, j, k)] - V(i - 1, j, k) * q.amx - V(i + 1, j, k) * q.apx -
                               V(i, j, k - 1) * q.amz - V(i, j, k + 1) * q.apz + c->nlw[f];
                    double b = (double)IBV(ib, i, j, k);
                    am[j] = q.amy * (1.0 - b);
                    ap[j] = q.apy * (1.0 - b);
                    ac[j] = (q.acx + q.acy + q.acz) * (1.0 - b) + b;
                    rhs[j] = r * (1.0 - b) + (double)c->ghostMG[f] * V(i, j, k);
                    if (fabs(ac[j]) < tiny) { am[j] = 0.0; ap[j] = 0.0; ac[j] = 1.0; rhs[j] = V(i, j, k); }
                }
                if (pbc[2] == PBC_DIRICHLET && finest) rhs[1] = rhs[1] - ppp[2] * am[1];
                if (pbc[3] == PBC_DIRICHLET && finest) rhs[my - 1] = rhs[my - 1] - ppp[3] * ap[my - 1];
                tdma_w(am, ac, ap, rhs, sol, gam, 1, my - 1);
                for (int j = 1; j <= my - 1; ++j) V(i, j, k) = V(i, j, k) * (1.0 - om) + om * sol[j];
                if (pbc[2] == PBC_DIRICHLET && finest) V(i, 0, k) = ppp[2];
                if (pbc[3] == PBC_DIRICHLET && finest) V(i, my, k) = ppp[3];
            }
    /* z-lines */
    if (c->p.ndim == DIM_3D)
        for (int col = 0; col < ncol; ++col)
            for (int j = 1; j <= my - 1; ++j)
                for (int i = 1; i <= mx - 1; ++i) {
                    if (!line_active(c, 2, col, i, j)) continue;
                    for (int k = 1; k <= mz - 1; ++k) {
                        coefs9 q = cell_coefs(c, i, j, k, lx, ly, lz);
                        size_t f = FI(c, i, j, k);
                        double r = R[VI(sx, sy, i, j, k)] - V(i, j - 1, k) * q.amy - V(i, j + 1, k) * q.apy -
                                   V(i - 1, j, k) * q.amx - V(i + 1, j, k) * q.apx + c->nlw[f];
                        double b = (double)IBV(ib, i, j, k);
                        am[k] = q.amz * (1.0 - b);
                        ap[k] = q.apz * (1.0 - b);
                        ac[k] = (q.acx + q.acy + q.acz) * (1.0 - b) + b;
                        rhs[k] = r * (1.0 - b) + (double)c->ghostMG[f] * V(i, j, k);
                        if (fabs(ac[k]) < tiny) { am[k] = 0.0; ap[k] = 0.0; ac[k] = 1.0; rhs[k] = V(i, j, k); }
                    }
                    if (pbc[4] == PBC_DIRICHLET && finest) rhs[1] = rhs[1] - ppp[4] * am[1];
                    if (pbc[5] == PBC_DIRICHLET && finest) rhs[mz - 1] = rhs[mz - 1] - ppp[5] * ap[mz - 1];
                    tdma_w(am, ac, ap, rhs, sol, gam, 1, mz - 1);
                    for (int k = 1; k <= mz - 1; ++k) V(i, j, k) = V(i, j, k) * (1.0 - om) + om * sol[k];
                    if (pbc[4] == PBC_DIRICHLET && finest) V(i, j, 0) = ppp[4];
                    if (pbc[5] == PBC_DIRICHLET && finest) V(i, j, mz) = ppp[5];
                }
#undef V
    free(am); free(ac); free(ap); free(rhs); free(sol); free(gam);
}

/* IBM/CORE_MG.F90:2274-2387 MG_Residual */
static void mg_residual(or_ctx *c, const double *var, const double *R, double *resL,
                        int lx, int ly, int lz, int mx, int my, int mz)
{
    int sx = mx + 1, sy = my + 1;
    i8v ib = c->ibMG;
#define V(i, j, k) var[VI(sx, sy, i, j, k)]
    for (int k = 1; k <= mz - 1; ++k)
        for (int j = 1; j <= my - 1; ++j)
            for (int i = 1; i <= mx - 1; ++i) {
                coefs9 q = cell_coefs(c, i, j, k, lx, ly, lz);
                double b = (double)IBV(ib, i, j, k);
                double bmx = q.amx * (1.0 - b), bpx = q.apx * (1.0 - b);
                double bmy = q.amy * (1.0 - b), bpy = q.apy * (1.0 - b);
                double bmz = q.amz * (1.0 - b), bpz = q.apz * (1.0 - b);
                double bc = (q.acx + q.acy + q.acz) * (1.0 - b) + b;
                double res = R[VI(sx, sy, i, j, k)] - V(i, j, k) * bc - V(i - 1, j, k) * bmx - V(i + 1, j, k) * bpx -
                             V(i, j - 1, k) * bmy - V(i, j + 1, k) * bpy - V(i, j, k - 1) * bmz -
                             V(i, j, k + 1) * bpz + c->nlw[FI(c, i, j, k)];
                resL[VI(sx, sy, i, j, k)] = res * (1.0 - b);
            }
#undef V
}

/* IBM/CORE_MG.F90:2464-2723 MG_Restrict_X/Y/Z; nlev = fine level, m1 = coarse upper bound. */
static void mg_restrict(or_ctx *c, int d, const double *var, double *r, int nlev, int mx, int my, int mz, int m1)
{
    int sx = mx + 1, sy = my + 1;
    int csx = (d == 0) ? m1 + 1 : sx, csy = (d == 1) ? m1 + 1 : sy;
    i8v ib = c->ibMG;
    int e[3] = {mx - 1, my - 1, mz - 1};
    e[d] = m1 - 1;
    for (int k = 1; k <= e[2]; ++k)
        for (int j = 1; j <= e[1]; ++j)
            for (int i = 1; i <= e[0]; ++i) {
                int cc = (d == 0) ? i : (d == 1 ? j : k);
                int ii = 2 * cc, iim = 2 * cc - 1, iip = 2 * cc + 1;
                double area1 = MG1(c, d, x_MG, ii, nlev) - MG1(c, d, x_MG, iim, nlev);
                double area2 = MG1(c, d, x_MG, iip, nlev) - MG1(c, d, x_MG, ii, nlev);
                double area = area1 + area2;
                double w1 = area1 / area, w2 = area2 / area;
                int a[3] = {i, j, k}, b[3] = {i, j, k};
                a[d] = ii; b[d] = iim;
                double da = 1.0 - (double)IBV(ib, a[0], a[1], a[2]);
                double db = 1.0 - (double)IBV(ib, b[0], b[1], b[2]);
                double va = var[VI(sx, sy, a[0], a[1], a[2])], vb = var[VI(sx, sy, b[0], b[1], b[2])];
                double sum1 = da * w2 * va + db * w1 * vb;
                double temp = (d == 0) ? (da * w2 + db * w1) : (db * w1 + da * w2);
                r[VI(csx, csy, i, j, k)] = (temp > 0.0) ? sum1 / temp : sum1;
            }
}

/* IBM/CORE_MG.F90:2885-3523 MG_Prolong_X/Y/Z: coarse correc -> fine phi.
 * ibMG must be the coarse (nlev+1) view.  m1 = coarse upper bound, mfine = fine upper bound. */
static void mg_prolong(or_ctx *c, int d, double *phi, const double *correc, int nlev, int mx, int my, int mz,
                       int m1, int mfine)
{
    i8v ib = c->ibMG;
    int csx = (d == 0) ? m1 + 1 : mx + 1, csy = (d == 1) ? m1 + 1 : my + 1;
    int fsx = (d == 0) ? mfine + 1 : mx + 1, fsy = (d == 1) ? mfine + 1 : my + 1;
    int nc = m1 - 1;
    double *w1 = zalloc(sizeof(double) * (size_t)(nc + 2)), *w2 = zalloc(sizeof(double) * (size_t)(nc + 2));
    double *w3 = zalloc(sizeof(double) * (size_t)(nc + 2)), *w4 = zalloc(sizeof(double) * (size_t)(nc + 2));
    for (int i = 1; i <= nc; ++i) {
        int ii = 2 * i, iim = 2 * i - 1;
        double d1 = sq_inv(MG1(c, d, xc_MG, iim, nlev) - MG1(c, d, xc_MG, i, nlev + 1));
        double d2 = sq_inv(MG1(c, d, xc_MG, iim, nlev) - MG1(c, d, xc_MG, i - 1, nlev + 1));
        double de = d1 + d2;
        w1[i] = d1 / de; w2[i] = d2 / de;
        d1 = sq_inv(MG1(c, d, xc_MG, ii, nlev) - MG1(c, d, xc_MG, i, nlev + 1));
        d2 = sq_inv(MG1(c, d, xc_MG, ii, nlev) - MG1(c, d, xc_MG, i + 1, nlev + 1));
        de = d1 + d2;
        w3[i] = d1 / de; w4[i] = d2 / de;
    }
    /* the two other directions run over their interiors */
    int e[3] = {mx - 1, my - 1, mz - 1};
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    for (int b = 1; b <= e[o2]; ++b)
        for (int a = 1; a <= e[o1]; ++a) {
#define CIDX(q) ((d == 0) ? VI(csx, csy, q, a, b) : (d == 1) ? VI(csx, csy, a, q, b) : VI(csx, csy, a, b, q))
#define FIDX(q) ((d == 0) ? VI(fsx, fsy, q, a, b) : (d == 1) ? VI(fsx, fsy, a, q, b) : VI(fsx, fsy, a, b, q))
#define DIB(q) (1.0 - (double)((d == 0) ? IBV(ib, q, a, b) : (d == 1) ? IBV(ib, a, q, b) : IBV(ib, a, b, q)))
            phi[FIDX(1)] = correc[CIDX(1)];
            double delta1 = w3[1] * DIB(1), delta2 = w4[1] * DIB(2), delta = delta1 + delta2;
            phi[FIDX(2)] = delta1 * correc[CIDX(1)] + delta2 * correc[CIDX(2)];
            if (delta > 0.0) phi[FIDX(2)] = phi[FIDX(2)] / delta;
            for (int i = 2; i <= nc - 1; ++i) {
                int ii = 2 * i, iim = 2 * i - 1;
                double v1 = correc[CIDX(i)], v2 = correc[CIDX(i - 1)], v3 = correc[CIDX(i + 1)];
                delta1 = w1[i] * DIB(i); delta2 = w2[i] * DIB(i - 1); delta = delta1 + delta2;
                phi[FIDX(iim)] = delta1 * v1 + delta2 * v2;
                if (delta > 0.0) phi[FIDX(iim)] = phi[FIDX(iim)] / delta;
                delta1 = w3[i] * DIB(i); delta2 = w4[i] * DIB(i + 1); delta = delta1 + delta2;
                phi[FIDX(ii)] = delta1 * v1 + delta2 * v3;
                if (delta > 0.0) phi[FIDX(ii)] = phi[FIDX(ii)] / delta;
            }
            int i = nc, ii = 2 * nc, iim = 2 * nc - 1;
            delta1 = w1[i] * DIB(i); delta2 = w2[i] * DIB(i - 1); delta = delta1 + delta2;
            phi[FIDX(iim)] = delta1 * correc[CIDX(i)] + delta2 * correc[CIDX(i - 1)];
            if (delta > 0.0) phi[FIDX(iim)] = phi[FIDX(iim)] / delta;
            phi[FIDX(ii)] = correc[CIDX(i)];
            if (nlev == 1 && mfine - 1 > 2 * i) phi[FIDX(mfine - 1)] = correc[CIDX(i)];
#undef CIDX
#undef FIDX
#undef DIB
        }
    free(w1); free(w2); free(w3); free(w4);
}

/* IBM/CORE_MG.F90:4707-4743 GCM_Pressure on the MG copy (0:nx,0:ny,0:nz). */
static void gcm_pressure(or_ctx *c, double *var, double *rhs)
{
    (void)rhs;
    set_outer_ghost_pres(c, var, c->nx, c->ny);
    gcm_p_set_bc_internal(c, var, c->nx, c->ny);
    gcm_enforce_p_compatibility(c, var, c->nx, c->ny);
    mg_prepare_bc(c, 1);
}

/* IBM/CORE_MG.F90:1239-1663 MG_X / MG_Y / MG_Z (recursive), direction d. */
static void mg_cycle(or_ctx *c, int d, double *var, double *rhs, int n, int nlev, int mx, int my, int mz,
                     int WF, int *GMM, int mgCycle)
{
    int lev[3] = {1, 1, 1};
    lev[d] = n;
    c->ibMG = ib_view(c, d, n);
    int totIter = (n == 1) ? c->p.iterFinest : ((n == c->nlev[d]) ? c->p.iterCoarsest : 1);
    mg_prepare_bc(c, n);
    if (n != 1) mg_prepare(c, mx - 1, my - 1, mz - 1);
    int gcm = (c->p.boundary_formulation == GCM_METHOD);
    if (n == 1 && gcm) gcm_pressure(c, var, rhs);
    if (WF == 1)
        for (int it = 0; it < totIter; ++it) mg_itsolv(c, var, rhs, lev[0], lev[1], lev[2], mx, my, mz);
    if (n == nlev) { if (mgCycle == 3) *GMM = 1; return; }
    size_t nfield = (size_t)(mx + 1) * (size_t)(my + 1) * (size_t)(mz + 1);
    double *r = zalloc(sizeof(double) * nfield);
    mg_residual(c, var, rhs, r, lev[0], lev[1], lev[2], mx, my, mz);
    int m1 = c->mgrid[d][n + 1] + 1;
    int cm[3] = {mx, my, mz};
    cm[d] = m1;
    size_t ncoarse = (size_t)(cm[0] + 1) * (size_t)(cm[1] + 1) * (size_t)(cm[2] + 1);
    double *r1 = zalloc(sizeof(double) * ncoarse), *phi = zalloc(sizeof(double) * ncoarse);
    mg_restrict(c, d, r, r1, n, mx, my, mz, m1);
    int count = (n != nlev - 1) ? *GMM : 1;
    for (int I = 1; I <= count; ++I)
        mg_cycle(c, d, phi, r1, n + 1, nlev, cm[0], cm[1], cm[2], I, GMM, mgCycle);
    c->ibMG = ib_view(c, d, n + 1);
    int fm[3] = {mx, my, mz};
    fm[d] = m1;
    mg_prolong(c, d, r, phi, n, fm[0], fm[1], fm[2], m1, (d == 0) ? mx : (d == 1 ? my : mz));
    c->ibMG = ib_view(c, d, n);
    int sx = mx + 1, sy = my + 1;
    for (int k = 1; k <= mz - 1; ++k)
        for (int j = 1; j <= my - 1; ++j)
            for (int i = 1; i <= mx - 1; ++i) {
                size_t q = VI(sx, sy, i, j, k);
                var[q] = var[q] + r[q] * (1.0 - (double)IBV(c->ibMG, i, j, k));
            }
    mg_prepare_bc(c, n);
    if (n != 1) mg_prepare(c, mx - 1, my - 1, mz - 1);
    if (n == 1 && gcm) gcm_pressure(c, var, rhs);
    int post;
    if (d == 0) post = (n == 1) ? 0 : 1;
    else if (d == 1) post = (n == 1) ? ((c->p.ndim == DIM_2D) ? c->p.iterFinest : 0) : 1;
    else post = (n == 1) ? c->p.iterFinest : 1;
    for (int it = 0; it < post; ++it) mg_itsolv(c, var, rhs, lev[0], lev[1], lev[2], mx, my, mz);
    if (d != 0 && n == 1 && gcm) gcm_pressure(c, var, rhs);
    if (n == 1 && mgCycle == 3) *GMM = 2;
    free(r); free(r1); free(phi);
}

/* IBM/CORE_MG.F90:281-334 MG_Solver on full (0:nx+1)^3 arrays; :391-527 MG_Solv_x/y/z. */
int or_mg_solver(or_ctx *c, double *var, const double *rr)
{
    int nx = c->nx, ny = c->ny, nz = c->nz;
    size_t n1 = (size_t)(nx + 1) * (size_t)(ny + 1) * (size_t)(nz + 1);
    double *rr1 = zalloc(sizeof(double) * n1), *var1 = zalloc(sizeof(double) * n1);
    for (int k = 0; k <= nz; ++k) for (int j = 0; j <= ny; ++j) for (int i = 0; i <= nx; ++i) {
        rr1[VI(nx + 1, ny + 1, i, j, k)] = rr[FI(c, i, j, k)];
        var1[VI(nx + 1, ny + 1, i, j, k)] = var[FI(c, i, j, k)];
    }
    int nd = (c->p.ndim == DIM_3D) ? 3 : 2;
    double *save = c->pPrime_mod;
    c->pPrime_mod = var;
    for (int d = 0; d < nd; ++d) {
        mg_prepare_iblank(c, d);
        int cycle_sel = (d == 2) ? c->p.mgcycle[0] : c->p.mgcycle[d];   /* MG_Solv_z tests mgCycleX, :515 */
        int GMM = (cycle_sel == 1) ? 1 : 2;
        mg_cycle(c, d, var1, rr1, 1, c->nlev[d], nx, ny, nz, 1, &GMM, c->p.mgcycle[d]);
        for (int k = 0; k <= nz; ++k) for (int j = 0; j <= ny; ++j) for (int i = 0; i <= nx; ++i)
            var[FI(c, i, j, k)] = var1[VI(nx + 1, ny + 1, i, j, k)];
    }
    c->pPrime_mod = save;
    free(rr1); free(var1);
    return 0;
}

/* -------------------------------------------------- solve_poisson ------ */
/* IBM/CORE_POISSON.F90:1111-1222 calc_residual: max-norm over fluid cells, first location of the max. */
double or_calc_residual(or_ctx *c, const double *var, const double *r, int *loc)
{
    double resm = 0.0;
    int l0 = 0, l1 = 0, l2 = 0;
    double d2 = (double)(c->p.ndim - DIM_2D);
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                size_t f = FI(c, i, j, k);
                double bmx = c->dxcinv[0][i] * c->dxinv[0][i] * (double)(1 - c->fl[0][f]);
                double bpx = c->dxcinv[0][i + 1] * c->dxinv[0][i] * (double)(1 - c->fl[1][f]);
                double bcx = -(bmx + bpx);
                double bmy = c->dxcinv[1][j] * c->dxinv[1][j] * (double)(1 - c->fl[2][f]);
                double bpy = c->dxcinv[1][j + 1] * c->dxinv[1][j] * (double)(1 - c->fl[3][f]);
                double bcy = -(bmy + bpy);
                double bmz = c->dxcinv[2][k] * c->dxinv[2][k] * (double)(1 - c->fl[4][f]) * d2;
                double bpz = c->dxcinv[2][k + 1] * c->dxinv[2][k] * (double)(1 - c->fl[5][f]) * d2;
                double bcz = -(bmz + bpz);
                double b = (double)(1 - c->iblank[f]);
                bmx *= b; bpx *= b; bmy *= b; bpy *= b; bmz *= b; bpz *= b;
                double bc = (bcx + bcy + bcz) * b + (double)c->iblank[f];
                double res = r[f] - var[f] * bc - var[FI(c, i - 1, j, k)] * bmx - var[FI(c, i + 1, j, k)] * bpx -
                             var[FI(c, i, j - 1, k)] * bmy - var[FI(c, i, j + 1, k)] * bpy -
                             var[FI(c, i, j, k - 1)] * bmz - var[FI(c, i, j, k + 1)] * bpz + c->nlw0[f];
                res = res * b;
                if (fabs(res) > resm) { resm = fabs(res); l0 = i; l1 = j; l2 = k; }
            }
    if (loc) { loc[0] = l0; loc[1] = l1; loc[2] = l2; }
    return resm;
}

/* IBM/CORE_POISSON.F90:419-490 subtracting_average_pressure (fresh_cell = 0). */
void or_subtract_average(or_ctx *c, double *p)
{
    double pTotal = 0.0, volTotal = 0.0;
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                size_t f = FI(c, i, j, k);
                double w = (double)(1 - c->iblank[f]);
                pTotal = pTotal + p[f] * c->dx[0][i] * c->dx[1][j] * c->dx[2][k] * w;
                volTotal = volTotal + c->dx[0][i] * c->dx[1][j] * c->dx[2][k] * w;
            }
    double pAverage = pTotal / volTotal;
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                size_t f = FI(c, i, j, k);
                if (c->iblank[f] == 1) p[f] = 0.0;
                else p[f] = p[f] - pAverage;
            }
    /* fresh cells: mean of the non-blanked, non-fresh 3x3(x3) neighbours
       (IBM/CORE_POISSON.F90:459-488); a fresh cell without such a neighbour
       divides 0 by 0, as the reference does */
    if (!c->fresh) return;
    for (int k = 1; k <= c->nz - 1; ++k)
        for (int j = 1; j <= c->ny - 1; ++j)
            for (int i = 1; i <= c->nx - 1; ++i) {
                if (c->fresh[FI(c, i, j, k)] != 1) continue;
                int i1 = 0;
                double p1 = 0.0;
                const int k1 = (c->p.ndim == DIM_3D) ? k - 1 : k, k2 = (c->p.ndim == DIM_3D) ? k + 1 : k;
                for (int kk = k1; kk <= k2; ++kk)
                    for (int jj = j - 1; jj <= j + 1; ++jj)
                        for (int ii = i - 1; ii <= i + 1; ++ii) {
                            size_t g = FI(c, ii, jj, kk);
                            if (c->iblank[g] != 1 && c->fresh[g] != 1) { i1 = i1 + 1; p1 = p1 + p[g]; }
                        }
                p[FI(c, i, j, k)] = p1 / (double)i1;
            }
}

void or_set_fresh(or_ctx *c, const int8_t *fresh)
{
    const size_t n = (size_t)(c->nx + 2) * (c->ny + 2) * (c->nz + 2);
    free(c->fresh);
    c->fresh = NULL;
    if (!fresh) return;
    c->fresh = (int8_t *)malloc(n);
    memcpy(c->fresh, fresh, n);
}

/* IBM/CORE_SET_BC.F90:635-699 set_pressure_dirichlet_bc */
static void set_pressure_dirichlet_bc(or_ctx *c)
{
    const int *pbc = c->p.pbc;
    for (int k = 0; k <= c->nz; ++k) for (int j = 0; j <= c->ny; ++j) {
        if (pbc[0] == PBC_DIRICHLET) c->fl[0][FI(c, 1, j, k)] = -1;
        if (pbc[1] == PBC_DIRICHLET) c->fl[1][FI(c, c->nxc, j, k)] = -1;
    }
    for (int k = 0; k <= c->nz; ++k) for (int i = 0; i <= c->nx; ++i) {
        if (pbc[2] == PBC_DIRICHLET) c->fl[2][FI(c, i, 1, k)] = -1;
        if (pbc[3] == PBC_DIRICHLET) c->fl[3][FI(c, i, c->nyc, k)] = -1;
    }
    for (int j = 0; j <= c->ny; ++j) for (int i = 0; i <= c->nx; ++i) {
        if (pbc[4] == PBC_DIRICHLET) c->fl[4][FI(c, i, j, 1)] = -1;
        if (pbc[5] == PBC_DIRICHLET) c->fl[5][FI(c, i, j, c->nzc)] = -1;
    }
}

/* IBM/CORE_POISSON.F90:901-1107 itsolv: plain line-SOR on the fine grid (pp_solver_type = 1). */
static void lsor_itsolv(or_ctx *c, double *var, const double *r)
{
    int nmax = c->nx + 2;
    if (c->ny + 2 > nmax) nmax = c->ny + 2;
    if (c->nz + 2 > nmax) nmax = c->nz + 2;
    double *am = zalloc(sizeof(double) * (size_t)nmax), *ac = zalloc(sizeof(double) * (size_t)nmax);
    double *ap = zalloc(sizeof(double) * (size_t)nmax), *rhs = zalloc(sizeof(double) * (size_t)nmax);
    double *sol = zalloc(sizeof(double) * (size_t)nmax);
    double *gam = zalloc(sizeof(double) * (size_t)nmax);
    double d2 = (double)(c->p.ndim - DIM_2D), om = c->p.omega;
    const int *pbc = c->p.pbc;
    const double *ppp = c->p.ppp;
#define V(i, j, k) var[FI(c, i, j, k)]
#define COEF(i, j, k)                                                                                   \
    size_t f = FI(c, i, j, k);                                                                          \
    double amx = c->dxcinv[0][i] * c->dxinv[0][i] * (double)(1 - c->fl[0][f]);                          \
    double apx = c->dxcinv[0][i + 1] * c->dxinv[0][i] * (double)(1 - c->fl[1][f]);                      \
    double acx = -(amx + apx);                                                                          \
    double amy = c->dxcinv[1][j] * c->dxinv[1][j] * (double)(1 - c->fl[2][f]);                          \
    double apy = c->dxcinv[1][j + 1] * c->dxinv[1][j] * (double)(1 - c->fl[3][f]);                      \
    double acy = -(amy + apy);                                                                          \
    double amz = c->dxcinv[2][k] * c->dxinv[2][k] * (double)(1 - c->fl[4][f]) * d2;                     \
    double apz = c->dxcinv[2][k + 1] * c->dxinv[2][k] * (double)(1 - c->fl[5][f]) * d2;                 \
    double acz = -(amz + apz);                                                                          \
    double bw = (double)(1 - c->iblank[f]), bb = (double)c->iblank[f];
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j) {
            for (int i = 1; i <= c->nxc; ++i) {
                COEF(i, j, k)
                double rr = r[f] - V(i, j - 1, k) * amy - V(i, j + 1, k) * apy - V(i, j, k - 1) * amz -
                            V(i, j, k + 1) * apz + c->nlw0[f];
                am[i] = amx * bw; ap[i] = apx * bw;
                ac[i] = (acx + acy + acz) * bw + bb;
                rhs[i] = rr * bw + (double)c->ghost[f] * V(i, j, k);
            }
            if (pbc[0] == PBC_DIRICHLET && pbc[1] == PBC_DIRICHLET) {
                rhs[1] = rhs[1] - ppp[0] * am[1];
                rhs[c->nxc] = rhs[c->nxc] - ppp[1] * ap[c->nxc];
            }
            tdma_w(am, ac, ap, rhs, sol, gam, 1, c->nxc);
            for (int i = 1; i <= c->nxc; ++i) V(i, j, k) = V(i, j, k) + om * (sol[i] - V(i, j, k));
            if (pbc[0] == PBC_DIRICHLET && pbc[1] == PBC_DIRICHLET) { V(0, j, k) = ppp[0]; V(c->nx, j, k) = ppp[1]; }
        }
    for (int k = 1; k <= c->nzc; ++k)
        for (int i = 1; i <= c->nxc; ++i) {
            for (int j = 1; j <= c->nyc; ++j) {
                COEF(i, j, k)
                double rr = r[f] - V(i - 1, j, k) * amx - V(i + 1, j, k) * apx - V(i, j, k - 1) * amz -
                            V(i, j, k + 1) * apz + c->nlw0[f];
                am[j] = amy * bw; ap[j] = apy * bw;
                ac[j] = (acx + acy + acz) * bw + bb;
                rhs[j] = rr * bw + (double)c->ghost[f] * V(i, j, k);
            }
            if (pbc[2] == PBC_DIRICHLET && pbc[3] == PBC_DIRICHLET) {
                rhs[1] = rhs[1] - ppp[2] * am[1];
                rhs[c->nyc] = rhs[c->nyc] - ppp[3] * ap[c->nyc];
            }
            tdma_w(am, ac, ap, rhs, sol, gam, 1, c->nyc);
            for (int j = 1; j <= c->nyc; ++j) V(i, j, k) = V(i, j, k) + om * (sol[j] - V(i, j, k));
        }
    if (c->p.ndim == DIM_3D)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                for (int k = 1; k <= c->nzc; ++k) {
                    COEF(i, j, k)
                    double rr = r[f] - V(i, j - 1, k) * amy - V(i, j + 1, k) * apy - V(i - 1, j, k) * amx -
                                V(i + 1, j, k) * apx + c->nlw0[f];
                    am[k] = amz * bw; ap[k] = apz * bw;
                    ac[k] = (acx + acy + acz) * bw + bb;
                    rhs[k] = rr * bw + (double)c->ghost[f] * V(i, j, k);
                }
                if (pbc[4] == PBC_DIRICHLET && pbc[5] == PBC_DIRICHLET) {
                    rhs[1] = rhs[1] - ppp[4] * am[1];
                    rhs[c->nzc] = rhs[c->nzc] - ppp[5] * ap[c->nzc];
                }
                tdma_w(am, ac, ap, rhs, sol, gam, 1, c->nzc);
                for (int k = 1; k <= c->nzc; ++k) V(i, j, k) = V(i, j, k) + om * (sol[k] - V(i, j, k));
            }
#undef V
#undef COEF
    free(am); free(ac); free(ap); free(rhs); free(sol); free(gam);
}

/* IBM/CORE_POISSON.F90:493-676 solve_poisson (LSOR and MG branches).
 * Returns 0 converged, 1 iterMax reached, 2 ghost rows did not converge, <0 error. */
int or_solve(or_ctx *c, double *pPrime, const double *nlu0, double *nlw0_out,
             int *iters, double *maxres_out, int *loc, double *res_hist)
{
    if (!c->geometry_set) return -2;
    const int *pbc = c->p.pbc;
    size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    memset(c->nlw0, 0, nf * sizeof(double));   /* rhs_poisson zeroes nlw0, IBM/CORE_POISSON.F90:147 */
    memset(c->nlw, 0, nf * sizeof(double));    /* standalone solve, IBM/MAIN.F90:2266 */
    c->ghost_nonconv = 0;
    if (pbc[0] == PBC_DIRICHLET || pbc[2] == PBC_DIRICHLET || pbc[4] == PBC_DIRICHLET)
        set_pressure_dirichlet_bc(c);
    else
        or_subtract_average(c, pPrime);
    int iter = 0, l[3] = {0, 0, 0};
    double maxres = 1.0e10;
    int gcm = (c->p.boundary_formulation == GCM_METHOD);
    while (iter < c->p.iterMax_Poisson && maxres > c->p.restol_Poisson) {
        if (c->p.pp_solver_type == 1) {
            lsor_itsolv(c, pPrime, nlu0);
        } else {
            or_mg_solver(c, pPrime, nlu0);
        }
        if (gcm) or_gcm_correct_pressure(c, pPrime);
        maxres = or_calc_residual(c, pPrime, nlu0, l);
        if (res_hist) res_hist[iter] = maxres;
        iter = iter + 1;
        if (!(maxres == maxres)) break;
    }
    if (iters) *iters = iter;
    if (maxres_out) *maxres_out = maxres;
    if (loc) { loc[0] = l[0]; loc[1] = l[1]; loc[2] = l[2]; }
    if (nlw0_out) memcpy(nlw0_out, c->nlw0, nf * sizeof(double));
    if (!(maxres == maxres)) return -5;
    if (iter == c->p.iterMax_Poisson && maxres > c->p.restol_Poisson) return 1;
    if (c->ghost_nonconv) return 2;
    return 0;
}

/* ------------------------------------------ level-wise kernels (tests) -- */
int or_level_count(or_ctx *c, int d) { return c->nlev[d]; }
int or_level_size(or_ctx *c, int d, int n) { return c->mgrid[d][n]; }

void or_level_metrics(or_ctx *c, int d, int n, double *xnode, double *xc, double *dx,
                      double *dxinv, double *dxc, double *dxcinv)
{
    int N = c->n[d];
    for (int i = 0; i <= N + 1; ++i) {
        if (xnode) xnode[i] = MG1(c, d, x_MG, i, n);
        if (xc) xc[i] = MG1(c, d, xc_MG, i, n);
        if (dx) dx[i] = MG1(c, d, dx_MG, i, n);
        if (dxinv) dxinv[i] = MG1(c, d, dxinv_MG, i, n);
        if (dxc) dxc[i] = MG1(c, d, dxc_MG, i, n);
        if (dxcinv) dxcinv[i] = MG1(c, d, dxcinv_MG, i, n);
    }
}

void or_coarse_iblank(or_ctx *c, int d, int n, int8_t *out)
{
    mg_prepare_iblank(c, d);
    size_t e[3] = {(size_t)c->nx + 1, (size_t)c->ny + 1, (size_t)c->nz + 1};
    e[d] = (size_t)c->mgrid[d][n] + 2;
    memcpy(out, c->cib[d][n], e[0] * e[1] * e[2]);
}

/* Level state as seen by the smoother at level n of the d-cycle: iblank view,
 * MG flags (recomputed from the coarse iblank), ghost marks. */
static void level_state(or_ctx *c, int d, int n, int *m)
{
    mg_prepare_iblank(c, d);
    m[0] = c->nx; m[1] = c->ny; m[2] = c->nz;
    if (n > 1) m[d] = c->mgrid[d][n] + 1;
    double *save = c->pPrime_mod;
    c->pPrime_mod = NULL;
    c->ibMG = ib_view(c, d, n);
    mg_prepare_bc(c, n);
    if (n != 1) mg_prepare(c, m[0] - 1, m[1] - 1, m[2] - 1);
    c->pPrime_mod = save;
}

void or_level_flags(or_ctx *c, int d, int n, int8_t *out6)
{
    int m[3];
    level_state(c, d, n, m);
    size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    for (int s = 0; s < 6; ++s) memcpy(out6 + (size_t)s * nf, c->flMG[s], nf);
}

void or_itsolv_level(or_ctx *c, int d, int n, double *var, const double *r)
{
    int m[3], lev[3] = {1, 1, 1};
    lev[d] = n;
    level_state(c, d, n, m);
    mg_itsolv(c, var, r, lev[0], lev[1], lev[2], m[0], m[1], m[2]);
}

void or_residual_level(or_ctx *c, int d, int n, const double *var, const double *r, double *res)
{
    int m[3], lev[3] = {1, 1, 1};
    lev[d] = n;
    level_state(c, d, n, m);
    mg_residual(c, var, r, res, lev[0], lev[1], lev[2], m[0], m[1], m[2]);
}

void or_restrict_level(or_ctx *c, int d, int n, const double *res, double *r1)
{
    int m[3];
    level_state(c, d, n, m);
    mg_restrict(c, d, res, r1, n, m[0], m[1], m[2], c->mgrid[d][n + 1] + 1);
}

void or_prolong_level(or_ctx *c, int d, int n, const double *phi, double *corr)
{
    int m[3];
    level_state(c, d, n, m);
    int m1 = c->mgrid[d][n + 1] + 1;
    int fm[3] = {m[0], m[1], m[2]};
    fm[d] = m1;
    c->ibMG = ib_view(c, d, n + 1);
    mg_prolong(c, d, corr, phi, n, fm[0], fm[1], fm[2], m1, m[d]);
}

/* ------------------------------------- fractional-step routines either side of the solve ---- */
/* Interpolation weight fx(i) = (x(i) - xc(i-1)) / (xc(i) - xc(i-1)), IBM/CORE_GRID.F90:163-175. */
static double fxw(or_ctx *c, int d, int i)
{
    return (c->x[d][i] - c->xc[d][i - 1]) / (c->xc[d][i] - c->xc[d][i - 1]);
}

/* Face pressure correction of one direction: face1/face2 from the old faces,
 * copy-back, then the um/up masks, each in the reference's loop order
 * (IBM/CORE_FRAC_STEP_ROUTINES.F90:381-441; the same loops close the VAN_KAN
 * branch of face_vel, :111-177).  d = 0 x, 1 y, 2 z. */
static void face_correct(or_ctx *c, int d, double dt, const double *p, double *face, const double *bc)
{
    const int nc[3] = {c->nxc, c->nyc, c->nzc};
    const int n = nc[d];
    const int8_t *um = c->fl[2 * d], *up = c->fl[2 * d + 1];
    double *face1 = zalloc(sizeof(double) * (size_t)(n + 2)), *face2 = zalloc(sizeof(double) * (size_t)(n + 2));
    /* outer loops: x (k, j), y (k, i), z (j, i); the inner index runs along d */
    const int o1 = (d == 2) ? c->nyc : c->nzc, o2 = (d == 0) ? c->nyc : c->nxc;
    for (int a = 1; a <= o1; ++a)
        for (int b = 1; b <= o2; ++b) {
#define AT(t) (d == 0 ? FI(c, (t), b, a) : d == 1 ? FI(c, b, (t), a) : FI(c, b, a, (t)))
            for (int t = 1; t <= n; ++t) {
                const double pgm = (p[AT(t)] - p[AT(t - 1)]) * c->dxcinv[d][t];
                const double pgp = (p[AT(t + 1)] - p[AT(t)]) * c->dxcinv[d][t + 1];
                face1[t] = face[AT(t)] - dt * pgm * (1 - um[AT(t)]);
                face2[t] = face[AT(t + 1)] - dt * pgp * (1 - up[AT(t)]);
            }
            for (int t = 1; t <= n; ++t) {
                face[AT(t)] = face1[t];
                face[AT(t + 1)] = face2[t];
            }
            for (int t = 1; t <= n; ++t) {
                const double bv = bc ? bc[AT(t)] : 0.0;
                face[AT(t)] = face[AT(t)] * (1 - um[AT(t)]) + bv * um[AT(t)];
                face[AT(t + 1)] = face[AT(t + 1)] * (1 - up[AT(t)]) + bv * up[AT(t)];
            }
#undef AT
        }
    free(face1);
    free(face2);
}

static void gcm_vel_set_bc_internal(or_ctx *c, double *u, double *v, double *w);

/* GCM_set_face_vel_body (IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:387-423): the
 * faces of dead cells (blanked, not ghost) are zero. */
static void gcm_set_face_vel_body(or_ctx *c, double *face_u, double *face_v, double *face_w)
{
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                if (c->iblank[f] == 1 && c->ghost[f] == 0) {
                    face_u[FI(c, i + 1, j, k)] = 0.0; face_u[f] = 0.0;
                    face_v[FI(c, i, j + 1, k)] = 0.0; face_v[f] = 0.0;
                    face_w[FI(c, i, j, k + 1)] = 0.0; face_w[f] = 0.0;
                }
            }
}

/* face_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:6-240):
 * frac_step_type 0 NO_VAN_KAN (uTilde = u), 1 VAN_KAN (uTilde = u + dt grad p on
 * the interior, zero elsewhere, then the face pressure correction with p),
 * the boundary masks of both branches, and with GCM the ghost-cell faces of
 * VAN_KAN and GCM_set_face_vel_body.  bc arrays may be NULL (zero). */
void or_face_vel(or_ctx *c, int frac_step_type, double dt, const double *u, const double *v, const double *w,
                 const double *p, const double *bcxu, const double *bcyv, const double *bczw,
                 double *face_u, double *face_v, double *face_w)
{
    const size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    double *uT = zalloc(sizeof(double) * nf), *vT = zalloc(sizeof(double) * nf), *wT = zalloc(sizeof(double) * nf);
    const int8_t *ium = c->fl[0], *iup = c->fl[1], *jum = c->fl[2], *jup = c->fl[3], *kum = c->fl[4], *kup = c->fl[5];
#define BCV(a, f) ((a) ? (a)[f] : 0.0)
    if (frac_step_type == 1) {
        for (int k = 1; k <= c->nzc; ++k)
            for (int j = 1; j <= c->nyc; ++j)
                for (int i = 1; i <= c->nxc; ++i) {
                    const size_t f = FI(c, i, j, k);
                    const double pe = (fxw(c, 0, i + 1) * p[FI(c, i + 1, j, k)] + (1.0 - fxw(c, 0, i + 1)) * p[f]) * (1 - iup[f]) + p[f] * iup[f];
                    const double pw = (fxw(c, 0, i) * p[f] + (1.0 - fxw(c, 0, i)) * p[FI(c, i - 1, j, k)]) * (1 - ium[f]) + p[f] * ium[f];
                    const double pn = (fxw(c, 1, j + 1) * p[FI(c, i, j + 1, k)] + (1.0 - fxw(c, 1, j + 1)) * p[f]) * (1 - jup[f]) + p[f] * jup[f];
                    const double ps = (fxw(c, 1, j) * p[f] + (1.0 - fxw(c, 1, j)) * p[FI(c, i, j - 1, k)]) * (1 - jum[f]) + p[f] * jum[f];
                    const double pf = (fxw(c, 2, k + 1) * p[FI(c, i, j, k + 1)] + (1.0 - fxw(c, 2, k + 1)) * p[f]) * (1 - kup[f]) + p[f] * kup[f];
                    const double pb = (fxw(c, 2, k) * p[f] + (1.0 - fxw(c, 2, k)) * p[FI(c, i, j, k - 1)]) * (1 - kum[f]) + p[f] * kum[f];
                    const double pgx = (pe - pw) * c->dxinv[0][i];
                    const double pgy = (pn - ps) * c->dxinv[1][j];
                    const double pgz = (pf - pb) * c->dxinv[2][k];
                    uT[f] = u[f] + dt * pgx * (double)(1 - c->iblank[f]);
                    vT[f] = v[f] + dt * pgy * (double)(1 - c->iblank[f]);
                    wT[f] = w[f] + dt * pgz * (double)(1 - c->iblank[f]);
                }
    } else {
        memcpy(uT, u, sizeof(double) * nf);
        memcpy(vT, v, sizeof(double) * nf);
        memcpy(wT, w, sizeof(double) * nf);
    }
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                face_u[FI(c, i + 1, j, k)] = (fxw(c, 0, i + 1) * uT[FI(c, i + 1, j, k)] + (1.0 - fxw(c, 0, i + 1)) * uT[f]) * (1 - iup[f]) + BCV(bcxu, f) * iup[f];
                face_u[f] = (fxw(c, 0, i) * uT[f] + (1.0 - fxw(c, 0, i)) * uT[FI(c, i - 1, j, k)]) * (1 - ium[f]) + BCV(bcxu, f) * ium[f];
                face_v[FI(c, i, j + 1, k)] = (fxw(c, 1, j + 1) * vT[FI(c, i, j + 1, k)] + (1.0 - fxw(c, 1, j + 1)) * vT[f]) * (1 - jup[f]) + BCV(bcyv, f) * jup[f];
                face_v[f] = (fxw(c, 1, j) * vT[f] + (1.0 - fxw(c, 1, j)) * vT[FI(c, i, j - 1, k)]) * (1 - jum[f]) + BCV(bcyv, f) * jum[f];
                face_w[FI(c, i, j, k + 1)] = (fxw(c, 2, k + 1) * wT[FI(c, i, j, k + 1)] + (1.0 - fxw(c, 2, k + 1)) * wT[f]) * (1 - kup[f]) + BCV(bczw, f) * kup[f];
                face_w[f] = (fxw(c, 2, k) * wT[f] + (1.0 - fxw(c, 2, k)) * wT[FI(c, i, j, k - 1)]) * (1 - kum[f]) + BCV(bczw, f) * kum[f];
            }
    if (frac_step_type == 1) {
        face_correct(c, 0, dt, p, face_u, bcxu);
        face_correct(c, 1, dt, p, face_v, bcyv);
        face_correct(c, 2, dt, p, face_w, bczw);
    }
    /* both branches: the boundary masks once more (IBM/CORE_FRAC_STEP_ROUTINES.F90:178-195) */
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                face_u[f] = face_u[f] * (1 - ium[f]) + BCV(bcxu, f) * ium[f];
                face_u[FI(c, i + 1, j, k)] = face_u[FI(c, i + 1, j, k)] * (1 - iup[f]) + BCV(bcxu, f) * iup[f];
                face_v[f] = face_v[f] * (1 - jum[f]) + BCV(bcyv, f) * jum[f];
                face_v[FI(c, i, j + 1, k)] = face_v[FI(c, i, j + 1, k)] * (1 - jup[f]) + BCV(bcyv, f) * jup[f];
                face_w[f] = face_w[f] * (1 - kum[f]) + BCV(bczw, f) * kum[f];
                face_w[FI(c, i, j, k + 1)] = face_w[FI(c, i, j, k + 1)] * (1 - kup[f]) + BCV(bczw, f) * kup[f];
            }
#undef BCV
    /* VAN_KAN with ghost cells: the faces of a ghost cell interpolate u itself (:197-221) */
    if (frac_step_type == 1 && c->p.boundary_formulation == GCM_METHOD)
        for (int k = 1; k <= c->nzc; ++k)
            for (int j = 1; j <= c->nyc; ++j)
                for (int i = 1; i <= c->nxc; ++i) {
                    const size_t f = FI(c, i, j, k);
                    const double gY = (double)c->ghost[f], gN = 1.0 - gY;
                    face_u[FI(c, i + 1, j, k)] = gN * face_u[FI(c, i + 1, j, k)] + gY * (fxw(c, 0, i + 1) * u[FI(c, i + 1, j, k)] + (1.0 - fxw(c, 0, i + 1)) * u[f]);
                    face_u[f] = gN * face_u[f] + gY * (fxw(c, 0, i) * u[f] + (1.0 - fxw(c, 0, i)) * u[FI(c, i - 1, j, k)]);
                    face_v[FI(c, i, j + 1, k)] = gN * face_v[FI(c, i, j + 1, k)] + gY * (fxw(c, 1, j + 1) * v[FI(c, i, j + 1, k)] + (1.0 - fxw(c, 1, j + 1)) * v[f]);
                    face_v[f] = gN * face_v[f] + gY * (fxw(c, 1, j) * v[f] + (1.0 - fxw(c, 1, j)) * v[FI(c, i, j - 1, k)]);
                    face_w[FI(c, i, j, k + 1)] = gN * face_w[FI(c, i, j, k + 1)] + gY * (fxw(c, 2, k + 1) * w[FI(c, i, j, k + 1)] + (1.0 - fxw(c, 2, k + 1)) * w[f]);
                    face_w[f] = gN * face_w[f] + gY * (fxw(c, 2, k) * w[f] + (1.0 - fxw(c, 2, k)) * w[FI(c, i, j, k - 1)]);
                }
    if (c->p.boundary_formulation == GCM_METHOD) gcm_set_face_vel_body(c, face_u, face_v, face_w);
    free(uT); free(vT); free(wT);
}

/* rhs_poisson without the hybrid cut-cell branch (IBM/CORE_POISSON.F90:123-163,
 * 273-285): nlu0 zeroed, then dtinv * div(face) * (1 - iblank); returns sum. */
double or_rhs_poisson(or_ctx *c, double dt, const double *face_u, const double *face_v, const double *face_w,
                      double *nlu0)
{
    const size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    const double dtinv = 1.0 / dt;
    double sum = 0.0;
    memset(nlu0, 0, sizeof(double) * nf);
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                nlu0[f] = dtinv * ((face_u[FI(c, i + 1, j, k)] - face_u[f]) * c->dxinv[0][i]
                                   + (face_v[FI(c, i, j + 1, k)] - face_v[f]) * c->dxinv[1][j]
                                   + (face_w[FI(c, i, j, k + 1)] - face_w[f]) * c->dxinv[2][k]);
                nlu0[f] = nlu0[f] * (double)(1 - c->iblank[f]);
                sum = sum + nlu0[f] * c->dx[0][i] * c->dx[1][j] * c->dx[2][k];
            }
    return sum;
}

/* correct_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:244-448), non-periodic; with
 * GCM the ghost-cell velocities (once or_set_vel_ghosts registered them) and
 * GCM_set_face_vel_body. */
void or_correct_vel(or_ctx *c, double dt, const double *pPrime, double *u, double *v, double *w,
                    const double *bcxu, const double *bcyv, const double *bczw,
                    double *face_u, double *face_v, double *face_w)
{
    const double *p = pPrime;
    const int8_t *ium = c->fl[0], *iup = c->fl[1], *jum = c->fl[2], *jup = c->fl[3], *kum = c->fl[4], *kup = c->fl[5];
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                const double pe = (fxw(c, 0, i + 1) * p[FI(c, i + 1, j, k)] + (1.0 - fxw(c, 0, i + 1)) * p[f]) * (1 - iup[f]) + p[f] * iup[f];
                const double pw = (fxw(c, 0, i) * p[f] + (1.0 - fxw(c, 0, i)) * p[FI(c, i - 1, j, k)]) * (1 - ium[f]) + p[f] * ium[f];
                const double pn = (fxw(c, 1, j + 1) * p[FI(c, i, j + 1, k)] + (1.0 - fxw(c, 1, j + 1)) * p[f]) * (1 - jup[f]) + p[f] * jup[f];
                const double ps = (fxw(c, 1, j) * p[f] + (1.0 - fxw(c, 1, j)) * p[FI(c, i, j - 1, k)]) * (1 - jum[f]) + p[f] * jum[f];
                const double pf = (fxw(c, 2, k + 1) * p[FI(c, i, j, k + 1)] + (1.0 - fxw(c, 2, k + 1)) * p[f]) * (1 - kup[f]) + p[f] * kup[f];
                const double pb = (fxw(c, 2, k) * p[f] + (1.0 - fxw(c, 2, k)) * p[FI(c, i, j, k - 1)]) * (1 - kum[f]) + p[f] * kum[f];
                const double pgx = (pe - pw) * c->dxinv[0][i];
                const double pgy = (pn - ps) * c->dxinv[1][j];
                const double pgz = (pf - pb) * c->dxinv[2][k];
                u[f] = u[f] - dt * pgx * (double)(1 - c->iblank[f]);
                v[f] = v[f] - dt * pgy * (double)(1 - c->iblank[f]);
                w[f] = w[f] - dt * pgz * (double)(1 - c->iblank[f]);
            }
    /* ghost-cell velocities (:373) */
    if (c->p.boundary_formulation == GCM_METHOD && c->vg_on) gcm_vel_set_bc_internal(c, u, v, w);
    face_correct(c, 0, dt, p, face_u, bcxu);
    face_correct(c, 1, dt, p, face_v, bcyv);
    face_correct(c, 2, dt, p, face_w, bczw);
    if (c->p.boundary_formulation == GCM_METHOD) gcm_set_face_vel_body(c, face_u, face_v, face_w);
}

/* Ghost-cell velocities for or_correct_vel (NULL coeffD turns them off). */
void or_set_vel_ghosts(or_ctx *c, const double *coeffD, const double *uBI, const double *vBI, const double *wBI,
                       double bodyInterceptWeight, double imagePointWeight)
{
    free(c->vg_coeff); free(c->vg_bi);
    c->vg_coeff = c->vg_bi = NULL;
    c->vg_on = coeffD != NULL;
    if (!coeffD) return;
    const size_t n = (size_t)c->nGhost;
    c->vg_coeff = zalloc(sizeof(double) * 8 * n);
    memcpy(c->vg_coeff, coeffD, sizeof(double) * 8 * n);
    if (uBI) {
        c->vg_bi = zalloc(sizeof(double) * 3 * n);
        memcpy(c->vg_bi, uBI, sizeof(double) * n);
        memcpy(c->vg_bi + n, vBI, sizeof(double) * n);
        memcpy(c->vg_bi + 2 * n, wBI, sizeof(double) * n);
    }
    c->vg_bw = bodyInterceptWeight;
    c->vg_iw = imagePointWeight;
}

int or_vel_ghost_iters(or_ctx *c) { return c->vg_last_iters; }

/* GCM_vel_set_bc_internal (IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:126-247):
 * Gauss-Seidel over the ordered ghost list until max |du|+|dv|+|dw| <= restol_ad. */
static void gcm_vel_set_bc_internal(or_ctx *c, double *u, double *v, double *w)
{
    const size_t n0 = (size_t)c->nGhost;
    int iterGC = 0;
    double resVelMax = 1.0e10;
    while (iterGC < c->p.iterMax_ad && resVelMax > c->p.restol_ad) {
        resVelMax = 0.0;
        for (int n = 0; n < c->nGhost; ++n) {
            const int iG = c->gi[0][n], jG = c->gi[1][n], kG = c->gi[2][n];
            const double ub = c->vg_bi ? c->vg_bi[n] : 0.0, vb = c->vg_bi ? c->vg_bi[n0 + n] : 0.0,
                         wb = c->vg_bi ? c->vg_bi[2 * n0 + n] : 0.0;
            double uIP = 0.0, vIP = 0.0, wIP = 0.0;
            for (int r = 0; r < 8; ++r) {
                const int ii = c->gi[3][n] + incI[r], jj = c->gi[4][n] + incJ[r], kk = c->gi[5][n] + incK[r];
                const double cd = c->vg_coeff[8 * (size_t)n + r];
                if (ii != iG || jj != jG || kk != kG) {
                    const size_t f = FI(c, ii, jj, kk);
                    uIP = uIP + cd * u[f]; vIP = vIP + cd * v[f]; wIP = wIP + cd * w[f];
                } else {
                    uIP = uIP + cd * ub; vIP = vIP + cd * vb; wIP = wIP + cd * wb;
                }
            }
            const size_t g = FI(c, iG, jG, kG);
            const double uPrev = u[g], vPrev = v[g], wPrev = w[g];
            u[g] = ub * c->vg_bw - uIP * c->vg_iw;
            v[g] = vb * c->vg_bw - vIP * c->vg_iw;
            w[g] = wb * c->vg_bw - wIP * c->vg_iw;
            const double resVel = fabs(u[g] - uPrev) + fabs(v[g] - vPrev) + fabs(w[g] - wPrev);
            if (resVel > resVelMax) resVelMax = resVel;
        }
        iterGC = iterGC + 1;
    }
    c->vg_last_iters = iterGC;
}

/* update_pressure (IBM/CORE_FRAC_STEP_ROUTINES.F90:949-967). */
void or_update_pressure(or_ctx *c, int frac_step_type, const double *pPrime, double *p)
{
    const size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    for (size_t t = 0; t < nf; ++t) p[t] = (frac_step_type == 1) ? p[t] + pPrime[t] : pPrime[t];
    if (c->p.boundary_formulation == GCM_METHOD) gcm_p_set_bc_internal(c, p, c->nx + 1, c->ny + 1);
}

/* ------------------------------------------------------------------ set_bc -- */
/* One side of set_bc's SELECT CASE (IBM/CORE_SET_BC.F90:56-280): side s
 * (0 x1 .. 5 z2), uvw the cell's u, v, w, (i, j) its first two indices. */
static void set_bc_side(or_ctx *c, int s, const double *vel3, const double *freq3, double time,
                        double tstart_gust, double xout, double yout, const double *const *uvw, int i, int j,
                        double *out)
{
    const double pi = 4.0 * atan(1.0);   /* IBM/MAIN.F90:264 */
    const int a = s / 2;
    switch (c->p.bc[s]) {
    case BC_DIRICHLET:
        for (int q = 0; q < 3; ++q) out[q] = vel3[q];
        break;
    case BC_ZERO_GRADIENT:
        for (int q = 0; q < 3; ++q) out[q] = *uvw[q];
        break;
    case 3:   /* BC_TYPE_PULSATILE_INFLOW */
        for (int q = 0; q < 3; ++q) out[q] = vel3[q] * sin(2.0 * pi * freq3[q] * time);
        if (s == 1) {   /* :96-104, the x2 gust switch */
            if (time > tstart_gust) out[0] = vel3[0] * fabs(sin(2.0 * pi * freq3[0] * time));
            else out[0] = 0;
        }
        break;
    case 4:   /* BC_TYPE_SYMMETRY: normal component zero */
        for (int q = 0; q < 3; ++q) out[q] = (q == a) ? 0.0 : *uvw[q];
        break;
    case 7:   /* BC_TYPE_SHEAR */
        for (int q = 0; q < 3; ++q) out[q] = vel3[q];
        if (a == 1) out[1] = vel3[1] * c->x[0][i] / xout;
        else out[a] = vel3[a] * c->x[1][j] / yout;
        break;
    }
}

/* The zero-gradient corrections of enforce_global_mass_consv
 * (IBM/CORE_SET_BC.F90:352-371) and GCM_enforce_global_mass_consv
 * (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:60-79): the normal component on the
 * whole plane of each zero-gradient side, minus side - corr, plus side + corr. */
static void zg_correct_planes(or_ctx *c, double *const *bc9, double correction_vel)
{
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    double *bcxu = bc9[0], *bcyv = bc9[4], *bczw = bc9[8];
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j) {
            if (c->p.bc[0] == BC_ZERO_GRADIENT) bcxu[FI(c, 1, j, k)] = bcxu[FI(c, 1, j, k)] - correction_vel;
            if (c->p.bc[1] == BC_ZERO_GRADIENT) bcxu[FI(c, c->nxc, j, k)] = bcxu[FI(c, c->nxc, j, k)] + correction_vel;
        }
    for (int k = 0; k <= nz; ++k)
        for (int i = 0; i <= nx; ++i) {
            if (c->p.bc[2] == BC_ZERO_GRADIENT) bcyv[FI(c, i, 1, k)] = bcyv[FI(c, i, 1, k)] - correction_vel;
            if (c->p.bc[3] == BC_ZERO_GRADIENT) bcyv[FI(c, i, c->nyc, k)] = bcyv[FI(c, i, c->nyc, k)] + correction_vel;
        }
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            if (c->p.bc[4] == BC_ZERO_GRADIENT) bczw[FI(c, i, j, 1)] = bczw[FI(c, i, j, 1)] - correction_vel;
            if (c->p.bc[5] == BC_ZERO_GRADIENT) bczw[FI(c, i, j, c->nzc)] = bczw[FI(c, i, j, c->nzc)] + correction_vel;
        }
}

/* set_bc without its internal-boundary calls (IBM/CORE_SET_BC.F90:22-298),
 * enforce_global_mass_consv (:304-377; iMarkm..kMarkp are zero outside SSM,
 * IBM/GCM_MEMORY_ALLOCATE.F90:68-69) and set_outer_ghost_vel
 * (IBM/CORE_SET_OUTER_GHOST.F90:1-63).  val and freq hold 6 x 3 values (side
 * x1..z2, component u, v, w); bc9 = bcxu,bcyu,bczu,bcxv,bcyv,bczv,bcxw,bcyw,bczw.
 * Returns -1 for a side type it does not restate (user-specified), else 0;
 * *correction = correction_vel (0 without zero-gradient sides). */
int or_set_bc(or_ctx *c, const double *val, const double *freq, double time, double tstart_gust, double xout,
              double yout, double *u, double *v, double *w, double *const *bc9, double *correction)
{
    for (int s = 0; s < 6; ++s) {
        const int t = c->p.bc[s];
        if (t != BC_DIRICHLET && t != BC_ZERO_GRADIENT && t != 3 && t != 4 && t != 7) return -1;
    }
    double *vel[3] = {u, v, w};
    double out[3];
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    /* x sides, :50-135 */
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int side = 0; side < 2; ++side) {
                const int i = side == 0 ? 1 : c->nxc;
                const size_t f = FI(c, i, j, k);
                const double *uvw[3] = {u + f, v + f, w + f};
                set_bc_side(c, side, val + 3 * side, freq + 3 * side, time, tstart_gust, xout, yout, uvw, i, j, out);
                for (int q = 0; q < 3; ++q) bc9[3 * q + 0][f] = out[q];
            }
    /* y sides, :137-221 */
    for (int k = 0; k <= nz; ++k)
        for (int i = 0; i <= nx; ++i)
            for (int side = 0; side < 2; ++side) {
                const int j = side == 0 ? 1 : c->nyc, s = 2 + side;
                const size_t f = FI(c, i, j, k);
                const double *uvw[3] = {u + f, v + f, w + f};
                set_bc_side(c, s, val + 3 * s, freq + 3 * s, time, tstart_gust, xout, yout, uvw, i, j, out);
                for (int q = 0; q < 3; ++q) bc9[3 * q + 1][f] = out[q];
            }
    /* z sides, :223-283 */
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i)
            for (int side = 0; side < 2; ++side) {
                const int k = side == 0 ? 1 : c->nzc, s = 4 + side;
                const size_t f = FI(c, i, j, k);
                const double *uvw[3] = {u + f, v + f, w + f};
                set_bc_side(c, s, val + 3 * s, freq + 3 * s, time, tstart_gust, xout, yout, uvw, i, j, out);
                for (int q = 0; q < 3; ++q) bc9[3 * q + 2][f] = out[q];
            }
    /* enforce_global_mass_consv */
    int zg = 0;
    for (int s = 0; s < 6; ++s) zg |= (c->p.bc[s] == BC_ZERO_GRADIENT);
    double correction_vel = 0.0;
    if (zg) {
        const int8_t *ium = c->fl[0], *iup = c->fl[1], *jum = c->fl[2], *jup = c->fl[3], *kum = c->fl[4], *kup = c->fl[5];
        double *bcxu = bc9[0], *bcyv = bc9[4], *bczw = bc9[8];
        double massflux = 0.0;
        for (int k = 1; k <= c->nzc; ++k)
            for (int j = 1; j <= c->nyc; ++j)
                for (int i = 1; i <= c->nxc; ++i) {
                    const size_t f = FI(c, i, j, k);
                    const double dx = c->dx[0][i], dy = c->dx[1][j], dz = c->dx[2][k];
                    massflux = massflux + (-(bcxu[f] * ium[f] * dy * dz) + bcxu[f] * iup[f] * dy * dz
                                           - bcyv[f] * jum[f] * dx * dz + bcyv[f] * jup[f] * dx * dz
                                           - bczw[f] * kum[f] * dx * dy + bczw[f] * kup[f] * dx * dy)
                                              * (double)(1 - c->iblank[f]);
                }
        correction_vel = -massflux / c->p.outflow_area;
        zg_correct_planes(c, bc9, correction_vel);
    }
    if (correction) *correction = correction_vel;
    /* set_outer_ghost_vel */
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int q = 0; q < 3; ++q) {
                double *a = vel[q];
                const double *b = bc9[3 * q + 0];
                a[FI(c, 0, j, k)] = 2.0 * b[FI(c, 1, j, k)] - a[FI(c, 1, j, k)];
                a[FI(c, nx, j, k)] = 2.0 * b[FI(c, nx - 1, j, k)] - a[FI(c, nx - 1, j, k)];
            }
    for (int k = 0; k <= nz; ++k)
        for (int i = 0; i <= nx; ++i)
            for (int q = 0; q < 3; ++q) {
                double *a = vel[q];
                const double *b = bc9[3 * q + 1];
                a[FI(c, i, 0, k)] = 2.0 * b[FI(c, i, 1, k)] - a[FI(c, i, 1, k)];
                a[FI(c, i, ny, k)] = 2.0 * b[FI(c, i, ny - 1, k)] - a[FI(c, i, ny - 1, k)];
            }
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i)
            for (int q = 0; q < 3; ++q) {
                double *a = vel[q];
                const double *b = bc9[3 * q + 2];
                a[FI(c, i, j, 0)] = 2.0 * b[FI(c, i, j, 1)] - a[FI(c, i, j, 1)];
                a[FI(c, i, j, nz)] = 2.0 * b[FI(c, i, j, nz - 1)] - a[FI(c, i, j, nz - 1)];
            }
    return 0;
}

/* ---------------------------------------------- momentum right-hand side ---- */
/* rhs_advec_diff (IBM/CORE_RHS_AD.F90:13-75) with its contained routines
 * rhs_advec (:80-382, the non-hybrid branch), rhs_loadAB (:385-430), rhs_diff
 * (:433-530) and rhs_vankan (:550-585), in the reference's call order.
 * advec_scheme 1 ADAMS_BASHFORTH2, 2/3 CRANK_NICOLSON1/2.  Array arguments are
 * full (0:nx+1,0:ny+1,0:nz+1) fields; bc9 holds bcxu,bcyu,bczu,bcxv,bcyv,bczv,
 * bcxw,bcyw,bczw and bcvisc3 bcxvisc,bcyvisc,bczvisc (NULL entries: zero);
 * exp_weight NULL: 1.5 (no fresh cells). */
static double arr_at(const double *a, size_t f) { return a ? a[f] : 0.0; }

/* Second-neighbour flags of the hybrid scheme (IBM/BOUNDARY_SET.F90:90-127,
 * set_outer_iup): iumm is 1 in the first two cells of an axis, iupp in the
 * last two; the internal-boundary settings of SSM are not used under GCM. */
static int hyb_mm(int i) { return (i == 1 || i == 2) ? 1 : 0; }
static int hyb_pp(int i, int ncell) { return (i == ncell || i == ncell - 1) ? 1 : 0; }

/* rhs_advec (IBM/CORE_RHS_AD.F90:80-382): central advection, blended with
 * second-order upwind face values by alfa when Hybrid (|alfa| > 1e-3,
 * IBM/MAIN.F90:649-652).  The x-direction upwind face value from the plus
 * side weights vel(ipp) with edxWeightp1, as the reference writes it
 * (:203-205); y and z use their p2 weights. */
static void rhs_advec_one(or_ctx *c, const double *vel, double *nlvel, const double *bcx, const double *bcy,
                          const double *bcz, const double *face_u, const double *face_v, const double *face_w)
{
    const int8_t *ium = c->fl[0], *iup = c->fl[1], *jum = c->fl[2], *jup = c->fl[3], *kum = c->fl[4], *kup = c->fl[5];
    const double alfa = c->p.alfa;
    const int hybrid = fabs(alfa) > 1.0e-3;
    const int three_d = (c->p.ndim == DIM_3D);
    const double *dxinv = c->dxinv[0], *dyinv = c->dxinv[1], *dzinv = c->dxinv[2];
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                const double vele = (fxw(c, 0, i + 1) * vel[FI(c, i + 1, j, k)] + (1.0 - fxw(c, 0, i + 1)) * vel[f]) * (1 - iup[f]) + arr_at(bcx, f) * iup[f];
                const double velw = (fxw(c, 0, i) * vel[f] + (1.0 - fxw(c, 0, i)) * vel[FI(c, i - 1, j, k)]) * (1 - ium[f]) + arr_at(bcx, f) * ium[f];
                if (hybrid) {
                    const int imm = (i - 2 > 0) ? i - 2 : 0, ipp = (i + 2 < nx) ? i + 2 : nx;
                    const double USign = copysign(1.0, face_u[f]), USignP = copysign(1.0, face_u[FI(c, i + 1, j, k)]);
                    const double em1 = (dxinv[i - 1] + 2.0 * dxinv[i]) / (dxinv[i - 1] + dxinv[i]);
                    const double em2 = dxinv[i] / (dxinv[i - 1] + dxinv[i]);
                    const double ep1 = (dxinv[ipp] + 2.0 * dxinv[i + 1]) / (dxinv[ipp] + dxinv[i + 1]);
                    const double wm1 = (dxinv[imm] + 2.0 * dxinv[i - 1]) / (dxinv[imm] + dxinv[i - 1]);
                    const double wm2 = dxinv[i - 1] / (dxinv[imm] + dxinv[i - 1]);
                    const double wp1 = (dxinv[i + 1] + 2.0 * dxinv[i]) / (dxinv[i + 1] + dxinv[i]);
                    const double wp2 = dxinv[i] / (dxinv[i + 1] + dxinv[i]);
                    const double mm = hyb_mm(i), pp = hyb_pp(i, c->nxc);
                    const double vele_up = ((1.0 + USignP) * (mm * vele + (1 - mm) * (em1 * vel[f] - em2 * vel[FI(c, i - 1, j, k)]))
                                            + (1.0 - USignP) * (pp * vele + (1 - pp) * (ep1 * vel[FI(c, i + 1, j, k)] - ep1 * vel[FI(c, ipp, j, k)])))
                                           * 0.5 * (1 - iup[f]) + arr_at(bcx, f) * iup[f];
                    const double velw_up = ((1.0 + USign) * (mm * velw + (1 - mm) * (wm1 * vel[FI(c, i - 1, j, k)] - wm2 * vel[FI(c, imm, j, k)]))
                                            + (1.0 - USign) * (pp * velw + (1 - pp) * (wp1 * vel[f] - wp2 * vel[FI(c, i + 1, j, k)])))
                                           * 0.5 * (1 - ium[f]) + arr_at(bcx, f) * ium[f];
                    nlvel[f] = (((1.0 - alfa) * vele + alfa * vele_up) * face_u[FI(c, i + 1, j, k)]
                                - ((1.0 - alfa) * velw + alfa * velw_up) * face_u[f]) * dxinv[i];
                } else {
                    nlvel[f] = (vele * face_u[FI(c, i + 1, j, k)] - velw * face_u[f]) * dxinv[i];
                }
            }
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                const double veln = (fxw(c, 1, j + 1) * vel[FI(c, i, j + 1, k)] + (1.0 - fxw(c, 1, j + 1)) * vel[f]) * (1 - jup[f]) + arr_at(bcy, f) * jup[f];
                const double vels = (fxw(c, 1, j) * vel[f] + (1.0 - fxw(c, 1, j)) * vel[FI(c, i, j - 1, k)]) * (1 - jum[f]) + arr_at(bcy, f) * jum[f];
                if (hybrid) {
                    const int jmm = (j - 2 > 0) ? j - 2 : 0, jpp = (j + 2 < ny) ? j + 2 : ny;
                    const double VSign = copysign(1.0, face_v[f]), VSignP = copysign(1.0, face_v[FI(c, i, j + 1, k)]);
                    const double nm1 = (dyinv[j - 1] + 2.0 * dyinv[j]) / (dyinv[j - 1] + dyinv[j]);
                    const double nm2 = dyinv[j] / (dyinv[j - 1] + dyinv[j]);
                    const double np1 = (dyinv[jpp] + 2.0 * dyinv[j + 1]) / (dyinv[jpp] + dyinv[j + 1]);
                    const double np2 = dyinv[j + 1] / (dyinv[jpp] + dyinv[j + 1]);
                    const double sm1 = (dyinv[jmm] + 2.0 * dyinv[j - 1]) / (dyinv[jmm] + dyinv[j - 1]);
                    const double sm2 = dyinv[j - 1] / (dyinv[jmm] + dyinv[j - 1]);
                    const double sp1 = (dyinv[j + 1] + 2.0 * dyinv[j]) / (dyinv[j + 1] + dyinv[j]);
                    const double sp2 = dyinv[j] / (dyinv[j + 1] + dyinv[j]);
                    const double mm = hyb_mm(j), pp = hyb_pp(j, c->nyc);
                    const double veln_up = ((1.0 + VSignP) * (mm * veln + (1 - mm) * (nm1 * vel[f] - nm2 * vel[FI(c, i, j - 1, k)]))
                                            + (1.0 - VSignP) * (pp * veln + (1 - pp) * (np1 * vel[FI(c, i, j + 1, k)] - np2 * vel[FI(c, i, jpp, k)])))
                                           * 0.5 * (1 - jup[f]) + arr_at(bcy, f) * jup[f];
                    const double vels_up = ((1.0 + VSign) * (mm * vels + (1 - mm) * (sm1 * vel[FI(c, i, j - 1, k)] - sm2 * vel[FI(c, i, jmm, k)]))
                                            + (1.0 - VSign) * (pp * vels + (1 - pp) * (sp1 * vel[f] - sp2 * vel[FI(c, i, j + 1, k)])))
                                           * 0.5 * (1 - jum[f]) + arr_at(bcy, f) * jum[f];
                    nlvel[f] = nlvel[f] + (((1.0 - alfa) * veln + alfa * veln_up) * face_v[FI(c, i, j + 1, k)]
                                           - ((1.0 - alfa) * vels + alfa * vels_up) * face_v[f]) * dyinv[j];
                } else {
                    nlvel[f] = nlvel[f] + (veln * face_v[FI(c, i, j + 1, k)] - vels * face_v[f]) * dyinv[j];
                }
            }
    if (three_d)
        for (int k = 1; k <= c->nzc; ++k)
            for (int j = 1; j <= c->nyc; ++j)
                for (int i = 1; i <= c->nxc; ++i) {
                    const size_t f = FI(c, i, j, k);
                    const double velf = (fxw(c, 2, k + 1) * vel[FI(c, i, j, k + 1)] + (1.0 - fxw(c, 2, k + 1)) * vel[f]) * (1 - kup[f]) + arr_at(bcz, f) * kup[f];
                    const double velb = (fxw(c, 2, k) * vel[f] + (1.0 - fxw(c, 2, k)) * vel[FI(c, i, j, k - 1)]) * (1 - kum[f]) + arr_at(bcz, f) * kum[f];
                    if (hybrid) {
                        const int kmm = (k - 2 > 0) ? k - 2 : 0, kpp = (k + 2 < nz) ? k + 2 : nz;
                        const double WSign = copysign(1.0, face_w[f]), WSignP = copysign(1.0, face_w[FI(c, i, j, k + 1)]);
                        const double fm1 = (dzinv[k - 1] + 2.0 * dzinv[k]) / (dzinv[k - 1] + dzinv[k]);
                        const double fm2 = dzinv[k] / (dzinv[k - 1] + dzinv[k]);
                        const double fp1 = (dzinv[kpp] + 2.0 * dzinv[k + 1]) / (dzinv[kpp] + dzinv[k + 1]);
                        const double fp2 = dzinv[k + 1] / (dzinv[kpp] + dzinv[k + 1]);
                        const double bm1 = (dzinv[kmm] + 2.0 * dzinv[k - 1]) / (dzinv[kmm] + dzinv[k - 1]);
                        const double bm2 = dzinv[k - 1] / (dzinv[kmm] + dzinv[k - 1]);
                        const double bp1 = (dzinv[k + 1] + 2.0 * dzinv[k]) / (dzinv[k + 1] + dzinv[k]);
                        const double bp2 = dzinv[k] / (dzinv[k + 1] + dzinv[k]);
                        const double mm = hyb_mm(k), pp = hyb_pp(k, c->nzc);
                        const double velf_up = ((1.0 + WSignP) * (mm * velf + (1 - mm) * (fm1 * vel[f] - fm2 * vel[FI(c, i, j, k - 1)]))
                                                + (1.0 - WSignP) * (pp * velf + (1 - pp) * (fp1 * vel[FI(c, i, j, k + 1)] - fp2 * vel[FI(c, i, j, kpp)])))
                                               * 0.5 * (1 - kup[f]) + arr_at(bcz, f) * kup[f];
                        const double velb_up = ((1.0 + WSign) * (mm * velb + (1 - mm) * (bm1 * vel[FI(c, i, j, k - 1)] - bm2 * vel[FI(c, i, j, kmm)]))
                                                + (1.0 - WSign) * (pp * velb + (1 - pp) * (bp1 * vel[f] - bp2 * vel[FI(c, i, j, k + 1)])))
                                               * 0.5 * (1 - kum[f]) + arr_at(bcz, f) * kum[f];
                        nlvel[f] = nlvel[f] + (((1.0 - alfa) * velf + alfa * velf_up) * face_w[FI(c, i, j, k + 1)]
                                               - ((1.0 - alfa) * velb + alfa * velb_up) * face_w[f]) * dzinv[k];
                    } else {
                        nlvel[f] = nlvel[f] + (velf * face_w[FI(c, i, j, k + 1)] - velb * face_w[f]) * dzinv[k];
                    }
                }
}

static void rhs_load_ab(or_ctx *c, int advec_scheme, const double *exp_weight, double *nlvel, double *nlvelOld)
{
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                if (advec_scheme == 1) {
                    const double ew = exp_weight ? exp_weight[f] : 1.5;
                    const double tempvel = ew * nlvel[f] - (ew - 1.0) * nlvelOld[f];
                    nlvelOld[f] = nlvel[f];
                    nlvel[f] = tempvel;
                } else {
                    nlvel[f] = nlvel[f] * 0.5;
                }
            }
}

static void rhs_diff_one(or_ctx *c, double dt, const double *vel, double *nlvel, const double *bcx, const double *bcy,
                         const double *bcz, const double *visc, const double *const *bcvisc3)
{
    const int8_t *ium = c->fl[0], *iup = c->fl[1], *jum = c->fl[2], *jup = c->fl[3], *kum = c->fl[4], *kup = c->fl[5];
    const double rnDim = (double)(c->p.ndim - DIM_2D);
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                const double nuE = (fxw(c, 0, i + 1) * visc[FI(c, i + 1, j, k)] + (1.0 - fxw(c, 0, i + 1)) * visc[f]) * (1 - iup[f]) + arr_at(bcvisc3[0], f) * iup[f];
                const double nuW = (fxw(c, 0, i) * visc[f] + (1.0 - fxw(c, 0, i)) * visc[FI(c, i - 1, j, k)]) * (1 - ium[f]) + arr_at(bcvisc3[0], f) * ium[f];
                const double nuN = (fxw(c, 1, j + 1) * visc[FI(c, i, j + 1, k)] + (1.0 - fxw(c, 1, j + 1)) * visc[f]) * (1 - jup[f]) + arr_at(bcvisc3[1], f) * jup[f];
                const double nuS = (fxw(c, 1, j) * visc[f] + (1.0 - fxw(c, 1, j)) * visc[FI(c, i, j - 1, k)]) * (1 - jum[f]) + arr_at(bcvisc3[1], f) * jum[f];
                const double nuF = (fxw(c, 2, k + 1) * visc[FI(c, i, j, k + 1)] + (1.0 - fxw(c, 2, k + 1)) * visc[f]) * (1 - kup[f]) + arr_at(bcvisc3[2], f) * kup[f];
                const double nuB = (fxw(c, 2, k) * visc[f] + (1.0 - fxw(c, 2, k)) * visc[FI(c, i, j, k - 1)]) * (1 - kum[f]) + arr_at(bcvisc3[2], f) * kum[f];
                double amx = (c->dxcinv[0][i] * (1 - ium[f]) + c->dxinv[0][i] * ium[f] * 2.0) * c->dxinv[0][i];
                double apx = (c->dxcinv[0][i + 1] * (1 - iup[f]) + c->dxinv[0][i] * iup[f] * 2.0) * c->dxinv[0][i];
                amx = amx * nuW;
                apx = apx * nuE;
                const double acx = -(amx + apx);
                double amy = (c->dxcinv[1][j] * (1 - jum[f]) + c->dxinv[1][j] * jum[f] * 2.0) * c->dxinv[1][j];
                double apy = (c->dxcinv[1][j + 1] * (1 - jup[f]) + c->dxinv[1][j] * jup[f] * 2.0) * c->dxinv[1][j];
                amy = amy * nuS;
                apy = apy * nuN;
                const double acy = -(amy + apy);
                double amz = (c->dxcinv[2][k] * (1 - kum[f]) + c->dxinv[2][k] * kum[f] * 2.0) * c->dxinv[2][k] * rnDim;
                double apz = (c->dxcinv[2][k + 1] * (1 - kup[f]) + c->dxinv[2][k] * kup[f] * 2.0) * c->dxinv[2][k] * rnDim;
                amz = amz * nuB;
                apz = apz * nuF;
                const double acz = -(amz + apz);
                const double diffvel = amx * (vel[FI(c, i - 1, j, k)] * (1 - ium[f]) + arr_at(bcx, f) * ium[f])
                                     + acx * vel[f]
                                     + apx * (vel[FI(c, i + 1, j, k)] * (1 - iup[f]) + arr_at(bcx, f) * iup[f])
                                     + amy * (vel[FI(c, i, j - 1, k)] * (1 - jum[f]) + arr_at(bcy, f) * jum[f])
                                     + acy * vel[f]
                                     + apy * (vel[FI(c, i, j + 1, k)] * (1 - jup[f]) + arr_at(bcy, f) * jup[f])
                                     + amz * (vel[FI(c, i, j, k - 1)] * (1 - kum[f]) + arr_at(bcz, f) * kum[f])
                                     + acz * vel[f]
                                     + apz * (vel[FI(c, i, j, k + 1)] * (1 - kup[f]) + arr_at(bcz, f) * kup[f]);
                nlvel[f] = vel[f] - dt * nlvel[f] + 0.5 * dt * diffvel;
            }
}

void or_rhs_advec_diff(or_ctx *c, int advec_scheme, int frac_step_type, double dt, const double *u,
                       const double *v, const double *w, const double *face_u, const double *face_v,
                       const double *face_w, const double *const *bc9, const double *visc,
                       const double *const *bcvisc3, const double *exp_weight, double *nluOld, double *nlvOld,
                       double *nlwOld, const double *p, double *nlu, double *nlv, double *nlw)
{
    const int three_d = (c->p.ndim == DIM_3D);
    rhs_advec_one(c, u, nlu, bc9[0], bc9[1], bc9[2], face_u, face_v, face_w);
    rhs_advec_one(c, v, nlv, bc9[3], bc9[4], bc9[5], face_u, face_v, face_w);
    if (three_d) rhs_advec_one(c, w, nlw, bc9[6], bc9[7], bc9[8], face_u, face_v, face_w);
    rhs_load_ab(c, advec_scheme, exp_weight, nlu, nluOld);
    rhs_load_ab(c, advec_scheme, exp_weight, nlv, nlvOld);
    if (three_d) rhs_load_ab(c, advec_scheme, exp_weight, nlw, nlwOld);
    rhs_diff_one(c, dt, u, nlu, bc9[0], bc9[1], bc9[2], visc, bcvisc3);
    rhs_diff_one(c, dt, v, nlv, bc9[3], bc9[4], bc9[5], visc, bcvisc3);
    if (three_d) rhs_diff_one(c, dt, w, nlw, bc9[6], bc9[7], bc9[8], visc, bcvisc3);
    if (frac_step_type == 1) {   /* rhs_vankan */
        const int8_t *ium = c->fl[0], *iup = c->fl[1], *jum = c->fl[2], *jup = c->fl[3], *kum = c->fl[4], *kup = c->fl[5];
        for (int k = 1; k <= c->nzc; ++k)
            for (int j = 1; j <= c->nyc; ++j)
                for (int i = 1; i <= c->nxc; ++i) {
                    const size_t f = FI(c, i, j, k);
                    const double pe = (fxw(c, 0, i + 1) * p[FI(c, i + 1, j, k)] + (1.0 - fxw(c, 0, i + 1)) * p[f]) * (1 - iup[f]) + p[f] * iup[f];
                    const double pw = (fxw(c, 0, i) * p[f] + (1.0 - fxw(c, 0, i)) * p[FI(c, i - 1, j, k)]) * (1 - ium[f]) + p[f] * ium[f];
                    const double pn = (fxw(c, 1, j + 1) * p[FI(c, i, j + 1, k)] + (1.0 - fxw(c, 1, j + 1)) * p[f]) * (1 - jup[f]) + p[f] * jup[f];
                    const double ps = (fxw(c, 1, j) * p[f] + (1.0 - fxw(c, 1, j)) * p[FI(c, i, j - 1, k)]) * (1 - jum[f]) + p[f] * jum[f];
                    const double pf = (fxw(c, 2, k + 1) * p[FI(c, i, j, k + 1)] + (1.0 - fxw(c, 2, k + 1)) * p[f]) * (1 - kup[f]) + p[f] * kup[f];
                    const double pb = (fxw(c, 2, k) * p[f] + (1.0 - fxw(c, 2, k)) * p[FI(c, i, j, k - 1)]) * (1 - kum[f]) + p[f] * kum[f];
                    nlu[f] = nlu[f] - dt * ((pe - pw) * c->dxinv[0][i]) * (double)(1 - c->iblank[f]);
                    nlv[f] = nlv[f] - dt * ((pn - ps) * c->dxinv[1][j]) * (double)(1 - c->iblank[f]);
                    nlw[f] = nlw[f] - dt * ((pf - pb) * c->dxinv[2][k]) * (double)(1 - c->iblank[f]);
                }
    }
}

/* ------------------------------------------- implicit momentum solve ---- */
/* set_solve_ad (IBM/CORE_SET_SOLVERS.F90:20-95, stationary boundary): the
 * implicit diffusion coefficients amx_ad..apz_ad (0:nx+1)^3, kept in the
 * context for or_rhs_adjust_bc / or_solve_ad. */
void or_set_solve_ad(or_ctx *c, double dt, const double *visc, const double *const *bcvisc3)
{
    const size_t nf = (size_t)(c->nx + 2) * (size_t)(c->ny + 2) * (size_t)(c->nz + 2);
    for (int q = 0; q < 6; ++q) {
        if (!c->ad[q]) c->ad[q] = zalloc(sizeof(double) * nf);
        memset(c->ad[q], 0, sizeof(double) * nf);
    }
    const int8_t *ium = c->fl[0], *iup = c->fl[1], *jum = c->fl[2], *jup = c->fl[3], *kum = c->fl[4], *kup = c->fl[5];
    const double rnDim = (double)(c->p.ndim - DIM_2D);
    for (int k = 1; k <= c->nz - 1; ++k)
        for (int j = 1; j <= c->ny - 1; ++j)
            for (int i = 1; i <= c->nx - 1; ++i) {
                const size_t f = FI(c, i, j, k);
                const double nuE = (fxw(c, 0, i + 1) * visc[FI(c, i + 1, j, k)] + (1.0 - fxw(c, 0, i + 1)) * visc[f]) * (1 - iup[f]) + arr_at(bcvisc3[0], f) * iup[f];
                const double nuW = (fxw(c, 0, i) * visc[f] + (1.0 - fxw(c, 0, i)) * visc[FI(c, i - 1, j, k)]) * (1 - ium[f]) + arr_at(bcvisc3[0], f) * ium[f];
                const double nuN = (fxw(c, 1, j + 1) * visc[FI(c, i, j + 1, k)] + (1.0 - fxw(c, 1, j + 1)) * visc[f]) * (1 - jup[f]) + arr_at(bcvisc3[1], f) * jup[f];
                const double nuS = (fxw(c, 1, j) * visc[f] + (1.0 - fxw(c, 1, j)) * visc[FI(c, i, j - 1, k)]) * (1 - jum[f]) + arr_at(bcvisc3[1], f) * jum[f];
                const double nuF = (fxw(c, 2, k + 1) * visc[FI(c, i, j, k + 1)] + (1.0 - fxw(c, 2, k + 1)) * visc[f]) * (1 - kup[f]) + arr_at(bcvisc3[2], f) * kup[f];
                const double nuB = (fxw(c, 2, k) * visc[f] + (1.0 - fxw(c, 2, k)) * visc[FI(c, i, j, k - 1)]) * (1 - kum[f]) + arr_at(bcvisc3[2], f) * kum[f];
                double t;
                t = (c->dxcinv[0][i] * (1 - ium[f]) + c->dxinv[0][i] * ium[f] * 2.0) * c->dxinv[0][i];
                c->ad[0][f] = -(0.5 * dt * nuW) * t;
                t = (c->dxcinv[0][i + 1] * (1 - iup[f]) + c->dxinv[0][i] * iup[f] * 2.0) * c->dxinv[0][i];
                c->ad[1][f] = -(0.5 * dt * nuE) * t;
                t = (c->dxcinv[1][j] * (1 - jum[f]) + c->dxinv[1][j] * jum[f] * 2.0) * c->dxinv[1][j];
                c->ad[2][f] = -(0.5 * dt * nuS) * t;
                t = (c->dxcinv[1][j + 1] * (1 - jup[f]) + c->dxinv[1][j] * jup[f] * 2.0) * c->dxinv[1][j];
                c->ad[3][f] = -(0.5 * dt * nuN) * t;
                t = (c->dxcinv[2][k] * (1 - kum[f]) + c->dxinv[2][k] * kum[f] * 2.0) * c->dxinv[2][k];
                c->ad[4][f] = -(0.5 * dt * nuB) * t * rnDim;
                t = (c->dxcinv[2][k + 1] * (1 - kup[f]) + c->dxinv[2][k] * kup[f] * 2.0) * c->dxinv[2][k];
                c->ad[5][f] = -(0.5 * dt * nuF) * t * rnDim;
            }
}

/* The row of cell (i,j,k) as itsolv_ad_x/y/z and calc_residual_ad form it
 * (IBM/CORE_SOLVE_AD.F90:343-390): per axis the coefficients with the
 * Crank-Nicolson convective terms (half_dt = 0 for ADAMS_BASHFORTH2). */
static void ad_row(or_ctx *c, double half_dt, const double *const *faces, int i, int j, int k, double am[3],
                   double ap[3], double ac[3])
{
    const size_t f = FI(c, i, j, k);
    const int idx[3] = {i, j, k};
    for (int a = 0; a < 3; ++a) {
        const int t = idx[a];
        const int8_t mm = c->fl[2 * a][f], pp = c->fl[2 * a + 1][f];
        const size_t fp = (a == 0) ? FI(c, i + 1, j, k) : (a == 1) ? FI(c, i, j + 1, k) : FI(c, i, j, k + 1);
        am[a] = c->ad[2 * a][f];
        ap[a] = c->ad[2 * a + 1][f];
        ac[a] = -(am[a] + ap[a]);
        double tmp1 = 1.0 - fxw(c, a, t), tmp2 = fxw(c, a, t + 1);
        am[a] = am[a] - half_dt * faces[a][f] * tmp1 * c->dxinv[a][t];
        ap[a] = ap[a] + half_dt * faces[a][fp] * tmp2 * c->dxinv[a][t];
        tmp1 = fxw(c, a, t) * (1 - mm);
        tmp2 = (1.0 - fxw(c, a, t + 1)) * (1 - pp);
        ac[a] = ac[a] + half_dt * (faces[a][fp] * tmp2 - faces[a][f] * tmp1) * c->dxinv[a][t];
    }
}

/* rhs_adjust_bc (IBM/CORE_RHS_AD.F90:588-780, stationary boundary, no FSI):
 * the boundary values of flagged faces move to the right-hand side. */
void or_rhs_adjust_bc(or_ctx *c, int advec_scheme, double dt, const double *const *faces, const double *const *bc9,
                      double *nlu, double *nlv, double *nlw)
{
    const double half_dt = (advec_scheme == 1) ? 0.0 : 0.5 * dt;
    if (!c->ad[0]) return;   /* or_set_solve_ad first */
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                const int idx[3] = {i, j, k};
                double md[3], pd[3];
                for (int a = 0; a < 3; ++a) {
                    const int t = idx[a];
                    const int8_t mm = c->fl[2 * a][f], pp = c->fl[2 * a + 1][f];
                    const size_t fp = (a == 0) ? FI(c, i + 1, j, k) : (a == 1) ? FI(c, i, j + 1, k) : FI(c, i, j, k + 1);
                    md[a] = c->ad[2 * a][f];
                    pd[a] = c->ad[2 * a + 1][f];
                    const double tmp1 = (1.0 - fxw(c, a, t)) * (1 - mm) + mm;
                    const double tmp2 = fxw(c, a, t + 1) * (1 - pp) + pp;
                    md[a] = md[a] - half_dt * faces[a][f] * tmp1 * c->dxinv[a][t];
                    pd[a] = pd[a] + half_dt * faces[a][fp] * tmp2 * c->dxinv[a][t];
                }
                double *nl[3] = {nlu, nlv, nlw};
                for (int q = 0; q < 3; ++q) {
                    const double *bx = bc9[3 * q], *by = bc9[3 * q + 1], *bz = bc9[3 * q + 2];
                    nl[q][f] = nl[q][f] - md[0] * arr_at(bx, f) * c->fl[0][f] - pd[0] * arr_at(bx, f) * c->fl[1][f]
                               - md[1] * arr_at(by, f) * c->fl[2][f] - pd[1] * arr_at(by, f) * c->fl[3][f]
                               - md[2] * arr_at(bz, f) * c->fl[4][f] - pd[2] * arr_at(bz, f) * c->fl[5][f];
                }
            }
}

/* itsolv_ad_x / _y / _z (IBM/CORE_SOLVE_AD.F90:314-762 and the _AB variants):
 * line Gauss-Seidel along axis d.  order 0: the reference's lexicographic
 * line order; order 1: red-black over the two transverse indices (colour 0
 * first), the order of the GPU sweep. */
static void itsolv_ad_dir(or_ctx *c, int d, double half_dt, const double *const *faces, double *var, const double *r,
                          int order)
{
    const int nc[3] = {c->nxc, c->nyc, c->nzc};
    const int n = nc[d];
    double *A = zalloc(sizeof(double) * (size_t)(n + 2)), *B = zalloc(sizeof(double) * (size_t)(n + 2));
    double *C = zalloc(sizeof(double) * (size_t)(n + 2)), *R = zalloc(sizeof(double) * (size_t)(n + 2));
    double *U = zalloc(sizeof(double) * (size_t)(n + 2)), *G = zalloc(sizeof(double) * (size_t)(n + 2));
    /* outer loops: x (k, j), y (k, i), z (i, j) */
    const int o1 = (d == 2) ? c->nxc : c->nzc;
    const int o2 = (d == 0) ? c->nyc : (d == 1 ? c->nxc : c->nyc);
    for (int pass = 0; pass < (order ? 2 : 1); ++pass)
        for (int q1 = 1; q1 <= o1; ++q1)
            for (int q2 = 1; q2 <= o2; ++q2) {
                if (order && ((q1 + q2) & 1) != pass) continue;
                for (int t = 1; t <= n; ++t) {
                    const int i = (d == 0) ? t : (d == 1 ? q2 : q1);
                    const int j = (d == 0) ? q2 : (d == 1 ? t : q2);
                    const int k = (d == 0) ? q1 : (d == 1 ? q1 : t);
                    const size_t f = FI(c, i, j, k);
                    double am[3], ap[3], ac[3];
                    ad_row(c, half_dt, faces, i, j, k, am, ap, ac);
                    const double rib = 1.0 - (double)c->iblank[f];
                    const size_t nb[3][2] = {{FI(c, i - 1, j, k), FI(c, i + 1, j, k)},
                                             {FI(c, i, j - 1, k), FI(c, i, j + 1, k)},
                                             {FI(c, i, j, k - 1), FI(c, i, j, k + 1)}};
                    double rhs;
                    if (d == 2) {   /* z-lines subtract term by term, y before x (:678-681) */
                        rhs = r[f] - var[nb[1][0]] * am[1] * (1 - c->fl[2][f]) - var[nb[1][1]] * ap[1] * (1 - c->fl[3][f])
                              - var[nb[0][0]] * am[0] * (1 - c->fl[0][f]) - var[nb[0][1]] * ap[0] * (1 - c->fl[1][f]);
                    } else {        /* x- and y-lines subtract one parenthesised sum */
                        const int a1 = (d == 0) ? 1 : 0;
                        const double s = var[nb[a1][0]] * am[a1] * (1 - c->fl[2 * a1][f])
                                       + var[nb[a1][1]] * ap[a1] * (1 - c->fl[2 * a1 + 1][f])
                                       + var[nb[2][0]] * am[2] * (1 - c->fl[4][f])
                                       + var[nb[2][1]] * ap[2] * (1 - c->fl[5][f]);
                        rhs = r[f] - s;
                    }
                    A[t] = am[d] * rib * (1 - c->fl[2 * d][f]);
                    C[t] = ap[d] * rib * (1 - c->fl[2 * d + 1][f]);
                    B[t] = 1.0 + (ac[0] + ac[1] + ac[2]) * rib;
                    R[t] = rhs * rib + var[f] * (double)c->ghost[f];
                }
                tdma_w(A, B, C, R, U, G, 1, n);
                for (int t = 1; t <= n; ++t) {
                    const int i = (d == 0) ? t : (d == 1 ? q2 : q1);
                    const int j = (d == 0) ? q2 : (d == 1 ? t : q2);
                    const int k = (d == 0) ? q1 : (d == 1 ? q1 : t);
                    var[FI(c, i, j, k)] = U[t];
                }
            }
    free(A); free(B); free(C); free(R); free(U); free(G);
}

/* calc_residual_ad (IBM/CORE_SOLVE_AD.F90:766-907, no fresh cells): max |res|
 * over the interior, res masked by (1 - iblank). */
static double calc_residual_ad(or_ctx *c, double half_dt, const double *const *faces, const double *var,
                               const double *r)
{
    double resm = 0.0;
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                double am[3], ap[3], ac[3];
                ad_row(c, half_dt, faces, i, j, k, am, ap, ac);
                double res = r[f] - var[f] * (1.0 + (ac[0] + ac[1] + ac[2]))
                             - var[FI(c, i - 1, j, k)] * am[0] * (1 - c->fl[0][f])
                             - var[FI(c, i + 1, j, k)] * ap[0] * (1 - c->fl[1][f])
                             - var[FI(c, i, j - 1, k)] * am[1] * (1 - c->fl[2][f])
                             - var[FI(c, i, j + 1, k)] * ap[1] * (1 - c->fl[3][f])
                             - var[FI(c, i, j, k - 1)] * am[2] * (1 - c->fl[4][f])
                             - var[FI(c, i, j, k + 1)] * ap[2] * (1 - c->fl[5][f]);
                res = res * (double)(1 - c->iblank[f]);
                if (fabs(res) > resm) resm = fabs(res);
            }
    return resm;
}

/* solve_ad (IBM/CORE_SOLVE_AD.F90:12-267), LSOR branch, stationary boundary:
 * itsolv_ad on u, v (, w), then with GCM the ghost-cell velocities
 * (GCM_GhostCell_Vel, IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:20-122, whose
 * mass-flux correction is inactive without zero-gradient faces), until the
 * largest residual is <= restol_ad or iterMax_ad iterations.  order: 0 the
 * reference's lexicographic line order, 1 red-black.  Returns the iteration
 * count; *maxres receives the final residual. */
/* remove_rhs_adjust_bc (sign +1) and rhs_readjust_bc (sign -1),
 * IBM/GCM_GLOBAL_MASS_CONSERVE.F90:90-252: the implicit diffusion coefficients
 * with the constant reinv (not viscTot, no convective part) times the boundary
 * values of flagged faces, added to or taken from nlu, nlv, nlw. */
static void rhs_bc_terms(or_ctx *c, double dt, double reinv, double *const *bc9, double *const *nl, int sign)
{
    const double rnDim = (double)(c->p.ndim - DIM_2D);
    const int8_t *ium = c->fl[0], *iup = c->fl[1], *jum = c->fl[2], *jup = c->fl[3], *kum = c->fl[4], *kup = c->fl[5];
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                double amxd = (c->dxcinv[0][i] * (1 - ium[f]) + c->dxinv[0][i] * ium[f] * 2.0) * c->dxinv[0][i];
                double apxd = (c->dxcinv[0][i + 1] * (1 - iup[f]) + c->dxinv[0][i] * iup[f] * 2.0) * c->dxinv[0][i];
                double amyd = (c->dxcinv[1][j] * (1 - jum[f]) + c->dxinv[1][j] * jum[f] * 2.0) * c->dxinv[1][j];
                double apyd = (c->dxcinv[1][j + 1] * (1 - jup[f]) + c->dxinv[1][j] * jup[f] * 2.0) * c->dxinv[1][j];
                double amzd = (c->dxcinv[2][k] * (1 - kum[f]) + c->dxinv[2][k] * kum[f] * 2.0) * c->dxinv[2][k];
                double apzd = (c->dxcinv[2][k + 1] * (1 - kup[f]) + c->dxinv[2][k] * kup[f] * 2.0) * c->dxinv[2][k];
                amxd = -(0.50 * dt * reinv) * amxd;
                apxd = -(0.50 * dt * reinv) * apxd;
                amyd = -(0.50 * dt * reinv) * amyd;
                apyd = -(0.50 * dt * reinv) * apyd;
                amzd = -(0.50 * dt * reinv) * amzd * rnDim;
                apzd = -(0.50 * dt * reinv) * apzd * rnDim;
                for (int q = 0; q < 3; ++q) {
                    const double *bx = bc9[3 * q], *by = bc9[3 * q + 1], *bz = bc9[3 * q + 2];
                    double *r = nl[q];
                    if (sign > 0)
                        r[f] = r[f] + amxd * bx[f] * ium[f] + apxd * bx[f] * iup[f] + amyd * by[f] * jum[f]
                               + apyd * by[f] * jup[f] + amzd * bz[f] * kum[f] + apzd * bz[f] * kup[f];
                    else
                        r[f] = r[f] - amxd * bx[f] * ium[f] - apxd * bx[f] * iup[f] - amyd * by[f] * jum[f]
                               - apyd * by[f] * jup[f] - amzd * bz[f] * kum[f] - apzd * bz[f] * kup[f];
                }
            }
}

/* GCM_enforce_global_mass_consv (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:6-86), the
 * end of GCM_GhostCell_Vel with zero-gradient sides: face_vel of the current
 * velocities (NO_VAN_KAN) into the step's faces, the net face flux out of the
 * fluid cells, the boundary terms of the right-hand sides removed, the
 * zero-gradient planes corrected by -massflux / outflow_area and the terms
 * put back with the corrected values. */
static void gcm_enforce_global_mass_consv(or_ctx *c, double dt, double reinv, double *u, double *v, double *w,
                                          double *const *faces, double *const *bc9, double *const *nl)
{
    or_face_vel(c, 0, dt, u, v, w, NULL, bc9[0], bc9[4], bc9[8], faces[0], faces[1], faces[2]);
    const double *fu = faces[0], *fv = faces[1], *fw = faces[2];
    double massflux = 0.0;
    for (int k = 1; k <= c->nzc; ++k)
        for (int j = 1; j <= c->nyc; ++j)
            for (int i = 1; i <= c->nxc; ++i) {
                const size_t f = FI(c, i, j, k);
                const double dx = c->dx[0][i], dy = c->dx[1][j], dz = c->dx[2][k];
                massflux = massflux + (-(fu[f] * dy * dz) + fu[FI(c, i + 1, j, k)] * dy * dz
                                       - fv[f] * dx * dz + fv[FI(c, i, j + 1, k)] * dx * dz
                                       - fw[f] * dx * dy + fw[FI(c, i, j, k + 1)] * dx * dy)
                                          * (double)(1 - c->iblank[f]);
            }
    rhs_bc_terms(c, dt, reinv, bc9, nl, +1);
    zg_correct_planes(c, bc9, -massflux / c->p.outflow_area);
    rhs_bc_terms(c, dt, reinv, bc9, nl, -1);
}

int or_solve_ad(or_ctx *c, int advec_scheme, double dt, double *const *faces_w, double *u, double *v, double *w,
                double *nlu, double *nlv, double *nlw, double *const *bc9, double reinv, int order, double *maxres)
{
    const double *const *faces = (const double *const *)faces_w;
    int zg = 0;
    for (int s = 0; s < 6; ++s) zg |= (c->p.bc[s] == BC_ZERO_GRADIENT);
    const int mass_consv = zg && c->p.boundary_formulation == GCM_METHOD;
    if (mass_consv && (!bc9 || !(c->p.outflow_area > 0.0))) return -1;
    double *nlr[3] = {nlu, nlv, nlw};
    const double half_dt = (advec_scheme == 1) ? 0.0 : 0.5 * dt;
    if (!c->ad[0]) return -1;   /* or_set_solve_ad first */
    const int three_d = (c->p.ndim == DIM_3D);
    const int gcm = (c->p.boundary_formulation == GCM_METHOD);
    double *vel[3] = {u, v, w};
    const double *rr[3] = {nlu, nlv, nlw};
    const int ncomp = three_d ? 3 : 2;
    double mr = 0.0;
    for (int q = 0; q < ncomp; ++q) {
        const double rq = calc_residual_ad(c, half_dt, faces, vel[q], rr[q]);
        if (rq > mr) mr = rq;
    }
    int iter = 0;
    if (gcm) mr = 1.0e10;   /* the GCM branch starts its loop unconditionally */
    while (iter < c->p.iterMax_ad && mr > c->p.restol_ad) {
        for (int q = 0; q < ncomp; ++q) {
            itsolv_ad_dir(c, 0, half_dt, faces, vel[q], rr[q], order);
            itsolv_ad_dir(c, 1, half_dt, faces, vel[q], rr[q], order);
            if (three_d) itsolv_ad_dir(c, 2, half_dt, faces, vel[q], rr[q], order);
        }
        if (gcm && c->vg_on) gcm_vel_set_bc_internal(c, u, v, w);
        if (mass_consv) gcm_enforce_global_mass_consv(c, dt, reinv, u, v, w, faces_w, bc9, nlr);
        /* CRANK_NICOLSON2: face_vel of the current velocities after the sweeps (and the
         * ghost-cell velocities under GCM), IBM/CORE_SOLVE_AD.F90:155,236; the rows' convective
         * terms and the residual then use the new faces */
        if (advec_scheme == 3)
            or_face_vel(c, 0, dt, u, v, w, NULL, bc9 ? bc9[0] : NULL, bc9 ? bc9[4] : NULL, bc9 ? bc9[8] : NULL,
                        faces_w[0], faces_w[1], faces_w[2]);
        mr = 0.0;
        for (int q = 0; q < ncomp; ++q) {
            const double rq = calc_residual_ad(c, half_dt, faces, vel[q], rr[q]);
            if (rq > mr) mr = rq;
        }
        ++iter;
    }
    if (maxres) *maxres = mr;
    return iter;
}
