/*
 * Oracle (TEST INFRASTRUCTURE ONLY): a plain-C, FP64, single-threaded
 * restatement of the reference pressure-Poisson multigrid path
 * (IBM/CORE_POISSON.F90 solve_poisson MG branch, IBM/CORE_MG.F90,
 * IBM/CORE_TDMA.F90, IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:250-384,
 * IBM/GCM_GLOBAL_MASS_CONSERVE.F90:260-394, IBM/CORE_SET_OUTER_GHOST.F90:66-213).
 *
 * Only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark use this library, and only as the checker.  The product path
 * (the CUDA library in flow_structure_interaction_fem_ibm_gb300/) never
 * links or calls it.
 *
 * Parity pin: the reference cannot be compiled in this environment (no
 * Fortran compiler), so this restatement is pinned by the reference's own
 * manufactured-solution known-answer test (Poisson_Tester,
 * IBM/CORE_POISSON.F90:1386-1790) and by internal cross-checks
 * (MG vs the plain line-SOR path, tdma vs a dense solve).
 *
 * Array conventions follow the reference exactly: Fortran column-major,
 * lower bound 0.  A "full" field is (0:nx+1,0:ny+1,0:nz+1); the MG working
 * copy is (0:nx,0:ny,0:nz); a level-n field of the d-cycle is
 * (0:m_d+1, ...) with the other two extents unchanged.
 */
#ifndef FSI_MG_ORACLE_H
#define FSI_MG_ORACLE_H
#include <stdint.h>

/* Same field order and types as fsi_mg_params in include/fsi_mg.h so that a
 * single ctypes Structure serves both libraries. */
typedef struct {
    int ndim;                 /* 2 or 3 */
    int nx, ny, nz;           /* node counts; cells = n-1 (nz=2 in 2D) */
    int pp_solver_type;       /* 3 = MG, 1 = LSOR */
    int iRedBlack;            /* 0 lexicographic, 1/2 reference colours, 3 full checkerboard */
    int mgcycle[3];           /* 1 V, 2 W, 3 F per direction */
    int iterFinest, iterCoarsest;
    int mgLevels[3];          /* 0 = automatic */
    int iterMax_Poisson, iterMax_ad;
    int bc[6];                /* velocity BC type x1,x2,y1,y2,z1,z2 */
    int pbc[6];               /* pressure BC type x1,x2,y1,y2,z1,z2 */
    int internal_boundary_present;
    int boundary_formulation; /* 0 none, 2 GCM */
    int coarse_flag_mode;     /* 0 reference (stale coarse flags without a body), 1 recompute */
    int precision_mode;       /* unused by the oracle */
    int outer_krylov;         /* unused by the oracle */
    double omega, restol_Poisson, restol_ad;
    double ppp[6];            /* Dirichlet pressure values x1,x2,y1,y2,z1,z2 */
    double outflow_area;
    double alfa;              /* hybrid advection weight; |alfa| > 1e-3 switches the hybrid scheme on */
} fsi_mg_params;

typedef struct or_ctx or_ctx;

or_ctx *or_create(const fsi_mg_params *p, const double *x, const double *y, const double *z);
void    or_destroy(or_ctx *c);
int     or_set_geometry(or_ctx *c, const int8_t *iblank, const int8_t *ghost,
                        const int8_t *ium, const int8_t *iup, const int8_t *jum,
                        const int8_t *jup, const int8_t *kum, const int8_t *kup,
                        int nGhost, const int32_t *iG, const int32_t *jG, const int32_t *kG,
                        const int32_t *iCI, const int32_t *jCI, const int32_t *kCI,
                        const double *coeffGCMN, const double *probeLength,
                        const double *pgrad);
int     or_solve(or_ctx *c, double *pPrime, const double *nlu0, double *nlw0_out,
                 int *iters, double *maxres, int *loc, double *res_hist);
int     or_mg_solver(or_ctx *c, double *var, const double *rr);
double  or_calc_residual(or_ctx *c, const double *var, const double *r, int *loc);
void    or_subtract_average(or_ctx *c, double *p);
/* fresh_cell (0:nx+1)^3 of a moving body for or_subtract_average (NULL: none) */
void    or_set_fresh(or_ctx *c, const int8_t *fresh);
void    or_gcm_correct_pressure(or_ctx *c, double *p);
int     or_level_count(or_ctx *c, int d);
int     or_level_size(or_ctx *c, int d, int n);
void    or_level_metrics(or_ctx *c, int d, int n, double *xnode, double *xc, double *dx,
                         double *dxinv, double *dxc, double *dxcinv);
void    or_coarse_iblank(or_ctx *c, int d, int n, int8_t *out);
void    or_level_flags(or_ctx *c, int d, int n, int8_t *out6);
void    or_itsolv_level(or_ctx *c, int d, int n, double *var, const double *r);
void    or_residual_level(or_ctx *c, int d, int n, const double *var, const double *r, double *res);
void    or_restrict_level(or_ctx *c, int d, int n, const double *res, double *r1);
void    or_prolong_level(or_ctx *c, int d, int n, const double *phi, double *corr);
void    or_ghost_update(or_ctx *c, double *var, int mx, int my, int mz, int *iters, double *resmax);
void    or_tdma(const double *a, const double *b, const double *c_, const double *r,
                double *u, int n1, int n2);
int     or_nghost_gs_last(or_ctx *c);
void    or_outer_ghost(or_ctx *c, double *var);
void    or_get_pgrad(or_ctx *c, double *pgrad);
/* fractional-step routines either side of the solve (full-layout arrays; bc may be NULL) */
void    or_face_vel(or_ctx *c, int frac_step_type, double dt, const double *u, const double *v, const double *w,
                    const double *p, const double *bcxu, const double *bcyv, const double *bczw,
                    double *face_u, double *face_v, double *face_w);
double  or_rhs_poisson(or_ctx *c, double dt, const double *face_u, const double *face_v, const double *face_w,
                       double *nlu0);
void    or_correct_vel(or_ctx *c, double dt, const double *pPrime, double *u, double *v, double *w,
                       const double *bcxu, const double *bcyv, const double *bczw,
                       double *face_u, double *face_v, double *face_w);
void    or_update_pressure(or_ctx *c, int frac_step_type, const double *pPrime, double *p);
/* set_bc (outer sides), enforce_global_mass_consv, set_outer_ghost_vel; val/freq 6 x 3 (side, component) */
int     or_set_bc(or_ctx *c, const double *val, const double *freq, double time, double tstart_gust, double xout,
                  double yout, double *u, double *v, double *w, double *const *bc9, double *correction);
void    or_set_vel_ghosts(or_ctx *c, const double *coeffD, const double *uBI, const double *vBI,
                          const double *wBI, double bodyInterceptWeight, double imagePointWeight);
int     or_vel_ghost_iters(or_ctx *c);
/* rhs_advec_diff; bc9 = bcxu,bcyu,bczu,bcxv,bcyv,bczv,bcxw,bcyw,bczw, bcvisc3 = bcx/y/zvisc (entries may be NULL) */
void    or_rhs_advec_diff(or_ctx *c, int advec_scheme, int frac_step_type, double dt, const double *u,
                          const double *v, const double *w, const double *face_u, const double *face_v,
                          const double *face_w, const double *const *bc9, const double *visc,
                          const double *const *bcvisc3, const double *exp_weight, double *nluOld, double *nlvOld,
                          double *nlwOld, const double *p, double *nlu, double *nlv, double *nlw);
/* implicit momentum solve: set_solve_ad, rhs_adjust_bc, solve_ad (order 0 reference, 1 red-black) */
void    or_set_solve_ad(or_ctx *c, double dt, const double *visc, const double *const *bcvisc3);
void    or_rhs_adjust_bc(or_ctx *c, int advec_scheme, double dt, const double *const *faces,
                         const double *const *bc9, double *nlu, double *nlv, double *nlw);
/* with zero-gradient sides and a GCM body every iteration ends with GCM_enforce_global_mass_consv,
 * which rewrites faces, the zero-gradient planes of bc9 and nlu..nlw (reinv: 1/Re) */
int     or_solve_ad(or_ctx *c, int advec_scheme, double dt, double *const *faces, double *u, double *v,
                    double *w, double *nlu, double *nlv, double *nlw, double *const *bc9, double reinv,
                    int order, double *maxres);
#endif
