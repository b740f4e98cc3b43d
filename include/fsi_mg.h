/*
 * fsi_mg.h -- C ABI of the GB300 (sm_103a) pressure-Poisson multigrid solver.
 *
 * Drop-in boundary for the fractional-step pressure solve of the reference
 * immersed-boundary FSI code.  Each entry point replaces one reference
 * routine and keeps its argument meaning; a Fortran host binds them through
 * ISO_C_BINDING interfaces (flow_structure_interaction_fem_ibm_gb300/fortran/fsi_mg_shim.F90).
 *
 * Array conventions are the reference's: Fortran column-major, lower bound 0.
 * A full field is REAL(8) (0:nx+1,0:ny+1,0:nz+1); flags are INTEGER(1) over
 * the same range; node arrays are (0:n+1).  Pointers are host pointers unless
 * the entry point says otherwise.  One host thread per handle; a handle owns
 * one CUDA stream and all device memory of its hierarchy.  That stream is
 * non-blocking: it does not wait for work on other streams, so device inputs
 * written on another stream (a torch tensor copy, for one) must be complete
 * before the call (cudaDeviceSynchronize or an event).  Every handle entry
 * point waits for its own work before it returns, so its outputs can be read
 * on any stream afterwards; fsi_mg_subtract_average_noalloc only queues its
 * work on the stream it is given.
 *
 * Status codes (all entry points):
 *    0  success / converged
 *    1  iterMax_Poisson reached with maxres > restol_Poisson (the reference
 *       prints its non-convergence message and continues,
 *       IBM/CORE_POISSON.F90:665-669)
 *    2  the ghost-cell rows did not converge within iterMax_ad
 *       (IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:374-378)
 *   <0  argument, configuration or CUDA error; fsi_mg_last_error() describes it.
 */
#ifndef FSI_MG_H
#define FSI_MG_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Hot-path input flags (IBM/MAIN.F90 read_inputs :415-489).  Field order is
 * part of the ABI. */
typedef struct {
    int ndim;                 /* 2 or 3 (DIM_2D / DIM_3D) */
    int nx, ny, nz;           /* node counts; cells are n-1; nz = 2 in 2D */
    int pp_solver_type;       /* must be 3 (PP_SOLVER_TYPE_MG) */
    int iRedBlack;            /* ignored: the GPU smoother is red-black over all lines */
    int mgcycle[3];           /* mgCycleX/Y/Z: 1 V, 2 W, 3 F */
    int iterFinest, iterCoarsest;
    int mgLevels[3];          /* 0 = automatic (IBM/CORE_MG.F90:48-78) */
    int iterMax_Poisson, iterMax_ad;
    int bc[6];                /* velocity BC types bcx1,bcx2,bcy1,bcy2,bcz1,bcz2 */
    int pbc[6];               /* pressure BC types pbcx1..pbcz2 (1 Dirichlet, 2 Neumann) */
    int internal_boundary_present;
    int boundary_formulation; /* 0 none, 2 GCM_METHOD */
    int coarse_flag_mode;     /* ignored by the GPU (coarse face flags always follow the coarse iblank) */
    int precision_mode;       /* 0 FP64 throughout, 1 FP32 cycle inside FP64 refinement */
    int outer_krylov;         /* 0: the reference's stationary outer iteration; m > 0: FGMRES(m) with
                                 MG_Solver as the preconditioner (same system, same max-norm test;
                                 with zero-gradient sides and a GCM body the cycles apply the
                                 operator of the compatibility correction's fixed point) */
    double omega;             /* line-SOR relaxation */
    double restol_Poisson;    /* absolute max-norm tolerance */
    double restol_ad;         /* ghost-row fixed-point tolerance */
    double ppp[6];            /* Dirichlet pressure values pppx1..pppz2 */
    double outflow_area;      /* from set_outflow_area (IBM/BOUNDARY_SET.F90:134-221) */
    double alfa;              /* hybrid advection weight (IBM/MAIN.F90:461,649-652): |alfa| > 1e-3 blends
                                 second-order upwind faces into rhs_advec (IBM/CORE_RHS_AD.F90:150-382) */
} fsi_mg_params;

/* MG_initial (IBM/CORE_MG.F90:31): level counts and sizes, coarse metrics,
 * device buffers.  x, y, z are the node arrays (0:n+1) produced by make_grid
 * (IBM/CORE_GRID.F90:29). */
int fsi_mg_create(const fsi_mg_params *params, const double *x, const double *y, const double *z,
                  void **handle);

/* Hand over the outputs of set_boundary (IBM/BOUNDARY_SET.F90:8) after every
 * geometry change: iblank, ghostCellMark and ium..kup (INTEGER(1), full
 * range), the ordered ghost list iGhost/jGhost/kGhost with the image-point
 * stencil base iCellIndex/jCellIndex/kCellIndex and coeffGCMN(8,nGhost),
 * probeLength(nGhost) (IBM/GCM_SET_BOUNDARY.F90:2-304), and the six boundary
 * pressure-gradient planes pgradx1,pgradx2 (0:ny+1,0:nz+1), pgrady1,pgrady2
 * (0:nx+1,0:nz+1), pgradz1,pgradz2 (0:nx+1,0:ny+1) packed in that order
 * (may be NULL: all zero).  Builds the coarse iblank hierarchy, face flags,
 * line factorisations and the ghost gather list on the device. */
int fsi_mg_set_geometry(void *handle, const int8_t *iblank, const int8_t *ghostCellMark,
                        const int8_t *ium, const int8_t *iup, const int8_t *jum, const int8_t *jup,
                        const int8_t *kum, const int8_t *kup,
                        int nGhost, const int32_t *iGhost, const int32_t *jGhost, const int32_t *kGhost,
                        const int32_t *iCellIndex, const int32_t *jCellIndex, const int32_t *kCellIndex,
                        const double *coeffGCMN, const double *probeLength, const double *pgrad);

/* solve_poisson, MG branch (IBM/CORE_POISSON.F90:493-676): mean removal (or
 * Dirichlet flagging), then MG_Solver -> GCM_correct_pressure -> calc_residual
 * until maxres <= restol_Poisson or iterMax_Poisson.  pPrime is INOUT, nlu0 IN,
 * nlw0_out OUT (may be NULL); iters, maxres, loc[3] (first location of the max
 * residual) and compTime (seconds) are OUT (each may be NULL).
 * Host buffers: each call copies pPrime and nlu0 in and pPrime out. */
int fsi_mg_solve(void *handle, double *pPrime, const double *nlu0, double *nlw0_out,
                 int *iters, double *maxres, int *loc, double *compTime);

/* Same as fsi_mg_solve with DEVICE pointers to full (0:nx+1)^3 arrays already
 * resident in HBM (no host transfer of the fields). */
int fsi_mg_solve_device(void *handle, double *d_pPrime, const double *d_nlu0, double *d_nlw0_out,
                        int *iters, double *maxres, int *loc, double *compTime);

/* MG_Solver (IBM/CORE_MG.F90:281): one x-, y- (and z-) semi-coarsening cycle
 * on var (INOUT) with right-hand side rr (IN); compTime OUT.  The smoother and
 * residual procedure arguments of the reference are fixed here. */
int fsi_mg_mg_solver(void *handle, double *var, const double *rr, double *compTime);

/* calc_residual (IBM/CORE_POISSON.F90:1111): max-norm of r - A var + nlw0
 * over fluid cells and the first location (i,j,k) attaining it. */
int fsi_mg_calc_residual(void *handle, const double *var, const double *r, double *resm, int *loc);

/* subtracting_average_pressure (IBM/CORE_POISSON.F90:419), including the
 * fresh cells registered with fsi_mg_set_fresh_cells. */
int fsi_mg_subtract_average(void *handle, double *pPrime);

/* The mean removal on device arrays, for callers that cannot allocate GPU
 * memory (a host code whose device memory is owned by its own pool, or a
 * time loop that must not pay cudaMalloc's implicit device synchronisation).
 * No counterpart in the reference.  It needs no handle and allocates nothing:
 * its partial sums live in a fixed device array of the library, one slot per
 * (j,k) row, so grids with (ny-1)*(nz-1) > 65536 rows are rejected (status
 * -1, message in fsi_mg_last_error).  d_pPrime (in/out) and d_iblank use the
 * full (0:nx+1,0:ny+1,0:nz+1) layout; d_dx, d_dy, d_dz hold the cell widths
 * dx(0:nx+1) etc.  d_iblank must hold 0 or 1 as the reference's iblank does:
 * it is not validated (that would need a copy to the host), and a cell counts
 * as blanked wherever it is non-zero.  Unlike fsi_mg_subtract_average it does
 * not set fresh cells of a moving body to their neighbours' mean
 * (IBM/CORE_POISSON.F90:459-488): callers with a moving body use the handle
 * entry point.  Work is queued on `stream` (a cudaStream_t, NULL for the
 * default stream) and the call returns without waiting.  The first call in a
 * CUDA context looks up the device address of that array (again after a
 * cudaDeviceReset or a re-created context); make that call before any stream
 * capture.  All calls share the array, so calls that can overlap on the GPU
 * (other streams, host threads) race. */
int fsi_mg_subtract_average_noalloc(double *d_pPrime, const int8_t *d_iblank, const double *d_dx, const double *d_dy,
                                    const double *d_dz, int ndim, int nx, int ny, int nz, void *stream);

/* fresh_cell (IBM/AMODULES.F90:397, allocated (0:nx+1,0:ny+1,0:nz+1) at
 * IBM/GCM_MEMORY_ALLOCATE.F90:27) of a moving body, INTEGER(1) 0 or 1: from
 * now on the mean removal of every solve (and fsi_mg_subtract_average) sets
 * each fresh cell to the mean of its non-blanked, non-fresh 3x3(x3)
 * neighbours (IBM/CORE_POISSON.F90:459-488).  NULL (or all zero) turns it
 * off.  Call after each fsi_mg_set_geometry that moved the body. */
int fsi_mg_set_fresh_cells(void *handle, const int8_t *fresh_cell);

/* GCM_correct_pressure (IBM/CORE_POISSON.F90:1794): outer ghost layer,
 * ghost-cell rows, compatibility correction of pgrad*, and nlw0 (OUT, may be NULL). */
int fsi_mg_correct_pressure(void *handle, double *pPrime, double *nlw0_out);

/* The fractional-step operations either side of the solve, on DEVICE arrays
 * in the full (0:nx+1,0:ny+1,0:nz+1) layout, for a time loop that keeps its
 * fields in HBM.  Face arrays face_u/face_v/face_w share that layout (face i
 * of x at (i,j,k), i = 1..nx).  bcxu/bcyv/bczw may be NULL (all zero).  They
 * use the flags of the last fsi_mg_set_geometry and need Neumann pressure
 * sides (status -1 otherwise).  Each call waits for its work to finish.
 *
 * face_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:6-240) followed by the
 * non-hybrid rhs_poisson (IBM/CORE_POISSON.F90:123-417): face velocities from
 * u, v, w (frac_step_type 0, NO_VAN_KAN) or from uTilde = u + dt grad p with
 * the face pressure correction (1, VAN_KAN; d_p is then the current
 * pressure), the boundary masks, and with boundary_formulation GCM the
 * VAN_KAN ghost-cell faces and GCM_set_face_vel_body; then nlu0 =
 * div(face)/dt (1 - iblank), zero outside the interior; sum OUT (may be NULL)
 * = sum nlu0 dx dy dz in a fixed order. */
int fsi_mg_face_vel_rhs(void *handle, int frac_step_type, double dt, const double *d_u, const double *d_v,
                        const double *d_w, const double *d_p, const double *d_bcxu, const double *d_bcyv,
                        const double *d_bczw, double *d_face_u, double *d_face_v, double *d_face_w, double *d_nlu0,
                        double *sum);

/* correct_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:244-448) without periodic
 * sides: u, v, w -= dt grad pPrime (1 - iblank), the ghost-cell velocities
 * (GCM_vel_set_bc_internal) once fsi_mg_set_velocity_ghosts registered
 * them, the face corrections in the reference's overwrite order and, with
 * GCM, GCM_set_face_vel_body (INOUT d_u..d_w, d_face_u..d_face_w).
 * Status 2: the ghost velocities did not converge within iterMax_ad. */
int fsi_mg_correct_vel(void *handle, double dt, const double *d_pPrime, double *d_u, double *d_v, double *d_w,
                       const double *d_bcxu, const double *d_bcyv, const double *d_bczw, double *d_face_u,
                       double *d_face_v, double *d_face_w);

/* Fields of the momentum right-hand side (device arrays, full layout).  bc
 * holds bcxu, bcyu, bczu, bcxv, bcyv, bczv, bcxw, bcyw, bczw and bcvisc
 * bcxvisc, bcyvisc, bczvisc (IBM/AMODULES.F90 boundary_arrays; NULL entries
 * are zero); exp_weight NULL means 1.5 everywhere (no fresh cells,
 * IBM/BOUNDARY_FRESH_CELL.F90:25). */
typedef struct {
    const double *u, *v, *w;
    const double *face_u, *face_v, *face_w;
    const double *bc[9];
    const double *viscTot;
    const double *bcvisc[3];
    const double *exp_weight;
    double *nluOld, *nlvOld, *nlwOld;   /* INOUT with ADAMS_BASHFORTH2 */
    const double *p;                    /* frac_step_type 1 (VAN_KAN) only */
    double *nlu, *nlv, *nlw;            /* OUT (interior cells) */
    double reinv;                       /* 1/Re: the boundary terms of GCM_enforce_global_mass_consv (solve_ad
                                           with zero-gradient sides and a GCM body) */
} fsi_mg_rhs_ad_fields;

/* Outer boundary values of set_bc, per side x1, x2, y1, y2, z1, z2 and
 * component u, v, w: vel = ux1, vx1, wx1, ux2, ... (IBM/AMODULES.F90
 * flow_parameters), freq = freq_ux1, ... (pulsatile inflow), the simulation
 * time, tstart_gust (gust switch of the x2 pulsatile u) and the domain
 * lengths xout, yout (shear profiles).  Field order is part of the ABI. */
typedef struct {
    double vel[6][3];
    double freq[6][3];
    double time, tstart_gust;
    double xout, yout;
} fsi_mg_bc_values;

/* set_bc, outer part (IBM/CORE_SET_BC.F90:22-298): the boundary values of
 * the first and last cells of each axis (full planes j = 0..ny, k = 0..nz
 * etc.) by the side types of fsi_mg_params.bc (1 Dirichlet, 2 zero gradient,
 * 3 pulsatile, 4 symmetry, 7 shear; 6 user-specified needs the Blasius
 * profile and is rejected), then with any zero-gradient side
 * enforce_global_mass_consv (:304-377: the boundary mass flux over the
 * face flags of the last fsi_mg_set_geometry, corrected by -massflux /
 * outflow_area on the zero-gradient sides; iMarkm..kMarkp are zero outside
 * SSM) and set_outer_ghost_vel (IBM/CORE_SET_OUTER_GHOST.F90:1-63: u, v, w of
 * the outer ghost layers, INOUT).  bc = the nine arrays in the order of
 * fsi_mg_rhs_ad_fields.bc (device, full layout, all required, OUT on the
 * planes).  The body-intercept values of a GCM body
 * (GCM_SetBodyInterceptValues) are fsi_mg_set_velocity_ghosts' inputs.
 * correction_vel OUT (0 without zero-gradient sides; may be NULL). */
int fsi_mg_set_bc(void *handle, const fsi_mg_bc_values *values, double *d_u, double *d_v, double *d_w,
                  double *const d_bc[9], double *correction_vel);

/* rhs_advec_diff (IBM/CORE_RHS_AD.F90:13-75): advection with the face
 * velocities (rhs_advec, :80-382: central, blended with second-order upwind
 * faces by fsi_mg_params.alfa when |alfa| > 1e-3), the
 * Adams-Bashforth or Crank-Nicolson loading of the advection term
 * (rhs_loadAB, :385-430; advec_scheme 1 ADAMS_BASHFORTH2, 2 CRANK_NICOLSON1,
 * 3 CRANK_NICOLSON2), the explicit half of the diffusion with the total
 * viscosity (rhs_diff, :433-530) and, with frac_step_type 1, the old
 * pressure gradient (rhs_vankan, :550-585): nl = vel - dt NL + dt/2 D(vel).
 * Uses the flags of the last fsi_mg_set_geometry (Neumann pressure sides).
 * In 2D the w component is only touched by rhs_vankan, as in the reference. */
int fsi_mg_rhs_advec_diff(void *handle, int advec_scheme, int frac_step_type, double dt,
                          const fsi_mg_rhs_ad_fields *fields);

/* rhs_adjust_bc (IBM/CORE_RHS_AD.F90:588-780, stationary boundary, no FSI):
 * the boundary values bc of flagged faces, times the implicit coefficients
 * (diffusion with viscTot / bcvisc, Crank-Nicolson convection with the
 * faces), move from the operator to nlu, nlv, nlw (INOUT).  Uses face_*,
 * bc, viscTot, bcvisc and nl* of the fields; advec_scheme 1 (AB2), or 2 / 3
 * (CRANK_NICOLSON1 / 2, the same terms). */
int fsi_mg_rhs_adjust_bc(void *handle, int advec_scheme, double dt, const fsi_mg_rhs_ad_fields *fields);

/* solve_ad (IBM/CORE_SOLVE_AD.F90:12-267), line-SOR branch, stationary
 * boundary: the implicit operator of set_solve_ad (IBM/CORE_SET_SOLVERS.F90:
 * 20-95) plus the Crank-Nicolson convective terms, applied to u, v (, w)
 * (device, INOUT) with right-hand sides nlu, nlv, nlw of the fields, line
 * sweeps along x, y, z per component, red-black over the lines (the
 * reference sweeps them lexicographically; both converge to the same
 * solution), then under GCM the ghost-cell velocities of
 * fsi_mg_set_velocity_ghosts, until max |calc_residual_ad| <= restol_ad or
 * iterMax_ad iterations (status 1, the reference prints and continues).
 * advec_scheme 1 (AB2), 2 (CRANK_NICOLSON1) or 3 (CRANK_NICOLSON2: after the
 * sweeps, the ghost velocities and the mass balance, every iteration evaluates
 * face_vel of the current velocities into fields.face_u..face_w (NO_VAN_KAN,
 * fields.p NULL; a NULL bc array reads as 0) and the rows and the residual
 * use the new faces, :155-157 and :236).  With zero-gradient sides and
 * a GCM body every iteration ends with GCM_enforce_global_mass_consv
 * (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:6-252): face_vel of the current velocities
 * (NO_VAN_KAN; fields.p must be NULL) into fields.face_u..face_w, the net face
 * flux, the boundary terms with reinv removed from nlu..nlw, the zero-gradient
 * planes of fields.bc corrected by -massflux / outflow_area and the terms put
 * back; these fields are then INOUT and all nine bc arrays are required.
 * iters and maxres OUT (may be NULL). */
int fsi_mg_solve_ad(void *handle, int advec_scheme, double dt, const fsi_mg_rhs_ad_fields *fields, double *d_u,
                    double *d_v, double *d_w, int *iters, double *maxres);

/* Ghost-cell velocities of the GCM body for fsi_mg_correct_vel
 * (GCM_vel_set_bc_internal, IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:126-247):
 * coeffGCMD(8,nGhost), the Dirichlet image-point weights of the ghost list
 * and stencils of the last fsi_mg_set_geometry (IBM/GCM_SET_BOUNDARY.F90:
 * 282,305-486), the body-intercept velocities uBodyIntercept,
 * vBodyIntercept, wBodyIntercept (nGhost each; all NULL: a body at rest) and
 * bodyInterceptWeight, imagePointWeight (IBM/MAIN.F90:913-914); host
 * arrays.  From then on fsi_mg_correct_vel ends its cell-centre update with
 * the ghost-velocity iteration u_g = uBI bodyInterceptWeight -
 * (sum_r coeffGCMD(r) u_r) imagePointWeight, the ghost's own stencil entry
 * taking uBI, to max |du|+|dv|+|dw| <= restol_ad (status 2 after iterMax_ad
 * sweeps, as the reference prints and continues).  Call again after each
 * fsi_mg_set_geometry (which turns it off) and whenever the intercept
 * velocities change; coeffGCMD NULL turns it off. */
int fsi_mg_set_velocity_ghosts(void *handle, const double *coeffGCMD, const double *uBI, const double *vBI,
                               const double *wBI, double bodyInterceptWeight, double imagePointWeight);

/* update_pressure (IBM/CORE_FRAC_STEP_ROUTINES.F90:949-967): p = pPrime
 * (frac_step_type 0) or p += pPrime (1), then the ghost-cell pressure rows
 * of GCM_p_set_bc_internal when boundary_formulation is GCM. */
int fsi_mg_update_pressure(void *handle, int frac_step_type, const double *d_pPrime, double *d_p);

/* Current boundary pressure-gradient planes (packed as in set_geometry). */
int fsi_mg_get_pgrad(void *handle, double *pgrad);

/* Hierarchy introspection: level count of direction d (0 x, 1 y, 2 z) and the
 * cell count of level n (1-based) along d (mgLevels_X, mgrid_I(n), ...). */
int fsi_mg_level_count(void *handle, int d);
int fsi_mg_level_size(void *handle, int d, int n);

/* Single-operator access for parity checks, host buffers in the reference's
 * level layout (0:m+1 along d at coarse levels, 0:n elsewhere):
 *   op 0 MG_itsolv at level n of cycle d (a = var INOUT, b = rhs IN)
 *   op 1 MG_Residual followed by MG_Restrict (a = var, b = rhs, c = coarse OUT)
 *   op 2 MG_Prolong followed by the correction var += phi (1-iblank)
 *        (a = coarse phi IN, b = fine var INOUT)
 *   op 3 coarse iblank of level n (a = int8 OUT)
 *   op 4 face flags of level n (a = int8 OUT, 6 full arrays ium..kup)
 *   op 5 ghost-cell rows on a level-1 array (a = var INOUT, b = int OUT iterations)
 *   op 6 outer ghost layer on a level-1 array (a = var INOUT)
 *   op 7 MG_itsolv in FP32, the mixed form's smoother (a = var INOUT, b = rhs
 *        IN, both rounded to FP32 on the device; the result is widened) */
int fsi_mg_debug_level_op(void *handle, int op, int d, int n, void *a, void *b, void *c);

/* Counters of the last solve: out[0] iterations, out[1] final maxres,
 * out[2] solve seconds (CUDA events on the handle's stream), out[3] total
 * ghost-row sweeps, out[4] kernel launches since create, out[5] device bytes
 * allocated, out[6] solve wall seconds, out[7] device seconds of the last
 * host-buffer solve including its host<->device copies. */
int fsi_mg_stats(void *handle, double *out, int n);

/* Max-norm residual after each outer iteration of the last solve (the values
 * the reference prints per iteration, IBM/CORE_POISSON.F90:657-659).  Writes
 * up to cap values into out (may be NULL) and returns the iteration count. */
int fsi_mg_residual_history(void *handle, double *out, int cap);

/* Time one kernel of the level-1 hierarchy on the handle's stream with CUDA
 * events, averaged over reps launches (after one warm-up launch), on the
 * current staging fields.  which: 0/1/2 one colour of the x/y/z line sweep,
 * 3 residual + x restriction, 4 x prolongation + correction, 5 calc_residual,
 * 6/7/8 the kernels of the last fsi_mg_face_vel_rhs / fsi_mg_correct_vel /
 * fsi_mg_update_pressure call replayed on its arrays (correct_vel and the
 * VAN_KAN update_pressure then apply their update reps+1 more times; the
 * ghost-cell rows of update_pressure are not replayed), 9 the kernel of the last
 * fsi_mg_rhs_advec_diff call, 10 the FP64 pipe roof (independent DFMA chains on
 * every SM, no memory traffic; alg_bytes then receives its FP64 flops per launch).
 * precision 0 FP64, 1 FP32 (0-5 only).  alg_bytes (may be NULL) receives the algorithmic
 * bytes one launch moves.  No counterpart in the reference: a measurement hook. */
int fsi_mg_time_kernel(void *handle, int which, int precision, int reps, double *avg_ms, double *alg_bytes);

/* Event timing of the level-1 line-relaxation launches inside solves (the
 * dominant kernel family).  enable = 1 resets the counters and turns the
 * timing on, 0 turns it off, -1 only reads; the solve graphs are re-captured
 * with a CUDA event pair around every level-1 line launch, read back after
 * each outer (or Arnoldi) step, which synchronises anyway.  out[6] (may be
 * NULL): FP32 launches, FP32 summed ms, FP32 algorithmic bytes per launch,
 * FP64 launches, FP64 summed ms, FP64 algorithmic bytes per launch.  No
 * counterpart in the reference: a measurement hook. */
int fsi_mg_line_timing(void *handle, int enable, double *out);

/* Text of the last error on this thread. */
const char *fsi_mg_last_error(void);

/* deallocate_memory (IBM/CORE_MEMORY_ALLOCATE.F90:189) for this handle. */
void fsi_mg_destroy(void *handle);

#ifdef __cplusplus
}
#endif
#endif /* FSI_MG_H */
