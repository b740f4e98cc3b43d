// Device kernels of the pressure-Poisson multigrid (sm_103a) and their host
// launchers.  A level array covers (0:m0, 0:m1, 0:m2), column-major with strides
// sx, sxy (level 1 keeps the caller's (0:nx+1)^3 pitch, coarse levels are dense).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fsimg {

// per-cell flag byte
enum : uint8_t {
    FB_IB = 1,    // iblank (of this level)
    FB_GM = 2,    // ghost-cell mark (level 1 only)
    FB_FACE = 4,  // face bits: 4 << (2*axis) minus side, 8 << (2*axis) plus side (flag value 1)
};
__host__ __device__ constexpr uint8_t fb_minus(int axis) { return (uint8_t)(4u << (2 * axis)); }
__host__ __device__ constexpr uint8_t fb_plus(int axis) { return (uint8_t)(8u << (2 * axis)); }

struct Dims {
    int m[3];          // upper bounds
    long long sx, sxy; // strides
    __host__ __device__ long long idx(int i, int j, int k) const { return i + sx * j + sxy * k; }
    __host__ __device__ long long count() const { return sxy * (long long)(m[2] + 1); }
};

template <typename T>
struct Coef {         // 1D face coefficients per axis: cm[i] = dcinv(i) dinv(i), cp[i] = dcinv(i+1) dinv(i)
    const T *cm[3];
    const T *cp[3];
};

template <typename T>
struct LineArgs {
    T *v;
    const T *r;
    const uint8_t *fl;
    const T *binv;
    const T *gam;
    T *U;
    Coef<T> c;
    Dims d;
    int colour;
    T omega;
    int dir_lo, dir_hi;   // finest-level Dirichlet ends along the line direction
    T ppp_lo, ppp_hi;
    const double *wpf = nullptr;   // factored partition table of this level and direction (FP64), or null
};

template <typename T>
struct FactorArgs {   // line factorisation of the smoother's tridiagonal systems
    const uint8_t *fl;
    Coef<double> c;
    Dims d;
    double *binv64, *gam64;
    float *binv32, *gam32;
};

template <typename T>
struct RestrictArgs {
    const T *v, *r;          // fine level
    const uint8_t *fl;       // fine flags
    Coef<T> c;               // fine coefficients
    Dims df, dc;
    const T *w1, *w2;        // per coarse index along D
    T *rc;                   // coarse rhs
};

template <typename T>
struct ProlongArgs {
    const T *phi;            // coarse correction
    const uint8_t *flc;      // coarse flags (iblank bit)
    T *v;                    // fine var
    const uint8_t *flf;      // fine flags
    Dims df, dc;
    const int *cA, *cB;      // per fine index along D
    const T *wA, *wB;
    const int8_t *mode;      // 0 skip, 1 copy cA, 2 masked interpolation
};

struct GhostArgs {
    int n;
    const long long *gidx;   // ghost cell linear index (level-1 layout)
    const long long *sidx;   // 8 stencil indices per ghost, -1 = the ghost itself (uNormal term)
    const int *sg;           // the same stencil as: cell index (>= 0) of a non-ghost cell,
                             // -(m + 2) for ghost cell number m, -1 for the uNormal term
    const int *gg_ptr;       // ghost-ghost couplings in CSR form: entries gg_ptr[n] .. gg_ptr[n+1]-1
    const int *gg_idx;       // of ghost n refer to ghost gg_idx[q] with weight (per precision) gg_coef[q]
};

// The fractional-step operations either side of the pressure solve, on
// level-1 full-layout FP64 arrays (face arrays share the cell layout: face
// index i of axis a sits at the cell (i, j, k) it is the minus face of).
struct StepArgs {
    const double *vel[3];     // cell velocities u, v, w
    double *velo[3];          // corrected velocities (correct_vel; may alias vel), uTilde (face_vel, VAN_KAN)
    const double *bc[3];      // bcxu, bcyv, bczw (null: zero)
    double *face[3];          // face_u, face_v, face_w
    double *nlu0;
    const double *p;          // pPrime
    const uint8_t *fl;        // level-1 flag bytes (iblank, face bits)
    const double *fx[3], *gx[3], *dxinv[3], *dxcinv[3], *dx[3];   // gx = 1 - fx
    Dims d;
    double dt, dtinv;
    int gcm;                  // boundary_formulation == GCM_METHOD
};
// face_vel + rhs_poisson (IBM/CORE_FRAC_STEP_ROUTINES.F90:36-177, IBM/CORE_POISSON.F90:155-163,
// 273-281; with van_kan, p is the current pressure and velo the uTilde scratch); sums[0]
// receives sum nlu0 dx dy dz; partials holds cap doubles.  nlu0 is zero outside the interior.
void launch_face_vel_rhs(const StepArgs &a, bool van_kan, double *partials, int cap, double *sums, cudaStream_t s);
// correct_vel cell-centre update and face corrections (IBM/CORE_FRAC_STEP_ROUTINES.F90:244-448,
// without the ghost-cell velocity interpolation)
void launch_correct_vel(const StepArgs &a, cudaStream_t s);
// Outer boundary values (set_bc, IBM/CORE_SET_BC.F90:22-298), level-1 full-layout FP64.
struct SetBcArgs {
    double *vel[3];             // u, v, w (outer ghost layers written by the ghost phase)
    double *bc[9];              // bcxu, bcyu, bczu, bcxv, ... (component-major: bc[3 comp + axis])
    const double *xn[3];        // node coordinates x(0:n+1)
    const uint8_t *fl;
    const double *dx[3];
    const double *sums;         // sums[0] = boundary mass flux (ghost phase, zero-gradient sides)
    int type[6];                // bcx1 .. bcz2
    double val[6][3];           // per side and component: the Dirichlet / pulsatile value or shear amplitude
    double xout, yout, outflow_area;
    Dims d;
};
// the boundary-value planes of all three axes
void launch_set_bc_planes(const SetBcArgs &a, cudaStream_t s);
// enforce_global_mass_consv's flux (IBM/CORE_SET_BC.F90:319-337) into sums[0]; partials holds cap doubles
void launch_bc_massflux(const SetBcArgs &a, double *partials, int cap, double *sums, cudaStream_t s);
// the zero-gradient corrections of axis `axis` (when mass_consv) followed by set_outer_ghost_vel's
// update of that axis' ghost layers (IBM/CORE_SET_OUTER_GHOST.F90); axes run in the order x, y, z
void launch_outer_ghost_vel(const SetBcArgs &a, int axis, bool mass_consv, cudaStream_t s);

// GCM_enforce_global_mass_consv's right-hand-side and boundary-value update
// (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:52-84) after the face flux sum is in sums[0].
struct ZgArgs {
    double *nl[3];              // nlu, nlv, nlw
    double *bc[9];              // as SetBcArgs::bc
    const uint8_t *fl;
    const double *cm[3], *cp[3], *cb[3];   // dcinv(i) dinv(i), dcinv(i+1) dinv(i), (2 dinv(i)) dinv(i)
    const double *sums;
    int type[6];
    double hdr;                 // 0.5 dt reinv
    double outflow_area;
    int three_d;
    Dims d;
};
// remove_rhs_adjust_bc with the current boundary values, then rhs_readjust_bc with the corrected ones
void launch_zg_rhs_terms(const ZgArgs &a, cudaStream_t s);
// the zero-gradient corrections of the normal components on the whole planes
void launch_zg_planes(const ZgArgs &a, cudaStream_t s);

// Momentum right-hand side (rhs_advec_diff, IBM/CORE_RHS_AD.F90:13-585), level-1 full-layout FP64.
struct RhsAdArgs {
    const double *vel[3];       // u, v, w
    const double *face[3];      // face_u, face_v, face_w
    const double *bc[9];        // bcxu, bcyu, bczu, bcxv, ... (component-major; null = zero)
    const double *visc;         // viscTot
    const double *bcvisc[3];    // null = zero
    const double *ew;           // exp_weight (null = 1.5)
    double *nlold[3];
    const double *p;            // VAN_KAN pressure
    double *nl[3];
    const uint8_t *fl;
    const double *fx[3], *gx[3], *dxinv[3];
    const double *cm[3], *cp[3], *cb[3];   // dcinv(i) dinv(i), dcinv(i+1) dinv(i), (2 dinv(i)) dinv(i)
    Dims d;
    double dt;
    double alfa;                // hybrid advection weight (used when hybrid is set)
    int ab2, vankan, three_d, hybrid;
};
void launch_rhs_advec_diff(const RhsAdArgs &a, cudaStream_t s);

// Implicit momentum operator (set_solve_ad + the Crank-Nicolson convective terms of
// itsolv_ad / calc_residual_ad): per cell the masked off-diagonals co[2a] = am_a (1 - m_a),
// co[2a+1] = ap_a (1 - p_a) and co[6] = acx + acy + acz (unmasked, without the 1).
struct AdCoefArgs {
    const double *face[3];
    const double *visc;
    const double *bcvisc[3];
    double *co[7];
    const uint8_t *fl;
    const double *fx[3], *gx[3], *dxinv[3];
    const double *cm[3], *cp[3], *cb[3];
    Dims d;
    double dt, half_dt;
    int three_d;
};
void launch_ad_coef(const AdCoefArgs &a, cudaStream_t s);
// rhs_adjust_bc (IBM/CORE_RHS_AD.F90:588-780): nl -= (boundary values of flagged faces) x coefficients
void launch_rhs_adjust_bc(const AdCoefArgs &c, const double *const bc[9], double *const nl[3], cudaStream_t s);
// one-time attributes of the warp-per-line momentum sweeps (called by init_kernels)
cudaError_t init_ad_line_kernels();
// one colour of the line sweep of itsolv_ad along axis dir on var with right-hand side r
void launch_ad_line(int dir, int colour, const AdCoefArgs &c, double *var, const double *r, double *gam,
                    cudaStream_t s);
// max |calc_residual_ad| over ncomp (2 or 3) components in one pass into *maxbits
void launch_ad_residual_all(const AdCoefArgs &c, double *const var[3], const double *const r[3], int ncomp,
                            unsigned long long *maxbits, cudaStream_t s);

// ghost-cell velocities u, v, w (GCM_vel_set_bc_internal); coeffD 8 per ghost, bi the
// body-intercept velocities (3 x n: u, v, w; null = zero), scratch 6 x n doubles
void launch_vel_ghosts(double *u, double *v, double *w, const GhostArgs &g, const double *coeffD, const double *bi,
                       double bw, double iw, double *scratch, int iterMax, double tol, int *d_iters,
                       unsigned long long *d_maxdelta, cudaStream_t s);
// update_pressure without its ghost rows (IBM/CORE_FRAC_STEP_ROUTINES.F90:949-967)
void launch_update_pressure(double *p, const double *pPrime, long long n, bool van_kan, cudaStream_t s);
// FP64 pipe roof: launches the DFMA-throughput kernel, returns its FP64 flops per launch
double launch_dfma_peak(double *out, cudaStream_t s);

// one-time kernel attributes (call before the first launch, outside stream capture)
cudaError_t init_kernels();

// ---- launchers (all asynchronous on the given stream) ----
template <typename T>
void launch_line(int dir, const LineArgs<T> &a, bool omega_one, cudaStream_t s);
void launch_factor(int dir, const FactorArgs<double> &a, cudaStream_t s);
// Factored partition tables (FP64 smoother): doubles needed for direction dir of
// a level (0 when its lines are not in the partition solver's range), and the
// setup kernel that fills them from the level's flags and coefficients.
long long wpf_table_doubles(int dir, const Dims &d);
void launch_wpf_setup(int dir, const FactorArgs<double> &a, double *tab, cudaStream_t s);
template <typename T>
void launch_resid_restrict(int D, const RestrictArgs<T> &a, cudaStream_t s);
template <typename T>
void launch_prolong_correct(int D, const ProlongArgs<T> &a, cudaStream_t s);
template <typename T>
void launch_outer_ghost(T *v, const Dims &d, const int sign[6], cudaStream_t s);
// scratch holds 3 n values of T (two ping-pong buffers and the fixed fluid part of each row);
// gg_coef: the ghost-ghost weights in the CSR order of g.gg_ptr / g.gg_idx
template <typename T>
void launch_ghost_rows(T *v, const GhostArgs &g, const T *coeff, const T *gg_coef, T *scratch, int iterMax,
                       double tol, double reltol, int *d_iters, unsigned long long *d_maxdelta, cudaStream_t s);
template <typename T>
void launch_fill(T *p, long long n, T val, cudaStream_t s);

// fine-level (level 1) reductions and updates, FP64
struct MaxLoc { double v; long long i; };
void launch_calc_residual(const double *p, const double *b, const double *nlw0, const uint8_t *fl,
                          const Coef<double> &c, const Dims &d, float *r32_out, MaxLoc *partials,
                          int nblocks, MaxLoc *result, cudaStream_t s, double *r64_out = nullptr);
// Krylov support (level-1 interior, fluid cells); T = double or float, dot
// products returned in FP64
template <typename T>
void launch_apply_op(const T *z, T *w, const uint8_t *fl, const Coef<T> &c, const Dims &d, cudaStream_t s);
template <typename T>
void launch_mdot(const T *const *V, int nv, const T *w, const uint8_t *fl, const Dims &d, double *partials,
                 int nblocks, double *out, cudaStream_t s);
template <typename T>
void launch_maxpy(T *w, const T *const *V, int nv, const double *coef, double sign, long long n, cudaStream_t s);
template <typename T, typename S>
void launch_scale_copy(T *dst, const S *src, const double *nrm2, long long n, cudaStream_t s);
int calc_residual_blocks(const Dims &d);
// fresh cells of a moving body take the mean of their non-blanked, non-fresh neighbours
void launch_fresh_cells(double *p, const uint8_t *fl, const uint8_t *fresh, const Dims &d, bool three_d,
                        cudaStream_t s);
// Mean removal (subtracting_average_pressure) with its partial sums in a
// file-scope device array instead of caller or handle memory: at most
// NOALLOC_MAX_ROWS (j, k) rows; devices numbered below NOALLOC_MAX_DEVICES.
constexpr int NOALLOC_MAX_ROWS = 65536;
constexpr int NOALLOC_MAX_DEVICES = 64;
cudaError_t launch_subtract_average_noalloc(double *p, const uint8_t *fl, const double *dx, const double *dy,
                                            const double *dz, const Dims &d, cudaStream_t s);
void launch_subtract_average(double *p, const uint8_t *fl, const double *dx, const double *dy,
                             const double *dz, const Dims &d, double *partials, int nblocks,
                             cudaStream_t s);
void launch_compat(const double *p, const uint8_t *fl, const double *pg, const double *dx,
                   const double *dy, const double *dz, const double *dxcinv, const double *dycinv,
                   const double *dzcinv, const int side_flag[6], const Dims &d, double *partials,
                   int nblocks, double *pgrad, const int bc_zero_grad[6], double outflow_area,
                   int nx, int ny, int nz, cudaStream_t s);
// w += (phi . z / outflow_area) n1: the rank-one part of the operator that the compatibility
// correction adds (phi . z the pressure-gradient flux of z through the unflagged faces of the
// fluid cells, n1 the nlw0 of a unit shift of the zero-gradient planes); flux receives phi . z
template <typename T>
void launch_compat_rank1(const T *z, T *w, const T *n1, const uint8_t *fl, const double *dx, const double *dy,
                         const double *dz, const double *dxcinv, const double *dycinv, const double *dzcinv,
                         const int side_flag[6], const Dims &d, double *partials, int nblocks, double *flux,
                         double outflow_area, int nx, int ny, int nz, cudaStream_t s);
void launch_nlw0(double *nlw0, const uint8_t *fl, const int side_flag[6], const double *pgrad,
                 const double *dxinv, const double *dyinv, const double *dzinv, const Dims &d,
                 int nx, int ny, int nz, cudaStream_t s);
void launch_accumulate(double *p, const float *e, long long n, cudaStream_t s);
void launch_convert_f2d(double *dst, const float *src, long long n, cudaStream_t s);
void launch_convert_d2f(float *dst, const double *src, long long n, cudaStream_t s);

// hierarchy setup
void launch_coarse_iblank(uint8_t *fl_c, const uint8_t *fl_f, const Dims &dc, const Dims &df, int D,
                          cudaStream_t s);
void launch_coarse_flags(uint8_t *fl, const Dims &d, const int side_bits[6], cudaStream_t s);

} // namespace fsimg
