// Kernels of the fractional-step operations either side of the pressure
// solve (face_vel, rhs_poisson, correct_vel, update_pressure) and of the
// momentum predictor (rhs_advec_diff, rhs_adjust_bc, solve_ad).  Each kernel
// cites the reference routine whose arithmetic it performs.
#include "device_util.cuh"
#include "partition_solve.cuh"

#include <algorithm>

namespace fsimg {

namespace {

// ---------------------------------------------------------------------------
// Fractional-step operations either side of the pressure solve.  Face index f
// of axis a is stored at the cell it is the minus face of; face n+1 sits in
// the plus-side boundary layer.  Every face is written by one thread.
//
// FP64 economy (GB300 issues FP64 at 1/64 of the FP32 rate, and these loops
// are FP64-pipe-bound long before HBM): the reference's mask products
// x (1 - m) + bc m with m in {0, 1} become selects (equal for finite values),
// 1 - fx comes from a table (the value the reference forms), dtinv is the
// host's 1/dt, and each face is interpolated once per cell.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double bc_at(const double *bc, long long o) { return bc ? bc[o] : 0.0; }

// dead cell: blanked and not a ghost cell (GCM_set_face_vel_body zeroes its faces)
__device__ __forceinline__ bool dead_cell(uint8_t f) { return (f & FB_IB) && !(f & FB_GM); }

// Final value of face t of axis a (the minus face of cell t at flat index o)
// in face_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:80-240).  The reference writes
// face f from cell f-1 (plus side) and then from cell f (minus side), so the
// interpolation keeps cell f's minus expression; with VANKAN the pressure
// correction with p follows (:111-177); both branches then apply cell f-1's
// plus mask and cell f's minus mask (:178-195), so a face is bc(f) if
// ium(f), else bc(f-1) if iup(f-1), else the interpolated (and corrected)
// value.  With GCM, VAN_KAN re-interpolates the faces of ghost cells from u
// itself (:197-221) and GCM_set_face_vel_body zeroes the faces of dead cells.
// Cell 0 lies outside the reference's loops, so face 1 has no previous cell.
template <bool VANKAN>
__device__ __forceinline__ double face_minus(const StepArgs &A, const double *U, int a, int t, long long o,
                                             long long s, uint8_t f)
{
    const uint8_t fp = (t >= 2) ? A.fl[o - s] : (uint8_t)0;
    double v;
    if (f & fb_minus(a)) v = bc_at(A.bc[a], o);
    else if (fp & fb_plus(a)) v = bc_at(A.bc[a], o - s);
    else {
        v = fma(A.fx[a][t], U[o], A.gx[a][t] * U[o - s]);
        if (VANKAN) v = fma(-A.dt, (A.p[o] - A.p[o - s]) * A.dxcinv[a][t], v);
    }
    if (A.gcm) {
        if (VANKAN && ((f | fp) & FB_GM)) v = fma(A.fx[a][t], A.vel[a][o], A.gx[a][t] * A.vel[a][o - s]);
        if (dead_cell(f) || dead_cell(fp)) v = 0.0;
    }
    return v;
}
// face n+1 from cell n (plus expression, plus mask of cell n; ghost / dead cell n with GCM)
template <bool VANKAN>
__device__ __forceinline__ double face_last(const StepArgs &A, const double *U, int a, int n, long long o,
                                            long long s, uint8_t f)
{
    double v;
    if (f & fb_plus(a)) v = bc_at(A.bc[a], o);
    else {
        v = fma(A.fx[a][n + 1], U[o + s], A.gx[a][n + 1] * U[o]);
        if (VANKAN) v = fma(-A.dt, (A.p[o + s] - A.p[o]) * A.dxcinv[a][n + 1], v);
    }
    if (A.gcm) {
        if (VANKAN && (f & FB_GM)) v = fma(A.fx[a][n + 1], A.vel[a][o + s], A.gx[a][n + 1] * A.vel[a][o]);
        if (dead_cell(f)) v = 0.0;
    }
    return v;
}
// cell-centre pressure gradient of correct_vel / face_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:272-349):
// pe, pw interpolated to the faces, the cell's own pressure on flagged faces
__device__ __forceinline__ double cell_pgrad(const StepArgs &A, int a, int t, long long o, long long s, uint8_t f)
{
    const double *P = A.p;
    const double p0 = P[o];
    const double pe = (f & fb_plus(a)) ? p0 : fma(A.fx[a][t + 1], P[o + s], A.gx[a][t + 1] * p0);
    const double pw = (f & fb_minus(a)) ? p0 : fma(A.fx[a][t], p0, A.gx[a][t] * P[o - s]);
    return (pe - pw) * A.dxinv[a][t];
}

// uTilde = u + dt grad p (1 - iblank), the VAN_KAN predictor of face_vel
// (IBM/CORE_FRAC_STEP_ROUTINES.F90:36-72), one thread per interior cell
__global__ void __launch_bounds__(TPB) k_vankan_tilde(StepArgs A)
{
    const Dims &d = A.d;
    const int n0 = d.m[0] - 1, n1 = d.m[1] - 1, n2 = d.m[2] - 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n0 * n1 * n2) return;
    int idx[3];
    cell_of((unsigned)t, (unsigned)n0, (unsigned)n1, idx[0], idx[1], idx[2]);
    const long long o = d.idx(idx[0], idx[1], idx[2]);
    const uint8_t f = A.fl[o];
    const bool fluid = !(f & FB_IB);
    for (int a = 0; a < 3; ++a) {
        const long long s = stride_of(d, a);
        const double u = A.vel[a][o];
        A.velo[a][o] = fluid ? fma(A.dt, cell_pgrad(A, a, idx[a], o, s, f), u) : u;
    }
}

// face_vel + rhs_poisson (IBM/CORE_POISSON.F90:155-163, 273-281).  A CTA of
// 32 x 8 threads owns a 32 x 8 tile of (i, j) and walks a chunk of k.  Each
// thread interpolates its cell's minus faces; the x plus face comes from the
// next lane (shuffle), the y plus face from the next row of the tile (shared
// memory, double-buffered by k parity), the z plus face is the next
// iteration's minus face (carried in a register).  The tile's last lane and
// last row interpolate their plus face themselves.  nlu0 = dtinv div(face)
// (1 - iblank); the block's share of sum nlu0 dx dy dz goes to partials.
// Threads past the grid's end run on clamped indices (in bounds) and store nothing.
template <bool VANKAN>
__global__ void __launch_bounds__(TPB) k_face_vel_rhs(StepArgs A, double *partials)
{
    const Dims &d = A.d;
    const int nxc = d.m[0] - 1, nyc = d.m[1] - 1, nzc = d.m[2] - 1;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i0 = blockIdx.x * 32 + tx + 1, j0 = blockIdx.y * 8 + ty + 1;
    const bool act = i0 <= nxc && j0 <= nyc;
    const int i = min(i0, nxc), j = min(j0, nyc);
    const int kc = (nzc + (int)gridDim.z - 1) / (int)gridDim.z;
    const int kb = 1 + (int)blockIdx.z * kc, ke = min(nzc, kb + kc - 1);
    const long long sx = d.sx, sxy = d.sxy;
    const double *Ux = VANKAN ? A.velo[0] : A.vel[0];
    const double *Uy = VANKAN ? A.velo[1] : A.vel[1];
    const double *Uz = VANKAN ? A.velo[2] : A.vel[2];
    const double dxi = A.dxinv[0][i], dyi = A.dxinv[1][j], dxdy = A.dx[0][i] * A.dx[1][j];
    __shared__ double sy[2][8][32];
    double acc = 0.0;
    double fzm = 0.0;
    if (kb <= ke) {
        const long long o = d.idx(i, j, kb);
        fzm = face_minus<VANKAN>(A, Uz, 2, kb, o, sxy, A.fl[o]);
    }
    for (int k = kb; k <= ke; ++k) {
        const long long o = d.idx(i, j, k);
        const uint8_t f = A.fl[o];
        // x
        const double fxm = face_minus<VANKAN>(A, Ux, 0, i, o, 1, f);
        const double xn = __shfl_down_sync(0xffffffffu, fxm, 1);
        double fxp;
        if (i == nxc) fxp = face_last<VANKAN>(A, Ux, 0, i, o, 1, f);
        else if (tx < 31) fxp = xn;
        else fxp = face_minus<VANKAN>(A, Ux, 0, i + 1, o + 1, 1, A.fl[o + 1]);
        // y
        const double fym = face_minus<VANKAN>(A, Uy, 1, j, o, sx, f);
        sy[k & 1][ty][tx] = fym;
        __syncthreads();
        double fyp;
        if (j == nyc) fyp = face_last<VANKAN>(A, Uy, 1, j, o, sx, f);
        else if (ty < 7) fyp = sy[k & 1][ty + 1][tx];
        else fyp = face_minus<VANKAN>(A, Uy, 1, j + 1, o + sx, sx, A.fl[o + sx]);
        // z
        double fzp;
        if (k == nzc) fzp = face_last<VANKAN>(A, Uz, 2, k, o, sxy, f);
        else fzp = face_minus<VANKAN>(A, Uz, 2, k + 1, o + sxy, sxy, A.fl[o + sxy]);
        double r = (fxp - fxm) * dxi;
        r = fma(fyp - fym, dyi, r);
        r = fma(fzp - fzm, A.dxinv[2][k], r);
        const double nl = (f & FB_IB) ? 0.0 : r * A.dtinv;
        if (act) {
            A.face[0][o] = fxm;
            if (i == nxc) A.face[0][o + 1] = fxp;
            A.face[1][o] = fym;
            if (j == nyc) A.face[1][o + sx] = fyp;
            A.face[2][o] = fzm;
            if (k == nzc) A.face[2][o + sxy] = fzp;
            A.nlu0[o] = nl;
            acc = fma(nl, dxdy * A.dx[2][k], acc);   // nlu0 dx dy dz
        }
        fzm = fzp;
    }
    const double tot = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = tot;
}

// correct_vel without the ghost-cell velocity interpolation
// (IBM/CORE_FRAC_STEP_ROUTINES.F90:272-366 cell centres, :381-441 faces,
// :446 GCM_set_face_vel_body): u -= dt grad pPrime (1 - iblank); each face
// takes face1 of its cell, then the plus mask of the previous cell and its own
// minus mask (the reference's overwrite order); the last face takes face2 of
// cell n and its plus mask; with GCM the faces of dead cells are zero.
__global__ void __launch_bounds__(TPB) k_correct_vel(StepArgs A)
{
    const Dims &d = A.d;
    const int n0 = d.m[0] - 1, n1 = d.m[1] - 1, n2 = d.m[2] - 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n0 * n1 * n2) return;
    int idx[3];
    cell_of((unsigned)t, (unsigned)n0, (unsigned)n1, idx[0], idx[1], idx[2]);
    const long long o = d.idx(idx[0], idx[1], idx[2]);
    const uint8_t f = A.fl[o];
    const bool fluid = !(f & FB_IB);
    const double *P = A.p;
    for (int a = 0; a < 3; ++a) {
        const long long s = stride_of(d, a);
        const int i = idx[a], n = d.m[a] - 1;
        const double u = A.vel[a][o];
        A.velo[a][o] = fluid ? fma(-A.dt, cell_pgrad(A, a, i, o, s, f), u) : u;
        double *F = A.face[a];
        const uint8_t fp = (i >= 2) ? A.fl[o - s] : (uint8_t)0;
        double v1;
        if (f & fb_minus(a)) v1 = bc_at(A.bc[a], o);
        else if (fp & fb_plus(a)) v1 = bc_at(A.bc[a], o - s);
        else v1 = fma(-A.dt, (P[o] - P[o - s]) * A.dxcinv[a][i], F[o]);
        if (A.gcm && (dead_cell(f) || dead_cell(fp))) v1 = 0.0;
        if (i == n) {
            double v2 = (f & fb_plus(a)) ? bc_at(A.bc[a], o)
                                         : fma(-A.dt, (P[o + s] - P[o]) * A.dxcinv[a][n + 1], F[o + s]);
            if (A.gcm && dead_cell(f)) v2 = 0.0;
            F[o + s] = v2;
        }
        F[o] = v1;
    }
}

__global__ void k_update_pressure(double *p, const double *pPrime, long long n, int van_kan)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = van_kan ? p[t] + pPrime[t] : pPrime[t];
}

// ---------------------------------------------------------------------------
// Outer boundary values, set_bc (IBM/CORE_SET_BC.F90:22-298).  The planes of
// the three axes are independent (each axis writes its own bc arrays and
// reads only u, v, w), so one launch covers them: one thread per plane point,
// the minus side (cell 1) before the plus side (cell n-1), the reference's
// order where the two are the same cell.  The ghost phase follows per axis
// in the reference's order x, y, z: each axis' ghost layers read cells that
// the previous axis wrote.
// ---------------------------------------------------------------------------
enum { BCT_ZERO_GRADIENT = 2, BCT_SYMMETRY = 4, BCT_SHEAR = 7 };

// boundary value of component c on side s (normal axis a) at cell o, plane point (i, j)
__device__ __forceinline__ double side_value(const SetBcArgs &A, int s, int a, int c, long long o, int i, int j)
{
    switch (A.type[s]) {
    case BCT_ZERO_GRADIENT: return A.vel[c][o];
    case BCT_SYMMETRY: return c == a ? 0.0 : A.vel[c][o];
    case BCT_SHEAR:   // the normal component scales with y(j)/yout (x and z sides) or x(i)/xout (y sides)
        if (c != a) return A.val[s][c];
        return a == 1 ? A.val[s][c] * A.xn[0][i] / A.xout : A.val[s][c] * A.xn[1][j] / A.yout;
    default: return A.val[s][c];   // Dirichlet; pulsatile, evaluated at the current time by the host
    }
}

// (p, q) plane point of the axis-a planes: the two transverse axes in index order
__device__ __forceinline__ void plane_axes(int a, int &b, int &c)
{
    b = (a == 0) ? 1 : 0;
    c = (a == 2) ? 1 : 2;
}

__global__ void __launch_bounds__(TPB) k_set_bc_planes(SetBcArgs A)
{
    const Dims &d = A.d;
    const long long P[3] = {(long long)(d.m[1] + 1) * (d.m[2] + 1), (long long)(d.m[0] + 1) * (d.m[2] + 1),
                            (long long)(d.m[0] + 1) * (d.m[1] + 1)};
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int a = 0;
    while (a < 3 && t >= P[a]) t -= P[a++];
    if (a == 3) return;
    int b, c;
    plane_axes(a, b, c);
    int ix[3];
    ix[b] = (int)(t % (d.m[b] + 1));
    ix[c] = (int)(t / (d.m[b] + 1));
    for (int side = 0; side < 2; ++side) {
        ix[a] = side == 0 ? 1 : d.m[a] - 1;
        const long long o = d.idx(ix[0], ix[1], ix[2]);
        const int s = 2 * a + side;
        for (int comp = 0; comp < 3; ++comp) A.bc[3 * comp + a][o] = side_value(A, s, a, comp, o, ix[0], ix[1]);
    }
}

// Boundary mass flux of enforce_global_mass_consv (IBM/CORE_SET_BC.F90:319-337):
// per fluid cell -bcxu dy dz on an ium face, +bcxu dy dz on an iup face, and
// likewise bcyv dx dz and bczw dx dy, summed in the reference's order within
// the cell; one partial sum per CTA.
__global__ void __launch_bounds__(TPB) k_bc_massflux(SetBcArgs A, double *partials)
{
    const Dims &d = A.d;
    const unsigned n0 = d.m[0] - 1, n1 = d.m[1] - 1;
    const unsigned n = n0 * n1 * (unsigned)(d.m[2] - 1);
    double acc = 0.0;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        cell_of(t, n0, n1, i, j, k);
        const long long o = d.idx(i, j, k);
        const uint8_t f = A.fl[o];
        if ((f & FB_IB) || !(f & 0xFC)) continue;
        const double dx = A.dx[0][i], dy = A.dx[1][j], dz = A.dx[2][k];
        const double bu = A.bc[0][o], bv = A.bc[4][o], bw = A.bc[8][o];
        double m = 0.0;
        if (f & fb_minus(0)) m = m - bu * dy * dz;
        if (f & fb_plus(0)) m = m + bu * dy * dz;
        if (f & fb_minus(1)) m = m - bv * dx * dz;
        if (f & fb_plus(1)) m = m + bv * dx * dz;
        if (f & fb_minus(2)) m = m - bw * dx * dy;
        if (f & fb_plus(2)) m = m + bw * dx * dy;
        acc += m;
    }
    const double tot = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

// enforce_global_mass_consv's corrections of axis AX (IBM/CORE_SET_BC.F90:352-371:
// the normal component on zero-gradient sides, correction_vel = -massflux /
// outflow_area), then set_outer_ghost_vel on that axis (IBM/CORE_SET_OUTER_GHOST.F90:
// 16-61): vel(0) = 2 bc(1) - vel(1), vel(n) = 2 bc(n-1) - vel(n-1) for u, v, w.
template <int AX>
__global__ void __launch_bounds__(TPB) k_outer_ghost_vel(SetBcArgs A, int mass_consv)
{
    const Dims &d = A.d;
    int b, c;
    plane_axes(AX, b, c);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)(d.m[b] + 1) * (d.m[c] + 1)) return;
    int ix[3];
    ix[b] = (int)(t % (d.m[b] + 1));
    ix[c] = (int)(t / (d.m[b] + 1));
    const int n = d.m[AX];
    const long long sa = stride_of(d, AX);
    ix[AX] = 0;
    const long long o0 = d.idx(ix[0], ix[1], ix[2]);
    const long long o1 = o0 + sa, on1 = o0 + (long long)(n - 1) * sa, on = o0 + (long long)n * sa;
    if (mass_consv) {
        const double corr = -A.sums[0] / A.outflow_area;
        double *bn = A.bc[4 * AX];   // bcxu, bcyv, bczw
        if (A.type[2 * AX] == BCT_ZERO_GRADIENT) bn[o1] = bn[o1] - corr;
        if (A.type[2 * AX + 1] == BCT_ZERO_GRADIENT) bn[on1] = bn[on1] + corr;
    }
    for (int comp = 0; comp < 3; ++comp) {
        double *v = A.vel[comp];
        const double *bcv = A.bc[3 * comp + AX];
        v[o0] = 2.0 * bcv[o1] - v[o1];
        v[on] = 2.0 * bcv[on1] - v[on1];
    }
}

// remove_rhs_adjust_bc then rhs_readjust_bc (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:90-252)
// for one interior cell: nl += sum a_f bc_f over its flagged faces with the
// current boundary values, then nl -= the same sum with the corrected values
// (the zero-gradient normal components of this cell, minus side then plus
// side, as the plane corrections form them).  a_f is the implicit diffusion
// coefficient with the constant reinv, -(0.5 dt reinv) x (dcinv dinv, or
// 2 dinv dinv on a flagged face), the z pair times (ndim - 2).  Cells without
// flagged faces add exact zeros and are skipped.
__global__ void __launch_bounds__(TPB) k_zg_rhs_terms(ZgArgs A)
{
    const Dims &d = A.d;
    const unsigned n0 = d.m[0] - 1, n1 = d.m[1] - 1, n2 = d.m[2] - 1;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n0 * n1 * n2) return;
    int ix[3];
    cell_of(t, n0, n1, ix[0], ix[1], ix[2]);
    const long long o = d.idx(ix[0], ix[1], ix[2]);
    const uint8_t f = A.fl[o];
    if (!(f & 0xFC)) return;
    const double corr = -A.sums[0] / A.outflow_area;
    double am[3], ap[3];
    for (int a = 0; a < 3; ++a) {
        const int i = ix[a];
        am[a] = (f & fb_minus(a)) ? A.cb[a][i] : A.cm[a][i];
        ap[a] = (f & fb_plus(a)) ? A.cb[a][i] : A.cp[a][i];
        am[a] = -A.hdr * am[a];
        ap[a] = -A.hdr * ap[a];
    }
    const double rnDim = A.three_d ? 1.0 : 0.0;
    am[2] = am[2] * rnDim;
    ap[2] = ap[2] * rnDim;
    const int ncells[3] = {(int)n0, (int)n1, (int)n2};
    for (int q = 0; q < 3; ++q) {
        if (!A.nl[q]) continue;   // nlw of a 2D run may be absent
        double b_old[3], b_new[3];
        for (int a = 0; a < 3; ++a) {
            b_old[a] = A.bc[3 * q + a][o];
            double b = b_old[a];
            if (q == a) {   // bcxu, bcyv, bczw: the zero-gradient corrections of this cell
                if (ix[a] == 1 && A.type[2 * a] == BCT_ZERO_GRADIENT) b = b - corr;
                if (ix[a] == ncells[a] && A.type[2 * a + 1] == BCT_ZERO_GRADIENT) b = b + corr;
            }
            b_new[a] = b;
        }
        double r = A.nl[q][o];
        for (int a = 0; a < 3; ++a) {
            if (f & fb_minus(a)) r = r + am[a] * b_old[a];
            if (f & fb_plus(a)) r = r + ap[a] * b_old[a];
        }
        for (int a = 0; a < 3; ++a) {
            if (f & fb_minus(a)) r = r - am[a] * b_new[a];
            if (f & fb_plus(a)) r = r - ap[a] * b_new[a];
        }
        A.nl[q][o] = r;
    }
}

// the plane corrections of GCM_enforce_global_mass_consv (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:60-79):
// one thread per plane point of all three axes, minus side then plus side
__global__ void __launch_bounds__(TPB) k_zg_planes(ZgArgs A)
{
    const Dims &d = A.d;
    const long long P[3] = {(long long)(d.m[1] + 1) * (d.m[2] + 1), (long long)(d.m[0] + 1) * (d.m[2] + 1),
                            (long long)(d.m[0] + 1) * (d.m[1] + 1)};
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int a = 0;
    while (a < 3 && t >= P[a]) t -= P[a++];
    if (a == 3) return;
    const bool lo = A.type[2 * a] == BCT_ZERO_GRADIENT, hi = A.type[2 * a + 1] == BCT_ZERO_GRADIENT;
    if (!lo && !hi) return;
    int b, c;
    plane_axes(a, b, c);
    int ix[3];
    ix[b] = (int)(t % (d.m[b] + 1));
    ix[c] = (int)(t / (d.m[b] + 1));
    const double corr = -A.sums[0] / A.outflow_area;
    double *bn = A.bc[4 * a];
    if (lo) {
        ix[a] = 1;
        const long long o = d.idx(ix[0], ix[1], ix[2]);
        bn[o] = bn[o] - corr;
    }
    if (hi) {
        ix[a] = d.m[a] - 1;
        const long long o = d.idx(ix[0], ix[1], ix[2]);
        bn[o] = bn[o] + corr;
    }
}

// ---------------------------------------------------------------------------
// Momentum right-hand side, rhs_advec_diff (IBM/CORE_RHS_AD.F90:13-75) with
// rhs_advec (:80-382, non-hybrid), rhs_loadAB (:385-430), rhs_diff (:433-530)
// and rhs_vankan (:550-585), one thread per interior cell and all three
// components (each step is local to the cell, so the reference's sequence of
// whole-array loops fuses).  FP64; mask products become selects and the
// diffusion coefficients come from per-axis tables holding the reference's
// products; the sums keep the reference's order.  In 2D the w component is
// left to rhs_vankan alone, as in the reference.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TPB) k_rhs_advec_diff(RhsAdArgs A)
{
    const Dims &d = A.d;
    const int n0 = d.m[0] - 1, n1 = d.m[1] - 1, n2 = d.m[2] - 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n0 * n1 * n2) return;
    int idx[3];
    cell_of((unsigned)t, (unsigned)n0, (unsigned)n1, idx[0], idx[1], idx[2]);
    const long long o = d.idx(idx[0], idx[1], idx[2]);
    const uint8_t f = A.fl[o];
    const int naxes = A.three_d ? 3 : 2;
    const int ncomp = A.three_d ? 3 : 2;
    // face viscosities and diffusion coefficients (shared by the components)
    double am[3] = {0.0, 0.0, 0.0}, ap[3] = {0.0, 0.0, 0.0}, ac[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < naxes; ++a) {
        const long long s = stride_of(d, a);
        const int i = idx[a];
        const bool mm = f & fb_minus(a), pp = f & fb_plus(a);
        const double *V = A.visc;
        // nuE / nuW: viscosity interpolated to the faces, bc*visc of this cell on flagged faces
        const double nuP = pp ? bc_at(A.bcvisc[a], o) : fma(A.fx[a][i + 1], V[o + s], A.gx[a][i + 1] * V[o]);
        const double nuM = mm ? bc_at(A.bcvisc[a], o) : fma(A.fx[a][i], V[o], A.gx[a][i] * V[o - s]);
        const double cmv = mm ? A.cb[a][i] : A.cm[a][i];
        const double cpv = pp ? A.cb[a][i] : A.cp[a][i];
        am[a] = cmv * nuM;
        ap[a] = cpv * nuP;
        ac[a] = -(am[a] + ap[a]);
    }
    for (int q = 0; q < ncomp; ++q) {
        const double *U = A.vel[q];
        const double uc = U[o];
        // rhs_advec
        double adv = 0.0;
        for (int a = 0; a < naxes; ++a) {
            const long long s = stride_of(d, a);
            const int i = idx[a];
            const bool mm = f & fb_minus(a), pp = f & fb_plus(a);
            const double *bc = A.bc[3 * q + a];
            const double ve = pp ? bc_at(bc, o) : fma(A.fx[a][i + 1], U[o + s], A.gx[a][i + 1] * uc);
            const double vw = mm ? bc_at(bc, o) : fma(A.fx[a][i], uc, A.gx[a][i] * U[o - s]);
            const double F0 = A.face[a][o], F1 = A.face[a][o + s];
            double term;
            if (A.hybrid) {
                // second-order upwind face values blended by alfa (IBM/CORE_RHS_AD.F90:150-382); the
                // reference's 0/1 mask products are selects here.  iumm / iupp mark the first and
                // last two cells of the axis (IBM/BOUNDARY_SET.F90:90-127), where the upwind value
                // falls back to the central one.
                const double *di = A.dxinv[a];
                const int nn = d.m[a], nc = nn - 1;
                const int imm = i - 2 > 0 ? i - 2 : 0, ipp = i + 2 < nn ? i + 2 : nn;
                const double em1 = (di[i - 1] + 2.0 * di[i]) / (di[i - 1] + di[i]);
                const double em2 = di[i] / (di[i - 1] + di[i]);
                const double ep1 = (di[ipp] + 2.0 * di[i + 1]) / (di[ipp] + di[i + 1]);
                // the x direction weights vel(ipp) with edxWeightp1, as the reference writes it
                const double ep2 = (a == 0) ? ep1 : di[i + 1] / (di[ipp] + di[i + 1]);
                const double wm1 = (di[imm] + 2.0 * di[i - 1]) / (di[imm] + di[i - 1]);
                const double wm2 = di[i - 1] / (di[imm] + di[i - 1]);
                const double wp1 = (di[i + 1] + 2.0 * di[i]) / (di[i + 1] + di[i]);
                const double wp2 = di[i] / (di[i + 1] + di[i]);
                const bool edge_m = (i <= 2), edge_p = (i >= nc - 1);
                const double Um = U[o - s], Up = U[o + s];
                const double e_from_m = edge_m ? ve : em1 * uc - em2 * Um;
                const double e_from_p = edge_p ? ve : ep1 * Up - ep2 * U[o + (long long)(ipp - i) * s];
                const double w_from_m = edge_m ? vw : wm1 * Um - wm2 * U[o - (long long)(i - imm) * s];
                const double w_from_p = edge_p ? vw : wp1 * uc - wp2 * Up;
                const double ve_up = pp ? bc_at(bc, o) : (signbit(F1) ? e_from_p : e_from_m);
                const double vw_up = mm ? bc_at(bc, o) : (signbit(F0) ? w_from_p : w_from_m);
                const double veh = (1.0 - A.alfa) * ve + A.alfa * ve_up;
                const double vwh = (1.0 - A.alfa) * vw + A.alfa * vw_up;
                term = (veh * F1 - vwh * F0) * A.dxinv[a][i];
            } else {
                term = (ve * F1 - vw * F0) * A.dxinv[a][i];
            }
            adv = (a == 0) ? term : adv + term;
        }
        // rhs_loadAB
        double nl;
        if (A.ab2) {
            const double ew = A.ew ? A.ew[o] : 1.5;
            const double old = A.nlold[q][o];
            nl = ew * adv - (ew - 1.0) * old;
            A.nlold[q][o] = adv;
        } else {
            nl = adv * 0.5;
        }
        // rhs_diff: amx W + acx V + apx E + amy S + acy V + apy N + amz B + acz V + apz F
        double diff = 0.0;
        bool first = true;
        for (int a = 0; a < 3; ++a) {
            if (a >= naxes) break;
            const long long s = stride_of(d, a);
            const bool mm = f & fb_minus(a), pp = f & fb_plus(a);
            const double *bc = A.bc[3 * q + a];
            const double vW = mm ? bc_at(bc, o) : U[o - s];
            const double vE = pp ? bc_at(bc, o) : U[o + s];
            diff = first ? am[a] * vW : fma(am[a], vW, diff);
            first = false;
            diff = fma(ac[a], uc, diff);
            diff = fma(ap[a], vE, diff);
        }
        A.nl[q][o] = fma(0.5 * A.dt, diff, fma(-A.dt, nl, uc));
    }
    if (A.vankan && !(f & FB_IB)) {
        const double *P = A.p;
        const double p0 = P[o];
        for (int a = 0; a < 3; ++a) {
            const long long s = stride_of(d, a);
            const int i = idx[a];
            const double pe = (f & fb_plus(a)) ? p0 : fma(A.fx[a][i + 1], P[o + s], A.gx[a][i + 1] * p0);
            const double pw = (f & fb_minus(a)) ? p0 : fma(A.fx[a][i], p0, A.gx[a][i] * P[o - s]);
            A.nl[a][o] = fma(-A.dt, (pe - pw) * A.dxinv[a][i], A.nl[a][o]);
        }
    }
}

// ---------------------------------------------------------------------------
// Implicit momentum solve (solve_ad, LSOR branch; IBM/CORE_SOLVE_AD.F90:12-907,
// IBM/CORE_SET_SOLVERS.F90:20-95).  The row of a cell is fixed during the
// iteration, so k_ad_coef forms it once per call: the implicit diffusion
// coefficients of set_solve_ad (-(dt/2 nu_face) times the metric products of
// the tables cm / cp / cb) and the Crank-Nicolson convective terms, masked as
// the sweeps and the residual use them.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TPB) k_ad_coef(AdCoefArgs A)
{
    const Dims &d = A.d;
    const int n0 = d.m[0] - 1, n1 = d.m[1] - 1, n2 = d.m[2] - 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n0 * n1 * n2) return;
    int idx[3];
    cell_of((unsigned)t, (unsigned)n0, (unsigned)n1, idx[0], idx[1], idx[2]);
    const long long o = d.idx(idx[0], idx[1], idx[2]);
    const uint8_t f = A.fl[o];
    double acs = 0.0;
    for (int a = 0; a < 3; ++a) {
        const long long s = stride_of(d, a);
        const int i = idx[a];
        const bool mm = f & fb_minus(a), pp = f & fb_plus(a);
        const double *V = A.visc;
        const double nuP = pp ? bc_at(A.bcvisc[a], o) : fma(A.fx[a][i + 1], V[o + s], A.gx[a][i + 1] * V[o]);
        const double nuM = mm ? bc_at(A.bcvisc[a], o) : fma(A.fx[a][i], V[o], A.gx[a][i] * V[o - s]);
        const double rn = (a == 2 && !A.three_d) ? 0.0 : 1.0;
        double am = -(0.5 * A.dt * nuM) * (mm ? A.cb[a][i] : A.cm[a][i]) * rn;
        double ap = -(0.5 * A.dt * nuP) * (pp ? A.cb[a][i] : A.cp[a][i]) * rn;
        double ac = -(am + ap);
        const double F0 = A.face[a][o], F1 = A.face[a][o + s], di = A.dxinv[a][i];
        am = am - A.half_dt * F0 * A.gx[a][i] * di;
        ap = ap + A.half_dt * F1 * A.fx[a][i + 1] * di;
        const double t1 = mm ? 0.0 : A.fx[a][i], t2 = pp ? 0.0 : A.gx[a][i + 1];
        ac = ac + A.half_dt * (F1 * t2 - F0 * t1) * di;
        A.co[2 * a][o] = mm ? 0.0 : am;
        A.co[2 * a + 1][o] = pp ? 0.0 : ap;
        acs = (a == 0) ? ac : acs + ac;
    }
    A.co[6][o] = acs;
}

// rhs_adjust_bc: the coefficients of rhs_adjust_bc differ from the row's in
// the convective weights of flagged faces (tmp1 = (1 - fx) (1 - m) + m,
// tmp2 = fx (1 - p) + p), so they are formed here again.
__global__ void __launch_bounds__(TPB) k_rhs_adjust_bc(AdCoefArgs A, const double *b0, const double *b1,
                                                       const double *b2, const double *b3, const double *b4,
                                                       const double *b5, const double *b6, const double *b7,
                                                       const double *b8, double *nl0, double *nl1, double *nl2)
{
    const Dims &d = A.d;
    const int n0 = d.m[0] - 1, n1 = d.m[1] - 1, n2 = d.m[2] - 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n0 * n1 * n2) return;
    int idx[3];
    cell_of((unsigned)t, (unsigned)n0, (unsigned)n1, idx[0], idx[1], idx[2]);
    const long long o = d.idx(idx[0], idx[1], idx[2]);
    const uint8_t f = A.fl[o];
    double md[3], pd[3];
    for (int a = 0; a < 3; ++a) {
        const long long s = stride_of(d, a);
        const int i = idx[a];
        const bool mm = f & fb_minus(a), pp = f & fb_plus(a);
        const double *V = A.visc;
        const double nuP = pp ? bc_at(A.bcvisc[a], o) : fma(A.fx[a][i + 1], V[o + s], A.gx[a][i + 1] * V[o]);
        const double nuM = mm ? bc_at(A.bcvisc[a], o) : fma(A.fx[a][i], V[o], A.gx[a][i] * V[o - s]);
        const double rn = (a == 2 && !A.three_d) ? 0.0 : 1.0;
        double am = -(0.5 * A.dt * nuM) * (mm ? A.cb[a][i] : A.cm[a][i]) * rn;
        double ap = -(0.5 * A.dt * nuP) * (pp ? A.cb[a][i] : A.cp[a][i]) * rn;
        const double t1 = mm ? 1.0 : A.gx[a][i], t2 = pp ? 1.0 : A.fx[a][i + 1];
        md[a] = am - A.half_dt * A.face[a][o] * t1 * A.dxinv[a][i];
        pd[a] = ap + A.half_dt * A.face[a][o + s] * t2 * A.dxinv[a][i];
    }
    const double *bc[9] = {b0, b1, b2, b3, b4, b5, b6, b7, b8};
    double *nl[3] = {nl0, nl1, nl2};
    for (int q = 0; q < 3; ++q) {
        if (!nl[q]) continue;
        double v = nl[q][o];
        for (int a = 0; a < 3; ++a) {
            const double *b = bc[3 * q + a];
            if (f & fb_minus(a)) v = fma(-md[a], bc_at(b, o), v);
            if (f & fb_plus(a)) v = fma(-pd[a], bc_at(b, o), v);
        }
        nl[q][o] = v;
    }
}

// One colour of the line sweep along DIR (itsolv_ad_x/y/z): one thread per
// line, lines of colour (q1 + q2) mod 2 over the transverse indices; the
// row is assembled as the reference does (identity rows for blanked cells,
// the ghost's own value kept) and solved by the Thomas algorithm of tdma
// (IBM/CORE_TDMA.F90:10-34) with gam in a scratch array.
template <int DIR>
__global__ void __launch_bounds__(TPB) k_ad_line(AdCoefArgs A, double *var, const double *r, double *gam, int colour)
{
    const Dims &d = A.d;
    using X = Axes<DIR>;
    const int nb = d.m[X::b] - 1, nc = d.m[X::c] - 1, L = d.m[X::a] - 1;
    const long long sa = stride_of(d, X::a), sb = stride_of(d, X::b), sc = stride_of(d, X::c);
    const int hb = (nb + 1) >> 1;
    const long long tl = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tl >= (long long)hb * nc) return;
    const int q = 1 + (int)(tl / hb);
    const int p0 = (((1 + q) & 1) == colour) ? 1 : 2;
    const int p = p0 + 2 * (int)(tl - (long long)(q - 1) * hb);
    if (p > nb) return;
    const long long base = p * sb + q * sc;
    // the transverse axes in the reference's order of the right-hand side terms
    const int t1 = X::b < X::c ? X::b : X::c, t2 = X::b < X::c ? X::c : X::b;
    const long long s1 = stride_of(d, t1), s2 = stride_of(d, t2);
    double binv = 0.0, uprev = 0.0, cprev = 0.0;
    for (int i = 1; i <= L; ++i) {
        const long long o = base + i * sa;
        const uint8_t f = A.fl[o];
        const double rib = (f & FB_IB) ? 0.0 : 1.0;
        double rhs;
        if (DIR == 2) {   // z-lines subtract term by term, y before x (IBM/CORE_SOLVE_AD.F90:678-681)
            rhs = r[o] - var[o - s2] * A.co[2 * t2][o] - var[o + s2] * A.co[2 * t2 + 1][o]
                  - var[o - s1] * A.co[2 * t1][o] - var[o + s1] * A.co[2 * t1 + 1][o];
        } else {          // x- and y-lines subtract one sum, lower axis first
            const double sm = var[o - s1] * A.co[2 * t1][o] + var[o + s1] * A.co[2 * t1 + 1][o]
                              + var[o - s2] * A.co[2 * t2][o] + var[o + s2] * A.co[2 * t2 + 1][o];
            rhs = r[o] - sm;
        }
        const double aa = A.co[2 * DIR][o] * rib, cc = A.co[2 * DIR + 1][o] * rib;
        const double bb = 1.0 + A.co[6][o] * rib;
        const double dd = rhs * rib + ((f & FB_GM) ? var[o] : 0.0);
        if (i == 1) {
            binv = 1.0 / bb;
            uprev = dd * binv;
        } else {
            const double g = cprev * binv;
            gam[o] = g;
            binv = 1.0 / (bb - aa * g);
            uprev = (dd - aa * uprev) * binv;
        }
        var[o] = uprev;   // the forward solution; the row's own value was read above
        cprev = cc;
    }
    for (int i = L - 1; i >= 1; --i) {
        const long long o = base + i * sa;
        var[o] = var[o] - gam[o + sa] * var[o + sa];
    }
}

// The same colour sweep with one warp per line (lines of 17..256 cells): the
// rows are assembled exactly as k_ad_line assembles them, staged in shared
// memory (x-lines: one warp along the line; y- and z-lines: 8 same-colour
// lines side by side, so the loads coalesce), and solved by the partition
// solver of the pressure smoother.  A CTA owns WP_LINES lines; each line's
// solution overwrites its own staged rows.
template <int DIR, int S, bool FULL>
__global__ void __launch_bounds__(256) k_ad_line_wp(AdCoefArgs A, double *var, const double *r, int colour)
{
    using X = Axes<DIR>;
    extern __shared__ unsigned char smem_raw[];
    constexpr int RP4 = wp_rows_pitch<S>();
    WpRow<double> *srow = reinterpret_cast<WpRow<double> *>(smem_raw);
    double *sx = reinterpret_cast<double *>(smem_raw);   // line g's solution: sx + 4 g RP4, row r at r + r/S
    const Dims &d = A.d;
    const int nb = d.m[X::b] - 1, nc = d.m[X::c] - 1;
    const int L = FULL ? 32 * S : d.m[X::a] - 1;
    const int hb = (nb + 1) >> 1;
    const int nlines = hb * nc;
    const int sa_ = (int)stride_of(d, X::a), sb_ = (int)stride_of(d, X::b), sc_ = (int)stride_of(d, X::c);
    // the transverse axes in the reference's order of the right-hand side terms
    constexpr int t1 = X::b < X::c ? X::b : X::c, t2 = X::b < X::c ? X::c : X::b;
    const int s1 = (t1 == X::b) ? sb_ : sc_, s2 = (t2 == X::b) ? sb_ : sc_;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    auto line_pq = [&](int g, int &p, int &q) -> bool {
        const int t = (int)blockIdx.x * WP_LINES + g;
        if (t >= nlines) return false;
        const int tq = t / hb;
        q = 1 + tq;
        const int p0 = (((1 + q) & 1) == colour) ? 1 : 2;
        p = p0 + 2 * (t - tq * hb);
        return p <= nb;
    };
    const int gs = (DIR == 0) ? warp : (tid & (WP_LINES - 1));
    const int rr = (DIR == 0) ? lane : (tid >> 3);
    int ps = 1, qs = 1;
    const bool oks = line_pq(gs, ps, qs);
    const int base = ps * sb_ + qs * sc_;
    if (oks) {
#pragma unroll 2
        for (int q0 = 0; q0 < S; ++q0) {
            const int rw = q0 * 32 + rr;
            if (rw >= L) break;
            const int o = base + (rw + 1) * sa_;
            const uint8_t f = A.fl[o];
            const double rib = (f & FB_IB) ? 0.0 : 1.0;
            double rhs;
            if (DIR == 2) {   // z-lines subtract term by term, y before x (IBM/CORE_SOLVE_AD.F90:678-681)
                rhs = r[o] - var[o - s2] * A.co[2 * t2][o] - var[o + s2] * A.co[2 * t2 + 1][o]
                      - var[o - s1] * A.co[2 * t1][o] - var[o + s1] * A.co[2 * t1 + 1][o];
            } else {          // x- and y-lines subtract one sum, lower axis first
                const double sm = var[o - s1] * A.co[2 * t1][o] + var[o + s1] * A.co[2 * t1 + 1][o]
                                  + var[o - s2] * A.co[2 * t2][o] + var[o + s2] * A.co[2 * t2 + 1][o];
                rhs = r[o] - sm;
            }
            WpRow<double> w;
            w.a = (rw == 0) ? 0.0 : A.co[2 * DIR][o] * rib;            // tdma ignores a(1) ...
            w.c = (rw == L - 1) ? 0.0 : A.co[2 * DIR + 1][o] * rib;    // ... and c(n)
            w.b = 1.0 + A.co[6][o] * rib;
            w.d = rhs * rib + ((f & FB_GM) ? var[o] : 0.0);
            srow[gs * RP4 + rw + rw / S] = w;
        }
    }
    __syncthreads();
    {
        int p, q;
        const bool valid = line_pq(warp, p, q);
        wp_solve_line<double, S>(srow + warp * RP4, sx + 4 * warp * RP4, L, valid, lane);
    }
    __syncthreads();
    if (oks) {
#pragma unroll 4
        for (int q0 = 0; q0 < S; ++q0) {
            const int rw = q0 * 32 + rr;
            if (rw >= L) break;
            var[base + (rw + 1) * sa_] = sx[4 * gs * RP4 + rw + rw / S];
        }
    }
}

template <int S>
size_t ad_wp_smem() { return sizeof(WpRow<double>) * (size_t)WP_LINES * wp_rows_pitch<S>(); }

template <int DIR, int S>
void launch_ad_wp_one(const AdCoefArgs &c, double *var, const double *r, int colour, long long lines, cudaStream_t s)
{
    const unsigned blocks = (unsigned)((lines + WP_LINES - 1) / WP_LINES);
    if (c.d.m[DIR] - 1 == 32 * S)
        k_ad_line_wp<DIR, S, true><<<blocks, 256, ad_wp_smem<S>(), s>>>(c, var, r, colour);
    else
        k_ad_line_wp<DIR, S, false><<<blocks, 256, ad_wp_smem<S>(), s>>>(c, var, r, colour);
}

// lines of 17..256 cells take the warp-per-line kernel; shorter ones one
// thread per line, longer ones too (no register room for S = 16 in FP64)
template <int DIR>
bool launch_ad_wp_dir(const AdCoefArgs &c, double *var, const double *r, int colour, int L, long long lines,
                      cudaStream_t s)
{
    if (L <= 16 || L > 256) return false;
    if (L <= 32) launch_ad_wp_one<DIR, 1>(c, var, r, colour, lines, s);
    else if (L <= 64) launch_ad_wp_one<DIR, 2>(c, var, r, colour, lines, s);
    else if (L <= 128) launch_ad_wp_one<DIR, 4>(c, var, r, colour, lines, s);
    else launch_ad_wp_one<DIR, 8>(c, var, r, colour, lines, s);
    return true;
}

template <int DIR, int S>
cudaError_t ad_wp_attr()
{
    const int b = (int)ad_wp_smem<S>();
    cudaError_t e = cudaFuncSetAttribute(k_ad_line_wp<DIR, S, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_ad_line_wp<DIR, S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
}

template <int DIR>
cudaError_t ad_wp_attr_dir()
{
    cudaError_t e;
    if ((e = ad_wp_attr<DIR, 1>()) != cudaSuccess) return e;
    if ((e = ad_wp_attr<DIR, 2>()) != cudaSuccess) return e;
    if ((e = ad_wp_attr<DIR, 4>()) != cudaSuccess) return e;
    return ad_wp_attr<DIR, 8>();
}

// calc_residual_ad of up to three components in one pass: the seven row
// coefficients of a cell are read once and applied to u, v and w (each
// component by the rows of calc_residual_ad, IBM/CORE_SOLVE_AD.F90), max |res| over all.
template <int NC>
__global__ void __launch_bounds__(TPB) k_ad_residual_n(AdCoefArgs A, const double *v0, const double *v1,
                                                       const double *v2, const double *r0, const double *r1,
                                                       const double *r2, unsigned long long *maxbits)
{
    const Dims &d = A.d;
    const int n0 = d.m[0] - 1, n1 = d.m[1] - 1, n2 = d.m[2] - 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double res = 0.0;
    if (t < (long long)n0 * n1 * n2) {
        int idx[3];
        cell_of((unsigned)t, (unsigned)n0, (unsigned)n1, idx[0], idx[1], idx[2]);
        const long long o = d.idx(idx[0], idx[1], idx[2]);
        if (!(A.fl[o] & FB_IB)) {
            double cm[3], cp[3];
            for (int a = 0; a < 3; ++a) { cm[a] = A.co[2 * a][o]; cp[a] = A.co[2 * a + 1][o]; }
            const double diag = 1.0 + A.co[6][o];
            const double *vv[3] = {v0, v1, v2}, *rr[3] = {r0, r1, r2};
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const double *var = vv[q];
                double v = rr[q][o] - var[o] * diag;
                for (int a = 0; a < 3; ++a) {
                    const long long s = stride_of(d, a);
                    v = v - var[o - s] * cm[a];
                    v = v - var[o + s] * cp[a];
                }
                res = fmax(res, fabs(v));
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) res = fmax(res, __shfl_xor_sync(0xffffffffu, res, off));
    if ((threadIdx.x & 31) == 0 && res > 0.0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(res));
}

// zero the non-interior part of a full (0:nx+1,0:ny+1,0:nz+1) array: planes
// k = 0, nz, nz+1; then rows j = 0, ny, ny+1 of k = 1..nzc; then cells
// i = 0, nx, nx+1 of the interior rows (the interior is written elsewhere)
__global__ void k_zero_shell(double *a, Dims d)
{
    const int nx = d.m[0], ny = d.m[1], nz = d.m[2];
    const long long sx = d.sx, sxy = d.sxy;
    const long long segA = 3 * sxy, segB = 3 * sx * (nz - 1), segC = 3LL * (ny - 1) * (nz - 1);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < segA + segB + segC;
         t += (long long)gridDim.x * blockDim.x) {
        long long o;
        if (t < segA) {
            const long long q = t / sxy, r = t - q * sxy;
            o = (q == 0 ? 0 : (q == 1 ? nz : nz + 1)) * sxy + r;
        } else if (t < segA + segB) {
            const long long u = t - segA, q = u / (sx * (nz - 1)), r = u - q * (sx * (nz - 1));
            const long long k = 1 + r / sx, i = r - (k - 1) * sx;
            o = i + sx * (q == 0 ? 0 : (q == 1 ? ny : ny + 1)) + sxy * k;
        } else {
            const long long u = t - segA - segB, q = u / ((long long)(ny - 1) * (nz - 1));
            const long long r = u - q * ((long long)(ny - 1) * (nz - 1));
            const long long k = 1 + r / (ny - 1), j = 1 + r % (ny - 1);
            o = (q == 0 ? 0 : (q == 1 ? nx : nx + 1)) + sx * j + sxy * k;
        }
        a[o] = 0.0;
    }
}

} // namespace

void launch_face_vel_rhs(const StepArgs &a, bool van_kan, double *partials, int cap, double *sums, cudaStream_t s)
{
    const int nxc = a.d.m[0] - 1, nyc = a.d.m[1] - 1, nzc = a.d.m[2] - 1;
    const long long n = (long long)nxc * nyc * nzc;
    // nlu0 = 0 outside the interior (the reference zeroes the whole array first)
    const long long nshell = 3 * a.d.sxy + 3 * a.d.sx * (nzc) + 3LL * nyc * nzc;
    k_zero_shell<<<nblk(nshell), TPB, 0, s>>>(a.nlu0, a.d);
    if (van_kan) k_vankan_tilde<<<nblk(n), TPB, 0, s>>>(a);
    // 32 x 8 tiles of (i, j); k split into chunks until the grid covers the
    // SMs several times over (at most cap blocks: one partial sum each)
    const int bx = (nxc + 31) / 32, by = (nyc + 7) / 8;
    int bz = std::max(1, std::min(nzc, (8 * 152 + bx * by - 1) / (bx * by)));
    bz = std::max(1, std::min(bz, cap / (bx * by)));
    const dim3 grid(bx, by, bz);
    if (van_kan) k_face_vel_rhs<true><<<grid, TPB, 0, s>>>(a, partials);
    else k_face_vel_rhs<false><<<grid, TPB, 0, s>>>(a, partials);
    k_sum_final<<<1, 1024, 0, s>>>(partials, bx * by * bz, 1, sums);
}

void launch_rhs_advec_diff(const RhsAdArgs &a, cudaStream_t s)
{
    const long long n = (long long)(a.d.m[0] - 1) * (a.d.m[1] - 1) * (a.d.m[2] - 1);
    k_rhs_advec_diff<<<nblk(n), TPB, 0, s>>>(a);
}

void launch_ad_coef(const AdCoefArgs &a, cudaStream_t s)
{
    const long long n = (long long)(a.d.m[0] - 1) * (a.d.m[1] - 1) * (a.d.m[2] - 1);
    k_ad_coef<<<nblk(n), TPB, 0, s>>>(a);
}

void launch_rhs_adjust_bc(const AdCoefArgs &c, const double *const bc[9], double *const nl[3], cudaStream_t s)
{
    const long long n = (long long)(c.d.m[0] - 1) * (c.d.m[1] - 1) * (c.d.m[2] - 1);
    k_rhs_adjust_bc<<<nblk(n), TPB, 0, s>>>(c, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], bc[6], bc[7], bc[8], nl[0],
                                            nl[1], nl[2]);
}

cudaError_t init_ad_line_kernels()
{
    cudaError_t e;
    if ((e = ad_wp_attr_dir<0>()) != cudaSuccess) return e;
    if ((e = ad_wp_attr_dir<1>()) != cudaSuccess) return e;
    return ad_wp_attr_dir<2>();
}

void launch_ad_line(int dir, int colour, const AdCoefArgs &c, double *var, const double *r, double *gam,
                    cudaStream_t s)
{
    // the transverse axes of Axes<dir>: lines of one colour = ceil(nb / 2) x nc
    const int b = (dir == 0) ? 1 : 0, cc = (dir == 2) ? 1 : 2;
    const long long lines = (long long)((c.d.m[b] - 1 + 1) / 2) * (c.d.m[cc] - 1);
    const int L = c.d.m[dir] - 1;
    if (dir == 0 ? launch_ad_wp_dir<0>(c, var, r, colour, L, lines, s)
        : dir == 1 ? launch_ad_wp_dir<1>(c, var, r, colour, L, lines, s)
                   : launch_ad_wp_dir<2>(c, var, r, colour, L, lines, s))
        return;
    if (dir == 0) k_ad_line<0><<<nblk(lines), TPB, 0, s>>>(c, var, r, gam, colour);
    else if (dir == 1) k_ad_line<1><<<nblk(lines), TPB, 0, s>>>(c, var, r, gam, colour);
    else k_ad_line<2><<<nblk(lines), TPB, 0, s>>>(c, var, r, gam, colour);
}

void launch_ad_residual_all(const AdCoefArgs &c, double *const var[3], const double *const r[3], int ncomp,
                            unsigned long long *maxbits, cudaStream_t s)
{
    const long long n = (long long)(c.d.m[0] - 1) * (c.d.m[1] - 1) * (c.d.m[2] - 1);
    if (ncomp == 3)
        k_ad_residual_n<3><<<nblk(n), TPB, 0, s>>>(c, var[0], var[1], var[2], r[0], r[1], r[2], maxbits);
    else
        k_ad_residual_n<2><<<nblk(n), TPB, 0, s>>>(c, var[0], var[1], nullptr, r[0], r[1], nullptr, maxbits);
}

void launch_correct_vel(const StepArgs &a, cudaStream_t s)
{
    const long long n = (long long)(a.d.m[0] - 1) * (a.d.m[1] - 1) * (a.d.m[2] - 1);
    k_correct_vel<<<nblk(n), TPB, 0, s>>>(a);
}

void launch_update_pressure(double *p, const double *pPrime, long long n, bool van_kan, cudaStream_t s)
{
    k_update_pressure<<<nblk(n), TPB, 0, s>>>(p, pPrime, n, van_kan ? 1 : 0);
}

void launch_set_bc_planes(const SetBcArgs &a, cudaStream_t s)
{
    const long long m0 = a.d.m[0] + 1, m1 = a.d.m[1] + 1, m2 = a.d.m[2] + 1;
    k_set_bc_planes<<<nblk(m1 * m2 + m0 * m2 + m0 * m1), TPB, 0, s>>>(a);
}

void launch_bc_massflux(const SetBcArgs &a, double *partials, int cap, double *sums, cudaStream_t s)
{
    const long long n = (long long)(a.d.m[0] - 1) * (a.d.m[1] - 1) * (a.d.m[2] - 1);
    const int nb = std::max(1, std::min({nblk(n), 8 * 152, cap}));
    k_bc_massflux<<<nb, TPB, 0, s>>>(a, partials);
    k_sum_final<<<1, 1024, 0, s>>>(partials, nb, 1, sums);
}

void launch_outer_ghost_vel(const SetBcArgs &a, int axis, bool mass_consv, cudaStream_t s)
{
    const int b = (axis == 0) ? 1 : 0, c = (axis == 2) ? 1 : 2;
    const int nb = nblk((long long)(a.d.m[b] + 1) * (a.d.m[c] + 1));
    if (axis == 0) k_outer_ghost_vel<0><<<nb, TPB, 0, s>>>(a, mass_consv ? 1 : 0);
    else if (axis == 1) k_outer_ghost_vel<1><<<nb, TPB, 0, s>>>(a, mass_consv ? 1 : 0);
    else k_outer_ghost_vel<2><<<nb, TPB, 0, s>>>(a, mass_consv ? 1 : 0);
}

void launch_zg_rhs_terms(const ZgArgs &a, cudaStream_t s)
{
    const long long n = (long long)(a.d.m[0] - 1) * (a.d.m[1] - 1) * (a.d.m[2] - 1);
    k_zg_rhs_terms<<<nblk(n), TPB, 0, s>>>(a);
}

void launch_zg_planes(const ZgArgs &a, cudaStream_t s)
{
    const long long m0 = a.d.m[0] + 1, m1 = a.d.m[1] + 1, m2 = a.d.m[2] + 1;
    k_zg_planes<<<nblk(m1 * m2 + m0 * m2 + m0 * m1), TPB, 0, s>>>(a);
}
} // namespace fsimg
