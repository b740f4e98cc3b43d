// Host side of the GB300 pressure-Poisson multigrid: hierarchy construction
// (MG_initial, IBM/CORE_MG.F90:31-278), device setup of flags, line factors
// and the ghost gather list, the V/W/F schedule of MG_Solver
// (IBM/CORE_MG.F90:281-527, 1239-1663) and the solve_poisson outer loop
// (IBM/CORE_POISSON.F90:493-676), behind the C ABI of include/fsi_mg.h.
//
// Level 1 of every cycle lives in the caller's full layout (0:nx+1)^3 so a
// device-resident pPrime/nlu0 is used in place; coarse levels are dense
// (0:m+1) arrays.  Everything runs on one stream owned by the handle; the
// fixed schedule of one outer iteration is captured once as a CUDA graph.
#include "mg_context.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

using namespace fsimg;

namespace fsimg {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

} // namespace fsimg

namespace {

// ------------------------------------------------------------- MG_initial --
int auto_levels(int cells)
{
    const int nCoarseGrids = 4, MG_LEVEL_MAX = 10;
    int ii = cells, nLevel;
    for (nLevel = 1; nLevel <= MG_LEVEL_MAX; ++nLevel) {
        ii = ii / 2;
        if (ii >= nCoarseGrids) continue;
        break;
    }
    return std::min(nLevel, MG_LEVEL_MAX);
}

void mg_initial(Ctx &c)
{
    const int N[3] = {c.nx, c.ny, c.nz};
    for (int d = 0; d < 3; ++d) {
        const int cells = N[d] - 1;
        int nl = c.p.mgLevels[d];
        if (nl == 0) nl = auto_levels(cells);
        if (d == 2 && c.p.ndim == 2) nl = 1;
        c.nlev[d] = nl;
        c.mgrid[d].assign(nl + 2, 0);
        c.mgrid[d][1] = cells;
        for (int l = 2; l <= nl; ++l) {
            int m = c.mgrid[d][l - 1];
            c.mgrid[d][l] = (m % 2 == 0) ? m / 2 : (m - 1) / 2;
        }
        const size_t len = N[d] + 2;
        auto mk = [&](std::vector<std::vector<double>> &a) { a.assign(nl + 1, std::vector<double>(len, 0.0)); };
        mk(c.xMG[d]); mk(c.xcMG[d]); mk(c.dxMG[d]); mk(c.dxinvMG[d]); mk(c.dxcMG[d]); mk(c.dxcinvMG[d]);
        for (int i = 0; i <= N[d]; ++i) {   // IBM/CORE_MG.F90:148-176
            c.dxcMG[d][1][i] = c.dxc[d][i];
            c.dxMG[d][1][i] = c.dx[d][i];
            c.dxcinvMG[d][1][i] = c.dxcinv[d][i];
            c.dxinvMG[d][1][i] = c.dxinv[d][i];
            c.xcMG[d][1][i] = c.xc[d][i];
        }
        for (int i = 0; i <= N[d] + 1; ++i) c.xMG[d][1][i] = c.x[d][i];
        for (int l = 2; l <= nl; ++l) {     // IBM/CORE_MG.F90:186-266
            const int m = c.mgrid[d][l];
            auto &X = c.xMG[d][l];
            for (int i = 1; i <= m + 1; ++i) X[i] = c.xMG[d][l - 1][2 * i - 1];
            X[0] = -X[2];
            X[m + 2] = 2.0 * X[m + 1] - X[m];
            for (int i = 0; i <= m + 1; ++i) {
                c.dxMG[d][l][i] = X[i + 1] - X[i];
                c.dxinvMG[d][l][i] = 1.0 / c.dxMG[d][l][i];
            }
            for (int i = 0; i <= m + 1; ++i) c.xcMG[d][l][i] = 0.5 * (X[i] + X[i + 1]);
            for (int i = 1; i <= m + 1; ++i) {
                c.dxcMG[d][l][i] = c.xcMG[d][l][i] - c.xcMG[d][l][i - 1];
                c.dxcinvMG[d][l][i] = 1.0 / c.dxcMG[d][l][i];
            }
        }
    }
}

// -------------------------------------------------------------- helpers ----
Dims full_dims(const Ctx &c)
{
    Dims d;
    d.m[0] = c.nx; d.m[1] = c.ny; d.m[2] = c.nz;
    d.sx = c.nx + 2;
    d.sxy = (long long)(c.nx + 2) * (c.ny + 2);
    return d;
}

Dims dense_dims(int m0, int m1, int m2)
{
    Dims d;
    d.m[0] = m0; d.m[1] = m1; d.m[2] = m2;
    d.sx = m0 + 1;
    d.sxy = (long long)(m0 + 1) * (m1 + 1);
    return d;
}

// 1D face coefficients of axis a at metric level lv for an array whose upper bound
// along a is m; Dirichlet doubling folded in at the boundary cells (flag -1).
int build_coef(Ctx &c, Level &L, int a, int lv, int m, bool dir_lo, bool dir_hi)
{
    std::vector<double> cm(m + 2, 0.0), cp(m + 2, 0.0);
    const bool twoD_z = (a == 2 && c.p.ndim == 2);
    for (int i = 1; i <= m - 1; ++i) {
        if (twoD_z) continue;
        cm[i] = c.dxcinvMG[a][lv][i] * c.dxinvMG[a][lv][i];
        cp[i] = c.dxcinvMG[a][lv][i + 1] * c.dxinvMG[a][lv][i];
    }
    if (!twoD_z) {
        if (dir_lo) cm[1] = cm[1] * 2.0;
        if (dir_hi) cp[m - 1] = cp[m - 1] * 2.0;
    }
    std::vector<float> cmf(cm.begin(), cm.end()), cpf(cp.begin(), cp.end());
    if (!L.cm64[a]) {   // sizes are fixed by the grid: allocate on the first set_geometry
        TRY(c.alloc(&L.cm64[a], cm.size()));
        TRY(c.alloc(&L.cp64[a], cp.size()));
        TRY(c.alloc(&L.cm32[a], cm.size()));
        TRY(c.alloc(&L.cp32[a], cp.size()));
    }
    CK(cudaMemcpyAsync(L.cm64[a], cm.data(), cm.size() * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(L.cp64[a], cp.data(), cp.size() * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(L.cm32[a], cmf.data(), cmf.size() * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(L.cp32[a], cpf.data(), cpf.size() * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

template <typename T> Coef<T> coef_of(const Level &L);
template <> Coef<double> coef_of<double>(const Level &L)
{
    Coef<double> k;
    for (int a = 0; a < 3; ++a) { k.cm[a] = L.cm64[a]; k.cp[a] = L.cp64[a]; }
    return k;
}
template <> Coef<float> coef_of<float>(const Level &L)
{
    Coef<float> k;
    for (int a = 0; a < 3; ++a) { k.cm[a] = L.cm32[a]; k.cp[a] = L.cp32[a]; }
    return k;
}

// allocate the per-level device state common to level 1 and coarse levels
int alloc_level(Ctx &c, Level &L, bool fields)
{
    const long long n = L.d.count();
    TRY(c.alloc(&L.fl, n));
    for (int a = 0; a < c.nd; ++a) {
        TRY(c.alloc(&L.binv64[a], n)); TRY(c.alloc(&L.gam64[a], n));
        TRY(c.alloc(&L.binv32[a], n)); TRY(c.alloc(&L.gam32[a], n));
    }
    if (fields) {
        TRY(c.alloc(&L.v64, n)); TRY(c.alloc(&L.r64, n));
        TRY(c.alloc(&L.v32, n)); TRY(c.alloc(&L.r32, n));
    }
    return 0;
}

// transfer tables between fine level F (index n) and coarse level n+1 along d
int build_transfer(Ctx &c, Transfer &F, int d, int n)
{
    const int nc = c.mgrid[d][n + 1];
    const int mf = (n == 1) ? (d == 0 ? c.nx : d == 1 ? c.ny : c.nz) : c.mgrid[d][n] + 1;
    // restriction weights (IBM/CORE_MG.F90:2508-2520)
    std::vector<double> w1(nc + 2, 0.0), w2(nc + 2, 0.0);
    const auto &X = c.xMG[d][n];
    for (int i = 1; i <= nc; ++i) {
        const int ii = 2 * i, iim = 2 * i - 1, iip = 2 * i + 1;
        const double area1 = X[ii] - X[iim], area2 = X[iip] - X[ii], area = area1 + area2;
        w1[i] = area1 / area;
        w2[i] = area2 / area;
    }
    // prolongation weights (IBM/CORE_MG.F90:2960-2977) and per-fine-index plan
    std::vector<double> pw1(nc + 2), pw2(nc + 2), pw3(nc + 2), pw4(nc + 2);
    const auto &xf = c.xcMG[d][n], &xcc = c.xcMG[d][n + 1];
    for (int i = 1; i <= nc; ++i) {
        const int ii = 2 * i, iim = 2 * i - 1;
        auto sq = [](double t) { return 1.0 / (t * t); };
        double d1 = sq(xf[iim] - xcc[i]), d2 = sq(xf[iim] - xcc[i - 1]), de = d1 + d2;
        pw1[i] = d1 / de; pw2[i] = d2 / de;
        d1 = sq(xf[ii] - xcc[i]); d2 = sq(xf[ii] - xcc[i + 1]); de = d1 + d2;
        pw3[i] = d1 / de; pw4[i] = d2 / de;
    }
    std::vector<int> cA(mf + 1, 0), cB(mf + 1, 0);
    std::vector<int8_t> mode(mf + 1, 0);
    std::vector<double> wA(mf + 1, 0.0), wB(mf + 1, 0.0);
    auto interp = [&](int fi, int a, double wa, int b, double wb) { mode[fi] = 2; cA[fi] = a; wA[fi] = wa; cB[fi] = b; wB[fi] = wb; };
    auto copy = [&](int fi, int a) { mode[fi] = 1; cA[fi] = a; cB[fi] = a; };
    copy(1, 1);
    interp(2, 1, pw3[1], 2, pw4[1]);
    for (int i = 2; i <= nc - 1; ++i) {
        interp(2 * i - 1, i, pw1[i], i - 1, pw2[i]);
        interp(2 * i, i, pw3[i], i + 1, pw4[i]);
    }
    interp(2 * nc - 1, nc, pw1[nc], nc - 1, pw2[nc]);
    copy(2 * nc, nc);
    if (n == 1 && mf - 1 > 2 * nc) copy(mf - 1, nc);
    std::vector<float> w1f(w1.begin(), w1.end()), w2f(w2.begin(), w2.end());
    std::vector<float> wAf(wA.begin(), wA.end()), wBf(wB.begin(), wB.end());
    if (!F.rw1_64) {
        TRY(c.alloc(&F.rw1_64, w1.size())); TRY(c.alloc(&F.rw2_64, w2.size()));
        TRY(c.alloc(&F.rw1_32, w1.size())); TRY(c.alloc(&F.rw2_32, w2.size()));
        TRY(c.alloc(&F.pcA, cA.size())); TRY(c.alloc(&F.pcB, cB.size())); TRY(c.alloc(&F.pmode, mode.size()));
        TRY(c.alloc(&F.pwA64, wA.size())); TRY(c.alloc(&F.pwB64, wB.size()));
        TRY(c.alloc(&F.pwA32, wA.size())); TRY(c.alloc(&F.pwB32, wB.size()));
    }
    CK(cudaMemcpyAsync(F.rw1_64, w1.data(), w1.size() * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.rw2_64, w2.data(), w2.size() * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.rw1_32, w1f.data(), w1f.size() * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.rw2_32, w2f.data(), w2f.size() * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.pcA, cA.data(), cA.size() * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.pcB, cB.data(), cB.size() * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.pmode, mode.data(), mode.size(), cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.pwA64, wA.data(), wA.size() * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.pwB64, wB.data(), wB.size() * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.pwA32, wAf.data(), wAf.size() * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(F.pwB32, wBf.data(), wBf.size() * 4, cudaMemcpyHostToDevice, c.s));
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

// ------------------------------------------------------------- smoother ----
template <typename T> T *lv_binv(Level &L, int a);
template <> double *lv_binv<double>(Level &L, int a) { return L.binv64[a]; }
template <> float *lv_binv<float>(Level &L, int a) { return L.binv32[a]; }
template <typename T> T *lv_gam(Level &L, int a);
template <> double *lv_gam<double>(Level &L, int a) { return L.gam64[a]; }
template <> float *lv_gam<float>(Level &L, int a) { return L.gam32[a]; }
template <typename T> T *scratch_U(Ctx &c);
template <> double *scratch_U<double>(Ctx &c) { return c.U64; }
template <> float *scratch_U<float>(Ctx &c) { return c.U32; }

// Adds the durations of the timed line launches [p0, p1) of a graph that has
// completed on the stream (the caller has synchronised it).
void lt_harvest(Ctx &c, int p0, int p1)
{
    for (int q = p0; q < p1; ++q) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, c.lt_ev[2 * q], c.lt_ev[2 * q + 1]) == cudaSuccess) {
            c.lt_ms[c.lt_f32[q]] += ms;
            c.lt_n[c.lt_f32[q]]++;
        } else {
            (void)cudaGetLastError();   // not recorded: skip without leaving the error pending
        }
    }
}

// MG_itsolv: x-, y- (and z-) line sweeps, each red then black.
template <typename T>
void itsolv(Ctx &c, Level &L, T *v, const T *r, bool finest, bool homogeneous)
{
    LineArgs<T> a;
    a.v = v; a.r = r; a.fl = L.fl; a.U = scratch_U<T>(c); a.c = coef_of<T>(L); a.d = L.d;
    a.omega = (T)c.p.omega;
    const bool om1 = (c.p.omega == 1.0);
    for (int dir = 0; dir < c.nd; ++dir) {
        a.wpf = std::is_same<T, double>::value ? L.wpf[dir] : nullptr;
        a.binv = lv_binv<T>(L, dir);
        a.gam = lv_gam<T>(L, dir);
        a.dir_lo = finest ? L.dlo[dir] : 0;
        a.dir_hi = finest ? L.dhi[dir] : 0;
        a.ppp_lo = homogeneous ? T(0) : (T)c.p.ppp[2 * dir];
        a.ppp_hi = homogeneous ? T(0) : (T)c.p.ppp[2 * dir + 1];
        for (int col = 0; col < 2; ++col) {
            a.colour = col;
            const bool timed = c.lt_on && &L == &c.L1 && 2 * c.lt_next + 1 < (int)c.lt_ev.size();
            // external records become event-record nodes when the stream is being captured
            if (timed) cudaEventRecordWithFlags(c.lt_ev[2 * c.lt_next], c.s, cudaEventRecordExternal);
            launch_line<T>(dir, a, om1, c.s);
            if (timed) {
                cudaEventRecordWithFlags(c.lt_ev[2 * c.lt_next + 1], c.s, cudaEventRecordExternal);
                c.lt_f32[c.lt_next] = std::is_same<T, float>::value ? 1 : 0;
                ++c.lt_next;
            }
            c.launches++;
        }
    }
}

template <typename T> T *lv_v(Level &L);
template <> double *lv_v<double>(Level &L) { return L.v64; }
template <> float *lv_v<float>(Level &L) { return L.v32; }
template <typename T> T *lv_r(Level &L);
template <> double *lv_r<double>(Level &L) { return L.r64; }
template <> float *lv_r<float>(Level &L) { return L.r32; }

// GCM_Pressure on level 1 (IBM/CORE_MG.F90:4707-4743): outer ghost layer and the
// ghost-cell rows.  The compatibility call inside MG only shifts pgrad*, which the
// MG smoother never reads; the outer GCM_correct_pressure recomputes it.
template <typename T>
void gcm_pressure(Ctx &c, T *v);
template <>
void gcm_pressure<double>(Ctx &c, double *v)
{
    launch_outer_ghost<double>(v, c.L1.d, c.sign, c.s);
    c.launches++;
    if (c.nGhost > 0) {
        GhostArgs g{c.nGhost, c.gidx, c.sidx, c.gsg, c.gg_ptr, c.gg_idx};
        launch_ghost_rows<double>(v, g, c.gco64, c.ggc64, c.gscr64, c.p.iterMax_ad, c.p.restol_ad, 0.0, c.d_iters, c.d_maxd,
                                  c.s);
        c.launches++;
    }
}
template <>
void gcm_pressure<float>(Ctx &c, float *v)
{
    launch_outer_ghost<float>(v, c.L1.d, c.sign, c.s);
    c.launches++;
    if (c.nGhost > 0) {
        GhostArgs g{c.nGhost, c.gidx, c.sidx, c.gsg, c.gg_ptr, c.gg_idx};
        launch_ghost_rows<float>(v, g, c.gco32, c.ggc32, c.gscr32, c.p.iterMax_ad, c.p.restol_ad, c.ghost32_reltol,
                                 c.d_iters, c.d_maxd,
                                 c.s);
        c.launches++;
    }
}

template <typename T> const T *rw1(Transfer &L);
template <> const double *rw1<double>(Transfer &L) { return L.rw1_64; }
template <> const float *rw1<float>(Transfer &L) { return L.rw1_32; }
template <typename T> const T *rw2(Transfer &L);
template <> const double *rw2<double>(Transfer &L) { return L.rw2_64; }
template <> const float *rw2<float>(Transfer &L) { return L.rw2_32; }
template <typename T> const T *pwA(Transfer &L);
template <> const double *pwA<double>(Transfer &L) { return L.pwA64; }
template <> const float *pwA<float>(Transfer &L) { return L.pwA32; }
template <typename T> const T *pwB(Transfer &L);
template <> const double *pwB<double>(Transfer &L) { return L.pwB64; }
template <> const float *pwB<float>(Transfer &L) { return L.pwB32; }

Level &level_of(Ctx &c, int d, int n) { return n == 1 ? c.L1 : c.C[d][n]; }

// MG_X / MG_Y / MG_Z (IBM/CORE_MG.F90:1239-1663) for direction d.  At level 1 the
// caller passes the level-1 var/rhs; coarse levels use their own arrays.  With
// mixed precision (T = float) every level, the coarsest included, is smoothed
// in FP32.
template <typename T>
void mg_cycle(Ctx &c, int d, T *var, const T *rhs, int n, int WF, int &GMM, bool homogeneous)
{
    Level &L = level_of(c, d, n);
    const int nlev = c.nlev[d];
    const int mgCycle = c.p.mgcycle[d];
    const int totIter = (n == 1) ? c.p.iterFinest : ((n == nlev) ? c.p.iterCoarsest : 1);
    const bool gcm = (c.p.boundary_formulation == GCM_METHOD);
    if (n == 1 && gcm) gcm_pressure<T>(c, var);
    if (WF == 1) {
        for (int it = 0; it < totIter; ++it) itsolv<T>(c, L, var, rhs, n == 1, homogeneous);
    }
    if (n == nlev) {
        if (mgCycle == 3) GMM = 1;
        return;
    }
    Level &Cn = c.C[d][n + 1];
    T *phi = lv_v<T>(Cn);
    T *r1 = lv_r<T>(Cn);
    {
        Transfer &Tn = c.T[d][n];
        RestrictArgs<T> a;
        a.v = var; a.r = rhs; a.fl = L.fl; a.c = coef_of<T>(L); a.df = L.d; a.dc = Cn.d;
        a.w1 = rw1<T>(Tn); a.w2 = rw2<T>(Tn); a.rc = r1;
        launch_resid_restrict<T>(d, a, c.s);
        launch_fill<T>(phi, Cn.d.count(), T(0), c.s);
        c.launches += 2;
    }
    const int count = (n != nlev - 1) ? GMM : 1;
    for (int I = 1; I <= count; ++I) mg_cycle<T>(c, d, phi, r1, n + 1, I, GMM, true);
    {
        Transfer &Tn = c.T[d][n];
        ProlongArgs<T> a;
        a.phi = phi; a.flc = Cn.fl; a.v = var; a.flf = L.fl; a.df = L.d; a.dc = Cn.d;
        a.cA = Tn.pcA; a.cB = Tn.pcB; a.wA = pwA<T>(Tn); a.wB = pwB<T>(Tn); a.mode = Tn.pmode;
        launch_prolong_correct<T>(d, a, c.s);
        c.launches++;
    }
    if (n == 1 && gcm) gcm_pressure<T>(c, var);
    int post;
    if (d == 0) post = (n == 1) ? 0 : 1;
    else if (d == 1) post = (n == 1) ? ((c.p.ndim == 2) ? c.p.iterFinest : 0) : 1;
    else post = (n == 1) ? c.p.iterFinest : 1;
    for (int it = 0; it < post; ++it) itsolv<T>(c, L, var, rhs, n == 1, homogeneous);
    if (d != 0 && n == 1 && gcm) gcm_pressure<T>(c, var);
    if (n == 1 && mgCycle == 3) GMM = 2;
}

// MG_Solver (IBM/CORE_MG.F90:281-334): x cycle, y cycle, z cycle (3D).
template <typename T>
void mg_solver(Ctx &c, T *var, const T *rhs, bool homogeneous)
{
    for (int d = 0; d < c.nd; ++d) {
        const int sel = (d == 2) ? c.p.mgcycle[0] : c.p.mgcycle[d];   // MG_Solv_z tests mgCycleX (:515)
        int GMM = (sel == 1) ? 1 : 2;
        mg_cycle<T>(c, d, var, rhs, 1, 1, GMM, homogeneous);
    }
}

// subtracting_average_pressure (IBM/CORE_POISSON.F90:419-490): volume-weighted
// fluid mean removed, dead cells zeroed, then the fresh cells of a moving body
void subtract_average(Ctx &c, double *p)
{
    launch_subtract_average(p, c.L1.fl, c.d_dx[0], c.d_dx[1], c.d_dx[2], c.L1.d, (double *)c.partials, c.nred, c.s);
    c.launches += 3;
    if (c.fresh_on) {
        launch_fresh_cells(p, c.L1.fl, c.fresh, c.L1.d, c.p.ndim == 3, c.s);
        c.launches++;
    }
}

// GCM_correct_pressure on the level-1 FP64 field (IBM/CORE_POISSON.F90:1794-1823)
void correct_pressure(Ctx &c, double *p, double *nlw0)
{
    launch_outer_ghost<double>(p, c.L1.d, c.sign, c.s);
    c.launches++;
    if (c.nGhost > 0) {
        GhostArgs g{c.nGhost, c.gidx, c.sidx, c.gsg, c.gg_ptr, c.gg_idx};
        launch_ghost_rows<double>(p, g, c.gco64, c.ggc64, c.gscr64, c.p.iterMax_ad, c.p.restol_ad, 0.0, c.d_iters, c.d_maxd,
                                  c.s);
        c.launches++;
    }
    if (c.compat_active) {
        int zg[6];
        for (int q = 0; q < 6; ++q) zg[q] = (c.p.bc[q] == BC_ZERO_GRADIENT);
        launch_compat(p, c.L1.fl, c.pgrad, c.d_dx[0], c.d_dx[1], c.d_dx[2], c.d_dxcinv[0], c.d_dxcinv[1],
                      c.d_dxcinv[2], c.side_raw, c.L1.d, (double *)c.partials, c.nred, c.pgrad, zg, c.p.outflow_area,
                      c.nx, c.ny, c.nz, c.s);
        c.launches += 3;
    }
    if (c.nlw0_nonzero && nlw0) {
        launch_nlw0(nlw0, c.L1.fl, c.side_raw, c.pgrad, c.d_dxinv[0], c.d_dxinv[1], c.d_dxinv[2], c.L1.d, c.nx, c.ny,
                    c.nz, c.s);
        c.launches++;
    }
}

void calc_residual(Ctx &c, const double *p, const double *b, float *r32)
{
    launch_calc_residual(p, b, c.nlw0_nonzero ? c.nlw0 : nullptr, c.L1.fl, coef_of<double>(c.L1), c.L1.d, r32,
                         c.partials, c.nred, c.result, c.s);
    c.launches += 2;
}

// One outer iteration of solve_poisson (IBM/CORE_POISSON.F90:640-663), ending
// with the residual max-norm in c.result.
void outer_iteration(Ctx &c, double *p, const double *b)
{
    if (c.p.precision_mode == 1) {
        // FP32 cycle on the correction e with rhs r32 = fl(b - A p), FP64 refinement
        launch_fill<float>(c.e32, c.L1.d.count(), 0.0f, c.s);
        c.launches++;
        mg_solver<float>(c, c.e32, c.r32, true);
        launch_accumulate(p, c.e32, c.L1.d.count(), c.s);
        c.launches++;
        if (c.p.boundary_formulation == GCM_METHOD) correct_pressure(c, p, c.nlw0);
        calc_residual(c, p, b, c.r32);
    } else {
        mg_solver<double>(c, p, b, false);
        if (c.p.boundary_formulation == GCM_METHOD) correct_pressure(c, p, c.nlw0);
        calc_residual(c, p, b, nullptr);
    }
}

int run_outer(Ctx &c, double *p, const double *b)
{
    if (c.graph && (c.graph_p != p || c.graph_b != b)) {
        cudaGraphExecDestroy(c.graph);
        c.graph = nullptr;
    }
    if (!c.graph) {
        cudaGraph_t g;
        const long long before = c.launches;
        c.lt_next = c.graph_lt0 = 0;
        CK(cudaStreamBeginCapture(c.s, cudaStreamCaptureModeThreadLocal));
        outer_iteration(c, p, b);
        CK(cudaStreamEndCapture(c.s, &g));
        c.graph_lt1 = c.lt_next;
        c.graph_kernels = c.launches - before;
        c.launches = before;
        cudaError_t e = cudaGraphInstantiate(&c.graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(-10, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        c.graph_p = p;
        c.graph_b = b;
    }
    CK(cudaGraphLaunch(c.graph, c.s));
    c.launches += c.graph_kernels;
    return 0;
}

int loc_of(const Ctx &c, long long idx, int *loc)
{
    const Dims d = c.L1.d;
    if (loc) {
        loc[0] = (int)(idx % d.sx);
        loc[1] = (int)((idx / d.sx) % (d.m[1] + 2));
        loc[2] = (int)(idx / d.sxy);
    }
    return 0;
}

int ensure_krylov(Ctx &c, int m)
{
    if (c.km >= m) return 0;
    if (m > 60) return fail(-1, "outer_krylov must be <= 60");
    const long long n1 = c.L1.d.count();
    if (c.p.precision_mode == 1) {
        while ((int)c.KV32.size() < m + 1) { float *q; TRY(c.alloc(&q, n1)); c.KV32.push_back(q); }
        while ((int)c.KZ32.size() < m) { float *q; TRY(c.alloc(&q, n1)); c.KZ32.push_back(q); }
        if (!c.kw32) TRY(c.alloc(&c.kw32, n1));
    } else {
        while ((int)c.KV.size() < m + 1) { double *q; TRY(c.alloc(&q, n1)); c.KV.push_back(q); }
        while ((int)c.KZ.size() < m) { double *q; TRY(c.alloc(&q, n1)); c.KZ.push_back(q); }
        if (!c.kzp) { TRY(c.alloc(&c.kzp, n1)); TRY(c.alloc(&c.kzr, n1)); }
    }
    if (!c.kw) {
        TRY(c.alloc(&c.kw, n1));
        TRY(c.alloc(&c.kpart, 8 * (size_t)c.nred + 8));
        TRY(c.alloc(&c.kdots, 256));
        CK(cudaMallocHost(&c.h_kdots, 256 * sizeof(double)));
    }
    c.km = m;
    return 0;
}

// z = M^-1 v: one MG_Solver schedule on the correction (zero initial guess,
// homogeneous boundary values) run as a CUDA graph on fixed buffers: FP32
// (r32 -> e32) in mixed mode, FP64 (kzr -> kzp) otherwise.  v and z are
// Krylov vectors of the same precision.
template <typename T>
int precondition(Ctx &c, const T *v, T *z)
{
    const long long n1 = c.L1.d.count();
    constexpr bool f32 = std::is_same<T, float>::value;
    T *in = f32 ? (T *)c.r32 : (T *)c.kzr;
    T *out = f32 ? (T *)c.e32 : (T *)c.kzp;
    CK(cudaMemcpyAsync(in, v, n1 * sizeof(T), cudaMemcpyDeviceToDevice, c.s));
    if (!c.pgraph) {
        cudaGraph_t g;
        const long long before = c.launches;
        c.lt_next = c.pgraph_lt0 = (int)c.lt_ev.size() / 4;   // second half of the pairs
        CK(cudaStreamBeginCapture(c.s, cudaStreamCaptureModeThreadLocal));
        launch_fill<T>(out, n1, T(0), c.s);
        mg_solver<T>(c, out, in, true);
        c.launches++;
        CK(cudaStreamEndCapture(c.s, &g));
        c.pgraph_lt1 = c.lt_next;
        c.pgraph_kernels = c.launches - before;
        c.launches = before;
        cudaError_t e = cudaGraphInstantiate(&c.pgraph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(-10, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    }
    CK(cudaGraphLaunch(c.pgraph, c.s));
    c.launches += c.pgraph_kernels;
    CK(cudaMemcpyAsync(z, out, n1 * sizeof(T), cudaMemcpyDeviceToDevice, c.s));
    return 0;
}

// Relative reduction one FP32 inner cycle aims for at most; the FP64 residual
// recomputed at the restart carries the refinement further.
constexpr double kKrylovInnerRtol = 1.0e-5;

// solve_poisson with FGMRES(m) around MG_Solver (outer_krylov = m).  Same
// discrete system (fluid rows with ghost values from the ghost-row fixed
// point), same stopping test (max-norm of the calc_residual residual, FP64).
// Iterations count preconditioner applications (one MG_Solver each).  T is
// the precision of the Krylov vectors, the preconditioner and the operator
// inside a cycle: FP64 in the plain form; FP32 in the mixed form, where each
// restart recomputes the residual in FP64 and adds the cycle's correction to
// p in FP64 (iterative refinement with an FP32 FGMRES inner solver).
// n1 = nlw0 of a unit shift of the zero-gradient planes (-1 on minus sides, +1 on plus
// sides, over the (0:n_a-1, 0:n_b-1) part of each plane that GCM_enforce_p_compatibility
// shifts), in FP64 and FP32; depends on the flags only
int ensure_compat_rank1(Ctx &c)
{
    if (c.n1_ready) return 0;
    const long long n1 = c.L1.d.count();
    if (!c.pg_unit) TRY(c.alloc(&c.pg_unit, c.npgrad));
    if (!c.n1_64) TRY(c.alloc(&c.n1_64, (size_t)n1));
    if (!c.n1_32) TRY(c.alloc(&c.n1_32, (size_t)n1));
    if (!c.kflux) TRY(c.alloc(&c.kflux, 2));
    const long long px = (long long)(c.ny + 2) * (c.nz + 2), py = (long long)(c.nx + 2) * (c.nz + 2),
                    pz = (long long)(c.nx + 2) * (c.ny + 2);
    const long long off[6] = {0, px, 2 * px, 2 * px + py, 2 * px + 2 * py, 2 * px + 2 * py + pz};
    const int sa[6] = {c.ny + 2, c.ny + 2, c.nx + 2, c.nx + 2, c.nx + 2, c.nx + 2};
    const int sb[6] = {c.nz + 2, c.nz + 2, c.nz + 2, c.nz + 2, c.ny + 2, c.ny + 2};
    if ((size_t)(off[5] + pz) > c.npgrad) return fail(-1, "pgrad buffer smaller than its six planes");
    std::vector<double> h(c.npgrad, 0.0);
    for (int q = 0; q < 6; ++q) {
        if (c.p.bc[q] != BC_ZERO_GRADIENT) continue;
        const double sign = (q % 2 == 0) ? -1.0 : 1.0;
        for (int b = 0; b <= sb[q] - 2; ++b)
            for (int a = 0; a <= sa[q] - 2; ++a) h[(size_t)(off[q] + a + (long long)sa[q] * b)] = sign;
    }
    CK(cudaMemcpyAsync(c.pg_unit, h.data(), c.npgrad * sizeof(double), cudaMemcpyHostToDevice, c.s));
    CK(cudaMemsetAsync(c.n1_64, 0, (size_t)n1 * sizeof(double), c.s));
    launch_nlw0(c.n1_64, c.L1.fl, c.side_raw, c.pg_unit, c.d_dxinv[0], c.d_dxinv[1], c.d_dxinv[2], c.L1.d, c.nx, c.ny,
                c.nz, c.s);
    launch_convert_d2f(c.n1_32, c.n1_64, n1, c.s);
    c.launches += 2;
    CK(cudaStreamSynchronize(c.s));   // h leaves scope
    c.n1_ready = true;
    return 0;
}

template <typename T>
int solve_krylov_t(Ctx &c, double *p, const double *b, int *iters, double *maxres_out, int *loc, double *compTime)
{
    constexpr bool f32 = std::is_same<T, float>::value;
    const int m = c.p.outer_krylov;
    TRY(ensure_krylov(c, m));
    std::vector<T *> &KV = [&]() -> std::vector<T *> & {
        if constexpr (f32) return c.KV32; else return c.KV;
    }();
    std::vector<T *> &KZ = [&]() -> std::vector<T *> & {
        if constexpr (f32) return c.KZ32; else return c.KZ;
    }();
    T *w = f32 ? (T *)c.kw32 : (T *)c.kw;
    const long long n1 = c.L1.d.count();
    const bool gcm = (c.p.boundary_formulation == GCM_METHOD);
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaEventRecord(c.ev0, c.s));
    const bool dirichlet = c.p.pbc[0] == PBC_DIRICHLET || c.p.pbc[2] == PBC_DIRICHLET || c.p.pbc[4] == PBC_DIRICHLET;
    if (dirichlet) return fail(-1, "outer_krylov needs all-Neumann pressure boundaries");
    // With zero-gradient sides each restart's GCM_correct_pressure shifts the outflow planes by
    // -(phi . p + chi(pgrad)) / outflow_area, a linear function of p: the iteration's fixed point
    // solves A p + (phi . p / outflow_area) n1 = b', b' independent of the planes.  The cycles
    // apply that operator (the rank-one term below), so the shift at the next restart leaves
    // the residual they reduced unchanged.
    const bool rank1 = c.compat_active && gcm;
    if (rank1) TRY(ensure_compat_rank1(c));
    const T *n1T = f32 ? (const T *)c.n1_32 : (const T *)c.n1_64;
    if (c.nlw0_nonzero) { launch_fill<double>(c.nlw0, n1, 0.0, c.s); c.launches++; }
    subtract_average(c, p);
    CK(cudaMemsetAsync(c.d_iters, 0, sizeof(int), c.s));
    CK(cudaMemsetAsync(c.d_maxd, 0, sizeof(unsigned long long), c.s));
    c.hist.clear();
    int it = 0;
    double maxres = 1.0e10;
    long long maxidx = 0;
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m, 0.0), sn(m, 0.0), g(m + 1, 0.0), y(m, 0.0);
    auto Hij = [&](int i, int j) -> double & { return H[(size_t)i + (size_t)(m + 1) * j]; };
    const Coef<double> coef = coef_of<double>(c.L1);
    const Coef<T> coefT = coef_of<T>(c.L1);
    const T *gco = f32 ? (const T *)c.gco32 : (const T *)c.gco64;
    T *gscr = f32 ? (T *)c.gscr32 : (T *)c.gscr64;
    while (true) {
        if (gcm) correct_pressure(c, p, c.nlw0);
        // FP64 residual r = b - A p (into kw), its max-norm and 2-norm
        launch_calc_residual(p, b, c.nlw0_nonzero ? c.nlw0 : nullptr, c.L1.fl, coef, c.L1.d, nullptr, c.partials,
                             c.nred, c.result, c.s, c.kw);
        c.launches += 2;
        CK(cudaMemcpyAsync(c.h_result, c.result, sizeof(MaxLoc), cudaMemcpyDeviceToHost, c.s));
        CK(cudaStreamSynchronize(c.s));
        maxres = c.h_result->v;
        maxidx = c.h_result->i;
        if (!c.hist.empty()) c.hist.back() = maxres;   // true value at the restart point
        if (!std::isfinite(maxres) || maxres <= c.p.restol_Poisson || it >= c.p.iterMax_Poisson) break;
        const double *r64 = c.kw;
        launch_mdot<double>(&r64, 1, c.kw, c.L1.fl, c.L1.d, c.kpart, c.nred, c.kdots, c.s);
        CK(cudaMemcpyAsync(c.h_kdots, c.kdots, sizeof(double), cudaMemcpyDeviceToHost, c.s));
        CK(cudaStreamSynchronize(c.s));
        const double beta = std::sqrt(c.h_kdots[0]);
        if (!(beta > 0.0)) break;
        launch_scale_copy<T, double>(KV[0], c.kw, c.kdots, n1, c.s);
        c.launches += 3;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        double target = 0.5 * beta * c.p.restol_Poisson / maxres;
        if (f32) target = std::max(target, kKrylovInnerRtol * beta);
        int k = 0;
        for (int j = 0; j < m; ++j) {
            TRY(precondition<T>(c, KV[j], KZ[j]));
            if (gcm) {   // ghost values of z from its fluid values (the map whose matrix A acts on)
                launch_outer_ghost<T>(KZ[j], c.L1.d, c.sign, c.s);
                if (c.nGhost > 0) {
                    GhostArgs ga{c.nGhost, c.gidx, c.sidx, c.gsg, c.gg_ptr, c.gg_idx};
                    launch_ghost_rows<T>(KZ[j], ga, gco, f32 ? (const T *)c.ggc32 : (const T *)c.ggc64, gscr,
                                         c.p.iterMax_ad, c.p.restol_ad, f32 ? c.ghost32_reltol : 0.0,
                                         c.d_iters, c.d_maxd, c.s);
                }
                c.launches += 2;
            }
            launch_apply_op<T>(KZ[j], w, c.L1.fl, coefT, c.L1.d, c.s);
            c.launches++;
            if (rank1) {
                launch_compat_rank1<T>(KZ[j], w, n1T, c.L1.fl, c.d_dx[0], c.d_dx[1], c.d_dx[2], c.d_dxcinv[0],
                                       c.d_dxcinv[1], c.d_dxcinv[2], c.side_raw, c.L1.d, (double *)c.partials,
                                       c.nred, c.kflux, c.p.outflow_area, c.nx, c.ny, c.nz, c.s);
                c.launches += 3;
            }
            const T *const *Vp = KV.data();
            // classical Gram-Schmidt, twice
            launch_mdot<T>(Vp, j + 1, w, c.L1.fl, c.L1.d, c.kpart, c.nred, c.kdots, c.s);
            launch_maxpy<T>(w, Vp, j + 1, c.kdots, -1.0, n1, c.s);
            launch_mdot<T>(Vp, j + 1, w, c.L1.fl, c.L1.d, c.kpart, c.nred, c.kdots + 64, c.s);
            launch_maxpy<T>(w, Vp, j + 1, c.kdots + 64, -1.0, n1, c.s);
            const T *wp = w;
            launch_mdot<T>(&wp, 1, w, c.L1.fl, c.L1.d, c.kpart, c.nred, c.kdots + 128, c.s);
            launch_scale_copy<T, T>(KV[j + 1], w, c.kdots + 128, n1, c.s);
            c.launches += 4 * ((j + 8) / 8) * 2 + 3;
            CK(cudaMemcpyAsync(c.h_kdots, c.kdots, 256 * sizeof(double), cudaMemcpyDeviceToHost, c.s));
            CK(cudaStreamSynchronize(c.s));
            if (c.lt_on) lt_harvest(c, c.pgraph_lt0, c.pgraph_lt1);
            for (int i = 0; i <= j; ++i) Hij(i, j) = c.h_kdots[i] + c.h_kdots[64 + i];
            const double hn = std::sqrt(c.h_kdots[128]);
            Hij(j + 1, j) = hn;
            // Givens rotations
            for (int i = 0; i < j; ++i) {
                const double a = Hij(i, j), bb = Hij(i + 1, j);
                Hij(i, j) = cs[i] * a + sn[i] * bb;
                Hij(i + 1, j) = -sn[i] * a + cs[i] * bb;
            }
            const double a = Hij(j, j), bb = Hij(j + 1, j);
            const double r = std::hypot(a, bb);
            cs[j] = (r > 0.0) ? a / r : 1.0;
            sn[j] = (r > 0.0) ? bb / r : 0.0;
            Hij(j, j) = r;
            Hij(j + 1, j) = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++it;
            k = j + 1;
            c.hist.push_back(maxres * std::fabs(g[j + 1]) / beta);   // estimate until the next true value
            if (std::fabs(g[j + 1]) <= target || it >= c.p.iterMax_Poisson || !(hn > 0.0)) break;
        }
        // y = H^-1 g (upper triangular k x k), p += sum y_i z_i
        for (int i = k - 1; i >= 0; --i) {
            double sacc = g[i];
            for (int l = i + 1; l < k; ++l) sacc -= Hij(i, l) * y[l];
            y[i] = sacc / Hij(i, i);
        }
        CK(cudaMemcpyAsync(c.kdots + 192, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, c.s));
        if constexpr (f32) {
            // correction summed in FP32, accumulated into p in FP64
            launch_fill<float>(c.e32, n1, 0.0f, c.s);
            launch_maxpy<float>(c.e32, KZ.data(), k, c.kdots + 192, 1.0, n1, c.s);
            launch_accumulate(p, c.e32, n1, c.s);
            c.launches += 2 + (k + 7) / 8;
        } else {
            launch_maxpy<double>(p, KZ.data(), k, c.kdots + 192, 1.0, n1, c.s);
            c.launches += (k + 7) / 8;
        }
    }
    CK(cudaEventRecord(c.ev1, c.s));
    int h_iters = 0;
    unsigned long long h_maxd = 0;
    CK(cudaMemcpyAsync(&h_iters, c.d_iters, sizeof(int), cudaMemcpyDeviceToHost, c.s));
    CK(cudaMemcpyAsync(&h_maxd, c.d_maxd, sizeof(h_maxd), cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    c.ghost_sweeps = h_iters;
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.last_iters = it;
    c.last_maxres = maxres;
    c.last_time = 1e-3 * (double)ms;
    c.last_wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (iters) *iters = it;
    if (maxres_out) *maxres_out = maxres;
    loc_of(c, maxidx, loc);
    if (compTime) *compTime = c.last_time;
    if (!std::isfinite(maxres)) return fail(-5, "residual is not finite (NaN or Inf in the inputs?)");
    if (maxres > c.p.restol_Poisson) return 1;
    return 0;
}

int solve_krylov(Ctx &c, double *p, const double *b, int *iters, double *maxres_out, int *loc, double *compTime)
{
    if (c.p.precision_mode == 1) return solve_krylov_t<float>(c, p, b, iters, maxres_out, loc, compTime);
    return solve_krylov_t<double>(c, p, b, iters, maxres_out, loc, compTime);
}

// solve_poisson MG branch on device-resident full-layout arrays
int solve_device(Ctx &c, double *p, const double *b, int *iters, double *maxres_out, int *loc, double *compTime)
{
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    if (c.p.outer_krylov > 0) return solve_krylov(c, p, b, iters, maxres_out, loc, compTime);
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaEventRecord(c.ev0, c.s));
    const bool dirichlet = c.p.pbc[0] == PBC_DIRICHLET || c.p.pbc[2] == PBC_DIRICHLET || c.p.pbc[4] == PBC_DIRICHLET;
    if (c.nlw0_nonzero) { launch_fill<double>(c.nlw0, c.L1.d.count(), 0.0, c.s); c.launches++; }
    if (!dirichlet) {   // subtracting_average_pressure (IBM/CORE_POISSON.F90:527-537)
        subtract_average(c, p);
    }
    if (c.p.precision_mode == 1) {
        // initial FP64 residual feeds the first FP32 cycle
        calc_residual(c, p, b, c.r32);
    }
    CK(cudaMemsetAsync(c.d_iters, 0, sizeof(int), c.s));
    CK(cudaMemsetAsync(c.d_maxd, 0, sizeof(unsigned long long), c.s));
    int iter = 0;
    double maxres = 1.0e10;
    long long maxidx = 0;
    c.hist.clear();
    while (iter < c.p.iterMax_Poisson && maxres > c.p.restol_Poisson) {
        TRY(run_outer(c, p, b));
        CK(cudaMemcpyAsync(c.h_result, c.result, sizeof(MaxLoc), cudaMemcpyDeviceToHost, c.s));
        CK(cudaStreamSynchronize(c.s));
        if (c.lt_on) lt_harvest(c, c.graph_lt0, c.graph_lt1);
        maxres = c.h_result->v;
        maxidx = c.h_result->i;
        c.hist.push_back(maxres);
        ++iter;
        if (!std::isfinite(maxres)) break;
    }
    CK(cudaEventRecord(c.ev1, c.s));
    int h_iters = 0;
    unsigned long long h_maxd = 0;
    CK(cudaMemcpyAsync(&h_iters, c.d_iters, sizeof(int), cudaMemcpyDeviceToHost, c.s));
    CK(cudaMemcpyAsync(&h_maxd, c.d_maxd, sizeof(h_maxd), cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    c.ghost_sweeps = h_iters;
    double maxd;
    std::memcpy(&maxd, &h_maxd, sizeof(maxd));
    auto t1 = std::chrono::steady_clock::now();
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    c.last_iters = iter;
    c.last_maxres = maxres;
    c.last_time = 1e-3 * (double)ms;   // device time between the first and last operation of the solve
    c.last_wall = std::chrono::duration<double>(t1 - t0).count();
    if (iters) *iters = iter;
    if (maxres_out) *maxres_out = maxres;
    loc_of(c, maxidx, loc);
    if (compTime) *compTime = c.last_time;
    if (!std::isfinite(maxres)) return fail(-5, "residual is not finite (NaN or Inf in the inputs?)");
    if (iter == c.p.iterMax_Poisson && maxres > c.p.restol_Poisson) return 1;
    if (c.nGhost > 0 && c.p.precision_mode == 0 && maxd > c.p.restol_ad) return 2;
    return 0;
}

// copy between a host array in the reference's level layout (0:m0,0:m1,0:m2 dense)
// and a device level array
template <typename T>
int copy_level(Ctx &c, const Level &L, T *dev, void *host, bool to_dev)
{
    const Dims d = L.d;
    const long long hsx = d.m[0] + 1, hsxy = hsx * (d.m[1] + 1);
    const long long nh = hsxy * (d.m[2] + 1);
    std::vector<T> tmp(d.count(), T(0));
    if (to_dev) {
        const T *h = (const T *)host;
        for (int k = 0; k <= d.m[2]; ++k)
            for (int j = 0; j <= d.m[1]; ++j)
                for (int i = 0; i <= d.m[0]; ++i) tmp[d.idx(i, j, k)] = h[i + hsx * j + hsxy * k];
        CK(cudaMemcpyAsync(dev, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, c.s));
        CK(cudaStreamSynchronize(c.s));
    } else {
        CK(cudaMemcpyAsync(tmp.data(), dev, tmp.size() * sizeof(T), cudaMemcpyDeviceToHost, c.s));
        CK(cudaStreamSynchronize(c.s));
        T *h = (T *)host;
        for (long long q = 0; q < nh; ++q) h[q] = T(0);
        for (int k = 0; k <= d.m[2]; ++k)
            for (int j = 0; j <= d.m[1]; ++j)
                for (int i = 0; i <= d.m[0]; ++i) h[i + hsx * j + hsxy * k] = tmp[d.idx(i, j, k)];
    }
    return 0;
}

} // namespace

// ========================================================================== C ABI
extern "C" {

const char *fsi_mg_last_error(void) { return g_err.c_str(); }

int fsi_mg_create(const fsi_mg_params *params, const double *x, const double *y, const double *z, void **handle)
{
    if (!params || !x || !y || !z || !handle) return fail(-1, "null argument");
    const fsi_mg_params &p = *params;
    if (p.ndim != 2 && p.ndim != 3) return fail(-1, "ndim must be 2 or 3");
    if (p.nx < 3 || p.ny < 3 || p.nz < 2) return fail(-1, "grid too small");
    if (p.ndim == 2 && p.nz != 2) return fail(-1, "2D grids have nz = 2");
    if (p.pp_solver_type != 3) return fail(-1, "only pp_solver_type = 3 (MG) runs on the GPU");
    for (int q = 0; q < 6; ++q) {
        if (p.bc[q] == BC_PERIODIC)
            return fail(-1, "periodic boundaries are not supported (the reference MG indexes var(nxc) on coarse levels)");
        if (p.pbc[q] != PBC_DIRICHLET && p.pbc[q] != PBC_NEUMANN) return fail(-1, "pbc must be 1 or 2");
    }
    for (int q = 0; q < 3; ++q)
        if (p.mgcycle[q] < 1 || p.mgcycle[q] > 3) return fail(-1, "mgcycle must be 1, 2 or 3");
    if (p.omega <= 0.0 || p.omega >= 2.0) return fail(-1, "omega must be in (0,2)");
    if (p.precision_mode != 0 && p.precision_mode != 1) return fail(-1, "precision_mode must be 0 or 1");
    if (p.outer_krylov < 0 || p.outer_krylov > 60) return fail(-1, "outer_krylov must be in 0..60");
    if ((long long)(p.nx + 1) * (p.ny + 1) * (p.nz + 1) >= (1LL << 31))
        return fail(-1, "grid too large: the (0:nx+1,0:ny+1,0:nz+1) layout must hold fewer than 2^31 cells");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(-12, "no CUDA device");
    CK(init_kernels());
    auto c = std::make_unique<Ctx>();
    c->p = p;
    c->nx = p.nx; c->ny = p.ny; c->nz = p.nz;
    c->nd = (p.ndim == 3) ? 3 : 2;
    CK(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking));
    CK(cudaEventCreate(&c->ev0));
    CK(cudaEventCreate(&c->ev1));
    CK(cudaEventCreate(&c->ev2));
    CK(cudaEventCreate(&c->ev3));
    const double *xs[3] = {x, y, z};
    const int N[3] = {p.nx, p.ny, p.nz};
    for (int d = 0; d < 3; ++d) {   // metrics of IBM/CORE_GRID.F90:96-139
        const int n = N[d];
        c->x[d].assign(xs[d], xs[d] + n + 2);
        c->xc[d].assign(n + 2, 0.0); c->dx[d].assign(n + 2, 0.0); c->dxinv[d].assign(n + 2, 0.0);
        c->dxc[d].assign(n + 2, 0.0); c->dxcinv[d].assign(n + 2, 0.0);
        for (int i = 0; i <= n; ++i) {
            c->xc[d][i] = 0.5 * (c->x[d][i + 1] + c->x[d][i]);
            c->dx[d][i] = c->x[d][i + 1] - c->x[d][i];
            if (!(c->dx[d][i] > 0.0)) return fail(-1, "node coordinates must increase");
            c->dxinv[d][i] = 1.0 / c->dx[d][i];
        }
        c->xc[d][n + 1] = c->x[d][n + 1];
        for (int i = 1; i <= n; ++i) {
            c->dxc[d][i] = c->xc[d][i] - c->xc[d][i - 1];
            c->dxcinv[d][i] = 1.0 / c->dxc[d][i];
        }
    }
    mg_initial(*c);
    for (int d = 0; d < c->nd; ++d) {
        for (int l = 2; l <= c->nlev[d]; ++l)
            if (c->mgrid[d][l] < 2) return fail(-1, "a coarse level has fewer than 2 cells; lower mgLevels");
        for (int l = 2; l < c->nlev[d]; ++l)
            if (c->mgrid[d][l] % 2 != 0)
                return fail(-1, "odd cell count on a coarse level is not supported; choose sizes that halve evenly");
    }
    // device state
    c->L1.d = full_dims(*c);
    TRY(alloc_level(*c, c->L1, false));
    for (int d = 0; d < c->nd; ++d) {
        c->C[d].resize(c->nlev[d] + 1);
        c->T[d].resize(c->nlev[d] + 1);
        for (int l = 2; l <= c->nlev[d]; ++l) {
            int m[3] = {c->nx, c->ny, c->nz};
            m[d] = c->mgrid[d][l] + 1;
            Level &L = c->C[d][l];
            L.d = dense_dims(m[0], m[1], m[2]);
            L.lev[d] = l;
            TRY(alloc_level(*c, L, true));
        }
    }
    const long long n1 = c->L1.d.count();
    TRY(c->alloc(&c->U64, n1));
    TRY(c->alloc(&c->U32, n1));
    TRY(c->alloc(&c->e32, n1));
    TRY(c->alloc(&c->r32, n1));
    TRY(c->alloc(&c->nlw0, n1));
    TRY(c->alloc(&c->stage, 2 * n1));
    c->nred = calc_residual_blocks(c->L1.d);
    TRY(c->alloc(&c->partials, (size_t)c->nred * 2 + 8));
    TRY(c->alloc(&c->result, 1));
    TRY(c->alloc(&c->d_iters, 1));
    TRY(c->alloc(&c->d_maxd, 1));
    CK(cudaMallocHost(&c->h_result, sizeof(MaxLoc)));
    for (int d = 0; d < 3; ++d) {
        TRY(c->alloc(&c->d_dx[d], N[d] + 2));
        TRY(c->alloc(&c->d_dxinv[d], N[d] + 2));
        TRY(c->alloc(&c->d_dxcinv[d], N[d] + 2));
        TRY(c->alloc(&c->d_xn[d], N[d] + 2));
        CK(cudaMemcpyAsync(c->d_xn[d], c->x[d].data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        CK(cudaMemcpyAsync(c->d_dx[d], c->dx[d].data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        CK(cudaMemcpyAsync(c->d_dxinv[d], c->dxinv[d].data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        CK(cudaMemcpyAsync(c->d_dxcinv[d], c->dxcinv[d].data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        std::vector<double> fx(N[d] + 2, 0.0);
        for (int i = 1; i <= N[d]; ++i)
            fx[i] = (c->x[d][i] - c->xc[d][i - 1]) / (c->xc[d][i] - c->xc[d][i - 1]);
        std::vector<double> gx(N[d] + 2, 0.0);
        for (int i = 1; i <= N[d]; ++i) gx[i] = 1.0 - fx[i];
        std::vector<double> adm(N[d] + 2, 0.0), adp(N[d] + 2, 0.0), adb(N[d] + 2, 0.0);
        for (int i = 1; i < N[d]; ++i) {
            adm[i] = c->dxcinv[d][i] * c->dxinv[d][i];
            adp[i] = c->dxcinv[d][i + 1] * c->dxinv[d][i];
            adb[i] = (c->dxinv[d][i] * 2.0) * c->dxinv[d][i];
        }
        TRY(c->alloc(&c->d_adm[d], N[d] + 2));
        TRY(c->alloc(&c->d_adp[d], N[d] + 2));
        TRY(c->alloc(&c->d_adb[d], N[d] + 2));
        CK(cudaMemcpyAsync(c->d_adm[d], adm.data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        CK(cudaMemcpyAsync(c->d_adp[d], adp.data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        CK(cudaMemcpyAsync(c->d_adb[d], adb.data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        TRY(c->alloc(&c->d_fx[d], N[d] + 2));
        TRY(c->alloc(&c->d_gx[d], N[d] + 2));
        CK(cudaMemcpyAsync(c->d_fx[d], fx.data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        CK(cudaMemcpyAsync(c->d_gx[d], gx.data(), (N[d] + 2) * 8, cudaMemcpyHostToDevice, c->s));
        CK(cudaStreamSynchronize(c->s));
    }
    c->npgrad = 2 * (size_t)(p.ny + 2) * (p.nz + 2) + 2 * (size_t)(p.nx + 2) * (p.nz + 2) +
                2 * (size_t)(p.nx + 2) * (p.ny + 2);
    TRY(c->alloc(&c->pgrad, c->npgrad));
    CK(cudaStreamSynchronize(c->s));
    *handle = c.release();
    return 0;
}

int fsi_mg_set_geometry(void *handle, const int8_t *iblank, const int8_t *ghostCellMark, const int8_t *ium,
                        const int8_t *iup, const int8_t *jum, const int8_t *jup, const int8_t *kum, const int8_t *kup,
                        int nGhost, const int32_t *iGhost, const int32_t *jGhost, const int32_t *kGhost,
                        const int32_t *iCellIndex, const int32_t *jCellIndex, const int32_t *kCellIndex,
                        const double *coeffGCMN, const double *probeLength, const double *pgrad)
{
    if (!handle) return fail(-1, "null handle");
    Ctx &c = *(Ctx *)handle;
    if (!iblank || !ghostCellMark || !ium || !iup || !jum || !jup || !kum || !kup) return fail(-1, "null flag array");
    if (nGhost < 0) return fail(-1, "nGhost < 0");
    if (nGhost > 0 && (!iGhost || !jGhost || !kGhost || !iCellIndex || !jCellIndex || !kCellIndex || !coeffGCMN))
        return fail(-1, "null ghost list");
    (void)probeLength;   // enters only through uNormal, which is 0 for viscous flow
    const int nx = c.nx, ny = c.ny, nz = c.nz, nxc = nx - 1, nyc = ny - 1, nzc = nz - 1;
    const Dims d1 = c.L1.d;
    const long long nf = d1.count();
    const int8_t *f6[6] = {ium, iup, jum, jup, kum, kup};
    // side values of the boundary faces: uniform over the face (set_outer_iup /
    // set_pressure_dirichlet_bc / remove_up_um), interior faces 0 or 1.
    const bool dir_any = c.p.pbc[0] == PBC_DIRICHLET || c.p.pbc[2] == PBC_DIRICHLET || c.p.pbc[4] == PBC_DIRICHLET;
    int side[6];
    for (int q = 0; q < 6; ++q) {
        const int ax = q / 2, hi = q % 2;
        const int bidx = hi ? (ax == 0 ? nxc : ax == 1 ? nyc : nzc) : 1;
        int val = -2;
        bool uniform = true;
        for (int k = 1; k <= nzc && uniform; ++k)
            for (int j = 1; j <= nyc && uniform; ++j)
                for (int i = 1; i <= nxc; ++i) {
                    const int idx3[3] = {i, j, k};
                    if (idx3[ax] != bidx) continue;
                    const int v = f6[q][d1.idx(i, j, k)];
                    if (val == -2) val = v;
                    else if (v != val) { uniform = false; break; }
                    if (ax == 0) break;
                }
        if (!uniform) return fail(-1, "boundary face flags must be uniform over each side");
        if (c.p.ndim == 2 && ax == 2) val = 0;
        if (dir_any && c.p.pbc[q] == PBC_DIRICHLET && !(c.p.ndim == 2 && ax == 2)) val = -1;   // set_pressure_dirichlet_bc
        if (val == 0 && !(c.p.ndim == 2 && ax == 2)) return fail(-1, "open (flag 0) outer faces need periodic BCs, which are not supported");
        side[q] = val;
    }
    for (int q = 0; q < 6; ++q) {
        c.side_raw[q] = side[q];
        c.sign[q] = (c.p.pbc[q] == PBC_NEUMANN) ? 1 : -1;
    }
    // pack the level-1 flag bytes (validating interior face values)
    std::vector<uint8_t> fl(nf, 0);
    long long nsolid = 0;
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                const long long o = d1.idx(i, j, k);
                uint8_t f = 0;
                if (iblank[o] != 0 && iblank[o] != 1) return fail(-1, "iblank must be 0 or 1");
                if (iblank[o] == 1) { f |= FB_IB; if (i >= 1 && i <= nxc && j >= 1 && j <= nyc && k >= 1 && k <= nzc) ++nsolid; }
                if (ghostCellMark[o] == 1) {
                    if (iblank[o] != 1) return fail(-1, "ghostCellMark set on a fluid cell");
                    f |= FB_GM;
                }
                const bool inside = i >= 1 && i <= nxc && j >= 1 && j <= nyc && k >= 1 && k <= nzc;
                const int idx3[3] = {i, j, k};
                const int lim[3] = {nxc, nyc, nzc};
                for (int q = 0; q < 6; ++q) {
                    const int ax = q / 2, hi = q % 2;
                    const bool bnd = hi ? (idx3[ax] == lim[ax]) : (idx3[ax] == 1);
                    int v = f6[q][o];
                    if (inside && bnd) v = side[q];
                    else if (inside && v != 0 && v != 1) return fail(-1, "interior face flags must be 0 or 1");
                    if (inside && v == 1) f |= (hi ? fb_plus(ax) : fb_minus(ax));
                }
                fl[o] = f;
            }
    if (nsolid > 0 && c.p.internal_boundary_present != 1)
        return fail(-1, "iblank has solid cells but internal_boundary_present is 0");
    CK(cudaMemcpyAsync(c.L1.fl, fl.data(), nf, cudaMemcpyHostToDevice, c.s));
    // level-1 coefficients; Dirichlet at the finest level
    const int N[3] = {nx, ny, nz};
    for (int a = 0; a < 3; ++a) {
        TRY(build_coef(c, c.L1, a, 1, N[a], side[2 * a] == -1, side[2 * a + 1] == -1));
        c.L1.dlo[a] = (c.p.pbc[2 * a] == PBC_DIRICHLET && dir_any && !(c.p.ndim == 2 && a == 2)) ? 1 : 0;
        c.L1.dhi[a] = (c.p.pbc[2 * a + 1] == PBC_DIRICHLET && dir_any && !(c.p.ndim == 2 && a == 2)) ? 1 : 0;
    }
    // coarse hierarchy per direction: iblank products, face flags, coefficients
    int sb[6];
    for (int q = 0; q < 6; ++q) sb[q] = (c.p.pbc[q] == PBC_DIRICHLET) ? 0 : 1;
    for (int d = 0; d < c.nd; ++d) {
        for (int l = 2; l <= c.nlev[d]; ++l) {
            Level &L = c.C[d][l];
            Level &F = level_of(c, d, l - 1);
            launch_coarse_iblank(L.fl, F.fl, L.d, F.d, d, c.s);
            launch_coarse_flags(L.fl, L.d, sb, c.s);
            for (int a = 0; a < 3; ++a) {
                const int lv = (a == d) ? l : 1;
                TRY(build_coef(c, L, a, lv, L.d.m[a], c.p.pbc[2 * a] == PBC_DIRICHLET,
                               c.p.pbc[2 * a + 1] == PBC_DIRICHLET));
            }
        }
        for (int l = 1; l < c.nlev[d]; ++l) TRY(build_transfer(c, c.T[d][l], d, l));
    }
    // line factorisations of every level and direction and, when the cycle
    // runs in FP64, the factored partition tables of the FP64 smoother
    auto factor = [&](Level &L, bool fp64_level) -> int {
        for (int a = 0; a < c.nd; ++a) {
            FactorArgs<double> fa;
            fa.fl = L.fl; fa.c = coef_of<double>(L); fa.d = L.d;
            fa.binv64 = L.binv64[a]; fa.gam64 = L.gam64[a]; fa.binv32 = L.binv32[a]; fa.gam32 = L.gam32[a];
            launch_factor(a, fa, c.s);
            const long long nt = fp64_level ? wpf_table_doubles(a, L.d) : 0;
            if (nt > 0) {
                if (!L.wpf[a]) TRY(c.alloc(&L.wpf[a], (size_t)nt));
                launch_wpf_setup(a, fa, L.wpf[a], c.s);
            }
        }
        return 0;
    };
    const bool all64 = (c.p.precision_mode == 0);
    TRY(factor(c.L1, all64));
    for (int d = 0; d < c.nd; ++d)
        for (int l = 2; l <= c.nlev[d]; ++l) TRY(factor(c.C[d][l], all64));
    // ghost gather list: linear indices in the level-1 layout; the ghost's own
    // stencil entry carries uNormal (0) and is marked -1.
    static const int incI[8] = {0, 0, 1, 1, 0, 0, 1, 1}, incJ[8] = {0, 1, 1, 0, 0, 1, 1, 0},
                     incK[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    c.nGhost = nGhost;
    if (nGhost > 0) {
        std::vector<long long> gi(nGhost), si(8 * (size_t)nGhost);
        std::vector<int> sg(8 * (size_t)nGhost);
        std::vector<float> cf(8 * (size_t)nGhost);
        for (int n = 0; n < nGhost; ++n) {
            const int ig = iGhost[n], jg = jGhost[n], kg = kGhost[n];
            if (ig < 1 || ig > nxc || jg < 1 || jg > nyc || kg < 1 || kg > nzc)
                return fail(-3, "ghost cell index out of range");
            if (!(fl[d1.idx(ig, jg, kg)] & FB_GM)) return fail(-3, "ghost list entry without ghostCellMark");
            gi[n] = d1.idx(ig, jg, kg);
            for (int r = 0; r < 8; ++r) {
                const int ii = iCellIndex[n] + incI[r], jj = jCellIndex[n] + incJ[r], kk = kCellIndex[n] + incK[r];
                if (ii < 0 || ii > nx || jj < 0 || jj > ny || kk < 0 || kk > nz)
                    return fail(-3, "image-point stencil outside (0:nx,0:ny,0:nz)");
                si[8 * (size_t)n + r] = (ii == ig && jj == jg && kk == kg) ? -1 : d1.idx(ii, jj, kk);
                cf[8 * (size_t)n + r] = (float)coeffGCMN[8 * (size_t)n + r];
            }
        }
        {   // stencil entries that are ghost cells refer to the ghost's number
            std::unordered_map<long long, int> gnum;
            gnum.reserve(2 * (size_t)nGhost);
            for (int n = 0; n < nGhost; ++n) gnum.emplace(gi[n], n);
            for (size_t e = 0; e < si.size(); ++e) {
                if (si[e] < 0) { sg[e] = -1; continue; }
                auto f = gnum.find(si[e]);
                sg[e] = (f != gnum.end()) ? -(f->second + 2) : (int)si[e];
            }
        }
        // ghost-ghost couplings in CSR form (the sweeps of the cluster kernel read only these)
        std::vector<int> ggp(nGhost + 1, 0), ggi;
        std::vector<double> ggc;
        for (int n = 0; n < nGhost; ++n) {
            for (int r = 0; r < 8; ++r) {
                const int e = sg[8 * (size_t)n + r];
                if (e <= -2) { ggi.push_back(-e - 2); ggc.push_back(coeffGCMN[8 * (size_t)n + r]); }
            }
            ggp[n + 1] = (int)ggi.size();
        }
        std::vector<float> ggcf(ggc.begin(), ggc.end());
        if ((long long)ggi.size() >= (1LL << 27)) return fail(-3, "too many ghost-ghost couplings");
        if (nGhost > c.ghost_cap || (int)ggi.size() > c.gg_cap) {
            for (void *q : {(void *)c.gg_ptr, (void *)c.gg_idx, (void *)c.ggc64, (void *)c.ggc32}) {
                auto it = std::find(c.allocs.begin(), c.allocs.end(), q);
                if (q && it != c.allocs.end()) { cudaFree(q); c.allocs.erase(it); }
            }
            const int cap = nGhost + nGhost / 4 + 64, ecap = std::max(8 * cap, (int)ggi.size() + 64);
            TRY(c.alloc(&c.gg_ptr, (size_t)cap + 1));
            TRY(c.alloc(&c.gg_idx, (size_t)ecap));
            TRY(c.alloc(&c.ggc64, (size_t)ecap));
            TRY(c.alloc(&c.ggc32, (size_t)ecap));
            c.gg_cap = ecap;
        }
        CK(cudaMemcpyAsync(c.gg_ptr, ggp.data(), ggp.size() * 4, cudaMemcpyHostToDevice, c.s));
        if (!ggi.empty()) {
            CK(cudaMemcpyAsync(c.gg_idx, ggi.data(), ggi.size() * 4, cudaMemcpyHostToDevice, c.s));
            CK(cudaMemcpyAsync(c.ggc64, ggc.data(), ggc.size() * 8, cudaMemcpyHostToDevice, c.s));
            CK(cudaMemcpyAsync(c.ggc32, ggcf.data(), ggcf.size() * 4, cudaMemcpyHostToDevice, c.s));
        }
        CK(cudaStreamSynchronize(c.s));
        if (nGhost > c.ghost_cap) {   // grow-only ghost buffers (body motion changes nGhost)
            for (void *q : {(void *)c.gidx, (void *)c.sidx, (void *)c.gco64, (void *)c.gco32, (void *)c.gscr64,
                            (void *)c.gscr32, (void *)c.gsg}) {
                auto it = std::find(c.allocs.begin(), c.allocs.end(), q);
                if (q && it != c.allocs.end()) { cudaFree(q); c.allocs.erase(it); }
            }
            const int cap = nGhost + nGhost / 4 + 64;
            TRY(c.alloc(&c.gidx, cap));
            TRY(c.alloc(&c.sidx, 8 * (size_t)cap));
            TRY(c.alloc(&c.gco64, 8 * (size_t)cap));
            TRY(c.alloc(&c.gco32, 8 * (size_t)cap));
            TRY(c.alloc(&c.gsg, 8 * (size_t)cap));
            TRY(c.alloc(&c.gscr64, 3 * (size_t)cap));   // two ping-pong buffers and the rows' fixed parts
            TRY(c.alloc(&c.gscr32, 3 * (size_t)cap));
            c.ghost_cap = cap;
        }
        CK(cudaMemcpyAsync(c.gidx, gi.data(), gi.size() * 8, cudaMemcpyHostToDevice, c.s));
        CK(cudaMemcpyAsync(c.sidx, si.data(), si.size() * 8, cudaMemcpyHostToDevice, c.s));
        CK(cudaMemcpyAsync(c.gsg, sg.data(), sg.size() * 4, cudaMemcpyHostToDevice, c.s));
        CK(cudaMemcpyAsync(c.gco64, coeffGCMN, 8 * (size_t)nGhost * 8, cudaMemcpyHostToDevice, c.s));
        CK(cudaMemcpyAsync(c.gco32, cf.data(), cf.size() * 4, cudaMemcpyHostToDevice, c.s));
        CK(cudaStreamSynchronize(c.s));
    }
    // boundary pressure gradients and the compatibility switch
    std::vector<double> pg(c.npgrad, 0.0);
    if (pgrad) std::memcpy(pg.data(), pgrad, c.npgrad * 8);
    CK(cudaMemcpyAsync(c.pgrad, pg.data(), c.npgrad * 8, cudaMemcpyHostToDevice, c.s));
    c.compat_active = false;
    for (int q = 0; q < 6; ++q) c.compat_active |= (c.p.bc[q] == BC_ZERO_GRADIENT);
    bool nz_pg = false;
    for (double v : pg) nz_pg |= (v != 0.0);
    c.nlw0_nonzero = c.compat_active || nz_pg;
    if (c.compat_active && !(c.p.outflow_area > 0.0)) return fail(-1, "outflow_area must be > 0 with zero-gradient BCs");
    CK(cudaStreamSynchronize(c.s));
    if (c.graph) { cudaGraphExecDestroy(c.graph); c.graph = nullptr; }
    if (c.pgraph) { cudaGraphExecDestroy(c.pgraph); c.pgraph = nullptr; }
    c.vg_on = false;   // the ghost list changed: velocity ghosts are registered again
    c.geometry = true;
    c.n1_ready = false;   // the unit-shift term follows the flags
    return 0;
}

int fsi_mg_solve_device(void *handle, double *d_pPrime, const double *d_nlu0, double *d_nlw0_out, int *iters,
                        double *maxres, int *loc, double *compTime)
{
    if (!handle || !d_pPrime || !d_nlu0) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    int rc = solve_device(c, d_pPrime, d_nlu0, iters, maxres, loc, compTime);
    if (rc < 0) return rc;
    if (d_nlw0_out) {
        if (c.nlw0_nonzero) cudaMemcpyAsync(d_nlw0_out, c.nlw0, c.L1.d.count() * 8, cudaMemcpyDeviceToDevice, c.s);
        else cudaMemsetAsync(d_nlw0_out, 0, c.L1.d.count() * 8, c.s);
        CK(cudaStreamSynchronize(c.s));
    }
    return rc;
}

int fsi_mg_solve(void *handle, double *pPrime, const double *nlu0, double *nlw0_out, int *iters, double *maxres,
                 int *loc, double *compTime)
{
    if (!handle || !pPrime || !nlu0) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    const long long n = c.L1.d.count();
    double *dp = c.stage, *db = c.stage + n;
    CK(cudaEventRecord(c.ev2, c.s));
    CK(cudaMemcpyAsync(dp, pPrime, n * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(db, nlu0, n * 8, cudaMemcpyHostToDevice, c.s));
    int rc = solve_device(c, dp, db, iters, maxres, loc, compTime);
    if (rc < 0) return rc;
    CK(cudaMemcpyAsync(pPrime, dp, n * 8, cudaMemcpyDeviceToHost, c.s));
    if (nlw0_out) {
        // without an outflow term the device buffer is zeroed and copied: a device memset and
        // a copy take well under the time of zeroing the host array on the CPU
        if (!c.nlw0_nonzero) CK(cudaMemsetAsync(c.nlw0, 0, n * 8, c.s));
        CK(cudaMemcpyAsync(nlw0_out, c.nlw0, n * 8, cudaMemcpyDeviceToHost, c.s));
    }
    CK(cudaEventRecord(c.ev3, c.s));
    CK(cudaStreamSynchronize(c.s));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, c.ev2, c.ev3));
    c.last_e2e = 1e-3 * (double)ms;   // includes the host<->device copies
    return rc;
}

int fsi_mg_mg_solver(void *handle, double *var, const double *rr, double *compTime)
{
    if (!handle || !var || !rr) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    const long long n = c.L1.d.count();
    double *dp = c.stage, *db = c.stage + n;
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaMemcpyAsync(dp, var, n * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(db, rr, n * 8, cudaMemcpyHostToDevice, c.s));
    mg_solver<double>(c, dp, db, false);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(var, dp, n * 8, cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    if (compTime) *compTime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

int fsi_mg_calc_residual(void *handle, const double *var, const double *r, double *resm, int *loc)
{
    if (!handle || !var || !r) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    const long long n = c.L1.d.count();
    double *dp = c.stage, *db = c.stage + n;
    CK(cudaMemcpyAsync(dp, var, n * 8, cudaMemcpyHostToDevice, c.s));
    CK(cudaMemcpyAsync(db, r, n * 8, cudaMemcpyHostToDevice, c.s));
    calc_residual(c, dp, db, nullptr);
    CK(cudaMemcpyAsync(c.h_result, c.result, sizeof(MaxLoc), cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    if (resm) *resm = c.h_result->v;
    loc_of(c, c.h_result->i, loc);
    return 0;
}

int fsi_mg_subtract_average(void *handle, double *pPrime)
{
    if (!handle || !pPrime) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    const long long n = c.L1.d.count();
    double *dp = c.stage;
    CK(cudaMemcpyAsync(dp, pPrime, n * 8, cudaMemcpyHostToDevice, c.s));
    subtract_average(c, dp);
    CK(cudaMemcpyAsync(pPrime, dp, n * 8, cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

int fsi_mg_subtract_average_noalloc(double *d_pPrime, const int8_t *d_iblank, const double *d_dx, const double *d_dy,
                                    const double *d_dz, int ndim, int nx, int ny, int nz, void *stream)
{
    if (!d_pPrime || !d_iblank || !d_dx || !d_dy || !d_dz) return fail(-1, "null argument");
    if (ndim != 2 && ndim != 3) return fail(-1, "ndim must be 2 or 3");
    if (nx < 3 || ny < 3 || nz < 2) return fail(-1, "grid too small");
    if (ndim == 2 && nz != 2) return fail(-1, "2D grids have nz = 2");
    if ((long long)(nx + 1) * (ny + 1) * (nz + 1) >= (1LL << 31))
        return fail(-1, "grid too large: the (0:nx+1,0:ny+1,0:nz+1) layout must hold fewer than 2^31 cells");
    const long long rows = (long long)(ny - 1) * (nz - 1);
    if (rows > NOALLOC_MAX_ROWS)
        return fail(-1, "fsi_mg_subtract_average_noalloc: the grid has " + std::to_string(rows) +
                            " (j,k) rows, (ny-1)*(nz-1); its fixed scratch holds at most " +
                            std::to_string(NOALLOC_MAX_ROWS) + " (use fsi_mg_subtract_average)");
    Dims d;
    d.m[0] = nx; d.m[1] = ny; d.m[2] = nz;
    d.sx = nx + 2;
    d.sxy = (long long)(nx + 2) * (ny + 2);
    // the kernels read d_iblank as it is: a cell is blanked where it is non-zero
    const cudaError_t e = launch_subtract_average_noalloc(d_pPrime, reinterpret_cast<const uint8_t *>(d_iblank),
                                                          d_dx, d_dy, d_dz, d, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return fail(-10, std::string("fsi_mg_subtract_average_noalloc: ") + cudaGetErrorString(e));
    return 0;
}

int fsi_mg_set_fresh_cells(void *handle, const int8_t *fresh_cell)
{
    if (!handle) return fail(-1, "null handle");
    Ctx &c = *(Ctx *)handle;
    if (!fresh_cell) { c.fresh_on = false; return 0; }
    const long long n = c.L1.d.count();
    long long nfresh = 0;
    for (long long q = 0; q < n; ++q) {
        if (fresh_cell[q] != 0 && fresh_cell[q] != 1) return fail(-3, "fresh_cell values must be 0 or 1");
        nfresh += fresh_cell[q];
    }
    if (!c.fresh) TRY(c.alloc(&c.fresh, (size_t)n));
    CK(cudaMemcpyAsync(c.fresh, fresh_cell, (size_t)n, cudaMemcpyHostToDevice, c.s));
    CK(cudaStreamSynchronize(c.s));
    c.fresh_on = nfresh > 0;
    return 0;
}

int fsi_mg_correct_pressure(void *handle, double *pPrime, double *nlw0_out)
{
    if (!handle || !pPrime) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    const long long n = c.L1.d.count();
    double *dp = c.stage;
    CK(cudaMemcpyAsync(dp, pPrime, n * 8, cudaMemcpyHostToDevice, c.s));
    correct_pressure(c, dp, c.nlw0);
    CK(cudaMemcpyAsync(pPrime, dp, n * 8, cudaMemcpyDeviceToHost, c.s));
    if (nlw0_out) {
        // without an outflow term the device buffer is zeroed and copied: a device memset and
        // a copy take well under the time of zeroing the host array on the CPU
        if (!c.nlw0_nonzero) CK(cudaMemsetAsync(c.nlw0, 0, n * 8, c.s));
        CK(cudaMemcpyAsync(nlw0_out, c.nlw0, n * 8, cudaMemcpyDeviceToHost, c.s));
    }
    CK(cudaStreamSynchronize(c.s));
    return 0;
}


int fsi_mg_get_pgrad(void *handle, double *pgrad)
{
    if (!handle || !pgrad) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    CK(cudaMemcpyAsync(pgrad, c.pgrad, c.npgrad * 8, cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

int fsi_mg_level_count(void *handle, int d)
{
    if (!handle || d < 0 || d > 2) return fail(-1, "bad argument");
    return ((Ctx *)handle)->nlev[d];
}

int fsi_mg_level_size(void *handle, int d, int n)
{
    if (!handle || d < 0 || d > 2) return fail(-1, "bad argument");
    Ctx &c = *(Ctx *)handle;
    if (n < 1 || n > c.nlev[d]) return fail(-1, "bad level");
    return c.mgrid[d][n];
}

int fsi_mg_debug_level_op(void *handle, int op, int d, int n, void *a, void *b, void *cc)
{
    if (!handle) return fail(-1, "null handle");
    Ctx &c = *(Ctx *)handle;
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    if (d < 0 || d >= c.nd || n < 1 || n > c.nlev[d]) return fail(-1, "bad level");
    Level &L = level_of(c, d, n);
    const long long nl = L.d.count();
    double *t0 = nullptr, *t1 = nullptr, *t2 = nullptr;
    TRY(c.alloc(&t0, nl));
    TRY(c.alloc(&t1, nl));
    int rc = 0;
    switch (op) {
    case 0:   // MG_itsolv
        TRY(copy_level(c, L, t0, a, true));
        TRY(copy_level(c, L, t1, b, true));
        itsolv<double>(c, L, t0, t1, n == 1, false);
        TRY(copy_level(c, L, t0, a, false));
        break;
    case 1: { // residual + restriction
        if (n == c.nlev[d]) return fail(-1, "no coarser level");
        Level &Cn = c.C[d][n + 1];
        TRY(c.alloc(&t2, Cn.d.count()));
        TRY(copy_level(c, L, t0, a, true));
        TRY(copy_level(c, L, t1, b, true));
        RestrictArgs<double> ra;
        ra.v = t0; ra.r = t1; ra.fl = L.fl; ra.c = coef_of<double>(L); ra.df = L.d; ra.dc = Cn.d;
        ra.w1 = c.T[d][n].rw1_64; ra.w2 = c.T[d][n].rw2_64; ra.rc = t2;
        launch_resid_restrict<double>(d, ra, c.s);
        TRY(copy_level(c, Cn, t2, cc, false));
        break;
    }
    case 2: { // prolongation + correction
        if (n == c.nlev[d]) return fail(-1, "no coarser level");
        Level &Cn = c.C[d][n + 1];
        TRY(c.alloc(&t2, Cn.d.count()));
        TRY(copy_level(c, Cn, t2, a, true));
        TRY(copy_level(c, L, t0, b, true));
        ProlongArgs<double> pa;
        pa.phi = t2; pa.flc = Cn.fl; pa.v = t0; pa.flf = L.fl; pa.df = L.d; pa.dc = Cn.d;
        Transfer &Tn = c.T[d][n];
        pa.cA = Tn.pcA; pa.cB = Tn.pcB; pa.wA = Tn.pwA64; pa.wB = Tn.pwB64; pa.mode = Tn.pmode;
        launch_prolong_correct<double>(d, pa, c.s);
        TRY(copy_level(c, L, t0, b, false));
        break;
    }
    case 3: { // coarse iblank
        std::vector<uint8_t> h(nl);
        CK(cudaMemcpy(h.data(), L.fl, nl, cudaMemcpyDeviceToHost));
        int8_t *out = (int8_t *)a;
        const long long hsx = L.d.m[0] + 1, hsxy = hsx * (L.d.m[1] + 1);
        for (int k = 0; k <= L.d.m[2]; ++k)
            for (int j = 0; j <= L.d.m[1]; ++j)
                for (int i = 0; i <= L.d.m[0]; ++i) out[i + hsx * j + hsxy * k] = (h[L.d.idx(i, j, k)] & FB_IB) ? 1 : 0;
        break;
    }
    case 4: { // face flags of level n in full (0:nx+1)^3 arrays, values -1/0/1 on the level's interior
        std::vector<uint8_t> h(nl);
        CK(cudaMemcpy(h.data(), L.fl, nl, cudaMemcpyDeviceToHost));
        const long long fsx = c.nx + 2, fsxy = fsx * (c.ny + 2), nfull = fsxy * (c.nz + 2);
        int8_t *out = (int8_t *)a;
        std::memset(out, 0, 6 * nfull);
        const int lim[3] = {L.d.m[0] - 1, L.d.m[1] - 1, L.d.m[2] - 1};
        for (int k = 1; k <= lim[2]; ++k)
            for (int j = 1; j <= lim[1]; ++j)
                for (int i = 1; i <= lim[0]; ++i) {
                    const uint8_t f = h[L.d.idx(i, j, k)];
                    const int idx3[3] = {i, j, k};
                    for (int q = 0; q < 6; ++q) {
                        const int ax = q / 2, hi = q % 2;
                        const bool bnd = hi ? idx3[ax] == lim[ax] : idx3[ax] == 1;
                        int v = (f & (hi ? fb_plus(ax) : fb_minus(ax))) ? 1 : 0;
                        if (bnd) v = (n == 1) ? c.side_raw[q] : ((c.p.pbc[q] == PBC_DIRICHLET) ? -1 : 1);
                        out[q * nfull + i + fsx * j + fsxy * k] = (int8_t)v;
                    }
                }
        break;
    }
    case 5: { // ghost rows on a level-1 array
        TRY(copy_level(c, L, t0, a, true));
        CK(cudaMemsetAsync(c.d_iters, 0, sizeof(int), c.s));
        if (c.nGhost > 0) {
            GhostArgs g{c.nGhost, c.gidx, c.sidx, c.gsg, c.gg_ptr, c.gg_idx};
            launch_ghost_rows<double>(t0, g, c.gco64, c.ggc64, c.gscr64, c.p.iterMax_ad, c.p.restol_ad, 0.0, c.d_iters,
                                      c.d_maxd, c.s);
        }
        TRY(copy_level(c, L, t0, a, false));
        if (b) CK(cudaMemcpy(b, c.d_iters, sizeof(int), cudaMemcpyDeviceToHost));
        break;
    }
    case 6: // outer ghost layer
        TRY(copy_level(c, L, t0, a, true));
        launch_outer_ghost<double>(t0, L.d, c.sign, c.s);
        TRY(copy_level(c, L, t0, a, false));
        break;
    case 7: { // MG_itsolv in FP32 (the mixed form's smoother): inputs rounded to FP32, result widened
        TRY(copy_level(c, L, t0, a, true));
        TRY(copy_level(c, L, t1, b, true));
        float *f0 = nullptr, *f1 = nullptr;
        TRY(c.alloc(&f0, nl));
        TRY(c.alloc(&f1, nl));
        launch_convert_d2f(f0, t0, nl, c.s);
        launch_convert_d2f(f1, t1, nl, c.s);
        itsolv<float>(c, L, f0, f1, n == 1, false);
        launch_convert_f2d(t0, f0, nl, c.s);
        TRY(copy_level(c, L, t0, a, false));
        CK(cudaStreamSynchronize(c.s));
        for (float *t : {f1, f0}) {
            auto it = std::find(c.allocs.begin(), c.allocs.end(), (void *)t);
            if (it != c.allocs.end()) { cudaFree(t); c.allocs.erase(it); }
        }
        break;
    }
    default:
        rc = fail(-1, "unknown op");
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c.s));
    // release the temporaries (they were appended last)
    for (double *t : {t2, t1, t0}) {
        if (!t) continue;
        auto it = std::find(c.allocs.begin(), c.allocs.end(), (void *)t);
        if (it != c.allocs.end()) { cudaFree(t); c.allocs.erase(it); }
    }
    return rc;
}

int fsi_mg_time_kernel(void *handle, int which, int precision, int reps, double *avg_ms, double *alg_bytes)
{
    if (!handle || !avg_ms || reps < 1) return fail(-1, "bad argument");
    Ctx &c = *(Ctx *)handle;
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    const bool f32 = (precision == 1);
    const long long n1 = c.L1.d.count();
    const double cells = (double)(c.nx - 1) * (c.ny - 1) * (c.nz - 1);
    const double eb = f32 ? 4.0 : 8.0;
    double *p = c.stage, *b = c.stage + n1;
    if (f32) {   // FP32 copies of the level-1 fields
        launch_convert_d2f(c.e32, p, n1, c.s);
        launch_convert_d2f(c.r32, b, n1, c.s);
    }
    double dfma_flops = 0.0;
    auto once = [&]() {
        if (which >= 0 && which <= 2) {
            if (which >= c.nd) return;
            const int dir = which;
            auto go = [&](auto *v, const auto *r, auto tag) {
                using T = decltype(tag);
                LineArgs<T> a;
                a.v = (T *)v; a.r = (const T *)r; a.fl = c.L1.fl; a.U = scratch_U<T>(c); a.c = coef_of<T>(c.L1);
                a.d = c.L1.d; a.omega = (T)c.p.omega; a.binv = lv_binv<T>(c.L1, dir); a.gam = lv_gam<T>(c.L1, dir);
                a.wpf = std::is_same<T, double>::value ? c.L1.wpf[dir] : nullptr;
                a.dir_lo = a.dir_hi = 0; a.ppp_lo = a.ppp_hi = T(0); a.colour = 0;
                launch_line<T>(dir, a, c.p.omega == 1.0, c.s);
            };
            if (f32) go(c.e32, c.r32, 0.0f); else go(p, b, 0.0);
        } else if (which == 3 && c.nlev[0] > 1) {
            auto go = [&](auto *v, const auto *r, auto tag) {
                using T = decltype(tag);
                Level &Cn = c.C[0][2];
                RestrictArgs<T> a;
                a.v = (const T *)v; a.r = (const T *)r; a.fl = c.L1.fl; a.c = coef_of<T>(c.L1); a.df = c.L1.d;
                a.dc = Cn.d; a.w1 = rw1<T>(c.T[0][1]); a.w2 = rw2<T>(c.T[0][1]); a.rc = lv_r<T>(Cn);
                launch_resid_restrict<T>(0, a, c.s);
            };
            if (f32) go(c.e32, c.r32, 0.0f); else go(p, b, 0.0);
        } else if (which == 4 && c.nlev[0] > 1) {
            auto go = [&](auto *v, auto tag) {
                using T = decltype(tag);
                Level &Cn = c.C[0][2];
                ProlongArgs<T> a;
                a.phi = lv_v<T>(Cn); a.flc = Cn.fl; a.v = (T *)v; a.flf = c.L1.fl; a.df = c.L1.d; a.dc = Cn.d;
                Transfer &T1 = c.T[0][1];
                a.cA = T1.pcA; a.cB = T1.pcB; a.wA = pwA<T>(T1); a.wB = pwB<T>(T1); a.mode = T1.pmode;
                launch_prolong_correct<T>(0, a, c.s);
            };
            if (f32) go(c.e32, 0.0f); else go(p, 0.0);
        } else if (which == 5) {
            calc_residual(c, p, b, f32 ? c.r32 : nullptr);
        } else if (which == 6 && c.have_fv) {
            launch_face_vel_rhs(c.last_fv, c.last_fv_vk, c.step_partials, c.step_cap, (double *)c.result, c.s);
        } else if (which == 7 && c.have_cv) {
            launch_correct_vel(c.last_cv, c.s);
        } else if (which == 8 && c.have_up) {
            launch_update_pressure(c.last_up_p, c.last_up_pp, c.L1.d.sxy * (c.nz + 2), c.last_up_vk, c.s);
        } else if (which == 9 && c.have_ad) {
            launch_rhs_advec_diff(c.last_ad, c.s);
        } else if (which == 10) {
            dfma_flops = launch_dfma_peak(c.stage, c.s);
        }
    };
    if ((which == 6 && !c.have_fv) || (which == 7 && !c.have_cv) || (which == 8 && !c.have_up) ||
        (which == 9 && !c.have_ad))
        return fail(-1, "time_kernel 6/7/8 replay the last face_vel_rhs/correct_vel/update_pressure call; make one first");
    once();   // warm-up
    CK(cudaEventRecord(c.ev0, c.s));
    for (int r = 0; r < reps; ++r) once();
    CK(cudaEventRecord(c.ev1, c.s));
    CK(cudaEventSynchronize(c.ev1));
    CK(cudaGetLastError());
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
    *avg_ms = (double)ms / reps;
    if (alg_bytes) {
        // algorithmic bytes per launch: one colour of a line sweep updates half the cells,
        // reading rhs, flags and the other colour's values and writing the new values;
        // residual+restriction reads var, rhs, flags and writes half a coarse cell per fine
        // cell; prolongation+correction reads half a coarse cell, flags, var and writes var;
        // calc_residual reads p, b, flags (and writes the FP32 residual in mixed mode).
        double bpc = 0.0;
        if (which <= 2) bpc = 0.5 * (eb + 1.0 + eb + eb);
        else if (which == 3) bpc = eb + eb + 1.0 + 0.5 * eb;
        else if (which == 4) bpc = 0.5 * eb + 1.0 + eb + eb;
        else if (which == 5) bpc = 8.0 + 8.0 + 1.0 + (f32 ? 4.0 : 0.0);
        // step routines (FP64): face_vel_rhs reads u, v, w (+ p with VAN_KAN) and the flags
        // and writes three faces and nlu0; correct_vel reads pPrime and the flags, updates
        // u, v, w and three faces; update_pressure reads pPrime (+ p) and writes p; each
        // non-null bc array adds a read
        else if (which == 6) {
            bpc = 24.0 + 1.0 + 24.0 + 8.0 + (c.last_fv_vk ? 8.0 : 0.0);
            for (int d = 0; d < 3; ++d) bpc += c.last_fv.bc[d] ? 8.0 : 0.0;
        } else if (which == 7) {
            bpc = 8.0 + 1.0 + 48.0 + 48.0;
            for (int d = 0; d < 3; ++d) bpc += c.last_cv.bc[d] ? 8.0 : 0.0;
        } else if (which == 8) {
            bpc = 16.0 + (c.last_up_vk ? 8.0 : 0.0);
        } else if (which == 9) {
            // u, v, w, three faces, viscTot, flags read; nlu, nlv, nlw written; AB2 history read + written,
            // exp_weight, p (VAN_KAN) and the non-null bc arrays read
            const RhsAdArgs &A = c.last_ad;
            bpc = 24.0 + 24.0 + 8.0 + 1.0 + 24.0 + (A.ab2 ? 48.0 + (A.ew ? 8.0 : 0.0) : 0.0) + (A.vankan ? 8.0 : 0.0);
            for (int q = 0; q < 9; ++q) bpc += A.bc[q] ? 8.0 : 0.0;
            for (int q = 0; q < 3; ++q) bpc += A.bcvisc[q] ? 8.0 : 0.0;
        }
        *alg_bytes = (which == 10) ? dfma_flops : bpc * cells;
    }
    return 0;
}

int fsi_mg_residual_history(void *handle, double *out, int cap)
{
    if (!handle) return fail(-1, "null handle");
    Ctx &c = *(Ctx *)handle;
    const int n = (int)c.hist.size();
    if (out)
        for (int q = 0; q < n && q < cap; ++q) out[q] = c.hist[q];
    return n;
}

int fsi_mg_stats(void *handle, double *out, int n)
{
    if (!handle || !out) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    const double v[8] = {(double)c.last_iters, c.last_maxres, c.last_time, (double)c.ghost_sweeps, (double)c.launches,
                         (double)c.bytes, c.last_wall, c.last_e2e};
    for (int q = 0; q < n && q < 8; ++q) out[q] = v[q];
    return 0;
}

int fsi_mg_line_timing(void *handle, int enable, double *out)
{
    if (!handle) return fail(-1, "null handle");
    Ctx &c = *(Ctx *)handle;
    if (enable >= 0 && (enable != 0) != c.lt_on) {
        CK(cudaStreamSynchronize(c.s));
        if (enable && c.lt_ev.empty()) {
            c.lt_ev.resize(2048);
            c.lt_f32.assign(1024, 0);
            for (auto &e : c.lt_ev) CK(cudaEventCreate(&e));
        }
        c.lt_on = enable != 0;
        // the solve graphs are re-captured with (or without) the event records
        if (c.graph) { cudaGraphExecDestroy(c.graph); c.graph = nullptr; }
        if (c.pgraph) { cudaGraphExecDestroy(c.pgraph); c.pgraph = nullptr; }
        c.graph_lt0 = c.graph_lt1 = c.pgraph_lt0 = c.pgraph_lt1 = 0;
    }
    if (enable == 1) {
        c.lt_ms[0] = c.lt_ms[1] = 0.0;
        c.lt_n[0] = c.lt_n[1] = 0;
    }
    if (out) {
        // algorithmic bytes of one colour of a level-1 line sweep: the colour's
        // rhs, flags and new values plus the other colour's values, and with a
        // relaxation omega != 1 the colour's old values (var (1 - omega) + omega sol)
        const double cells = (double)(c.nx - 1) * (c.ny - 1) * (c.p.ndim == 3 ? c.nz - 1 : 1);
        const double relaxed = (c.p.omega != 1.0) ? 1.0 : 0.0;
        out[0] = (double)c.lt_n[1];
        out[1] = c.lt_ms[1];
        out[2] = 0.5 * (4.0 + 1.0 + 4.0 + 4.0 + 4.0 * relaxed) * cells;
        out[3] = (double)c.lt_n[0];
        out[4] = c.lt_ms[0];
        out[5] = 0.5 * (8.0 + 1.0 + 8.0 + 8.0 + 8.0 * relaxed) * cells;
    }
    return 0;
}

void fsi_mg_destroy(void *handle)
{
    delete (Ctx *)handle;
}

} // extern "C"
