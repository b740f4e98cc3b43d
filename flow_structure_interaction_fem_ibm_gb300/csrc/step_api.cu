// Fractional-step entry points of the C ABI (include/fsi_mg.h) on device
// arrays: face_vel + rhs_poisson, correct_vel, set_bc, the momentum predictor
// (rhs_advec_diff, rhs_adjust_bc, solve_ad), the ghost-cell velocities and
// update_pressure.  Each validates its arguments against the handle's
// geometry and queues the kernels of step_kernels.cu on the handle's stream.
#include "mg_context.h"

#include <cmath>
#include <cstring>

using namespace fsimg;

extern "C" {

// ---------------------------------------------------------------------------
// Fractional-step operations either side of the solve, on device arrays.
// ---------------------------------------------------------------------------
static int step_ready(Ctx &c)
{
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    for (int q = 0; q < 6; ++q)
        if (c.side_raw[q] == -1)
            return fail(-1, "face_vel/correct_vel/update_pressure need Neumann pressure sides (the reference "
                            "flags Dirichlet sides with -1 in iup/ium, which these kernels do not carry)");
    return 0;
}

// one partial sum per CTA of the step reductions; worst case one CTA per
// 32 x 8 tile and k of face_vel_rhs
static int ensure_step_partials(Ctx &c)
{
    if (c.step_partials) return 0;
    c.step_cap = ((c.nx - 1 + 31) / 32) * ((c.ny - 1 + 7) / 8) * (c.nz - 1);
    return c.alloc(&c.step_partials, (size_t)c.step_cap);
}

static StepArgs step_args(Ctx &c, double dt)
{
    StepArgs a{};
    a.fl = c.L1.fl;
    a.d = c.L1.d;
    a.dt = dt;
    a.dtinv = 1.0 / dt;   // dtinv = oned/dt (IBM/MAIN.F90:1627)
    a.gcm = (c.p.boundary_formulation == GCM_METHOD) ? 1 : 0;
    for (int d = 0; d < 3; ++d) {
        a.fx[d] = c.d_fx[d]; a.gx[d] = c.d_gx[d];
        a.dxinv[d] = c.d_dxinv[d]; a.dxcinv[d] = c.d_dxcinv[d]; a.dx[d] = c.d_dx[d];
    }
    return a;
}

int fsi_mg_face_vel_rhs(void *handle, int frac_step_type, double dt, const double *d_u, const double *d_v,
                        const double *d_w, const double *d_p, const double *d_bcxu, const double *d_bcyv,
                        const double *d_bczw, double *d_face_u, double *d_face_v, double *d_face_w, double *d_nlu0,
                        double *sum)
{
    if (!handle || !d_u || !d_v || !d_w || !d_face_u || !d_face_v || !d_face_w || !d_nlu0)
        return fail(-1, "null argument");
    if (frac_step_type != 0 && frac_step_type != 1) return fail(-1, "frac_step_type must be 0 (NO_VAN_KAN) or 1 (VAN_KAN)");
    if (frac_step_type == 1 && !d_p) return fail(-1, "VAN_KAN needs the current pressure p");
    if (!(dt > 0.0)) return fail(-1, "dt must be positive");
    Ctx &c = *(Ctx *)handle;
    TRY(step_ready(c));
    const long long n = c.L1.d.sxy * (c.nz + 2);   // full (0:nx+1,0:ny+1,0:nz+1) arrays
    StepArgs a = step_args(c, dt);
    const double *vel[3] = {d_u, d_v, d_w};
    const double *bc[3] = {d_bcxu, d_bcyv, d_bczw};
    double *face[3] = {d_face_u, d_face_v, d_face_w};
    // (zeroed by alloc; outside the interior uTilde stays zero, where the
    // reference keeps whatever its module array held: those values reach only
    // flagged faces, with weight zero, and the open z faces of a 2D grid)
    if (frac_step_type == 1 && !c.vtilde) TRY(c.alloc(&c.vtilde, (size_t)(3 * n)));
    for (int d = 0; d < 3; ++d) {
        a.vel[d] = vel[d]; a.bc[d] = bc[d]; a.face[d] = face[d];
        a.velo[d] = (frac_step_type == 1) ? c.vtilde + d * n : nullptr;
    }
    a.nlu0 = d_nlu0;
    a.p = d_p;
    TRY(ensure_step_partials(c));
    launch_face_vel_rhs(a, frac_step_type == 1, c.step_partials, c.step_cap, (double *)c.result, c.s);
    c.last_fv = a; c.last_fv_vk = (frac_step_type == 1); c.have_fv = true;
    c.launches += (frac_step_type == 1) ? 4 : 3;
    CK(cudaMemcpyAsync(c.h_result, c.result, sizeof(double), cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    if (sum) *sum = *(const double *)c.h_result;
    return 0;
}

int fsi_mg_correct_vel(void *handle, double dt, const double *d_pPrime, double *d_u, double *d_v, double *d_w,
                       const double *d_bcxu, const double *d_bcyv, const double *d_bczw, double *d_face_u,
                       double *d_face_v, double *d_face_w)
{
    if (!handle || !d_pPrime || !d_u || !d_v || !d_w || !d_face_u || !d_face_v || !d_face_w)
        return fail(-1, "null argument");
    if (!(dt > 0.0)) return fail(-1, "dt must be positive");
    Ctx &c = *(Ctx *)handle;
    TRY(step_ready(c));
    StepArgs a = step_args(c, dt);
    double *vel[3] = {d_u, d_v, d_w};
    const double *bc[3] = {d_bcxu, d_bcyv, d_bczw};
    double *face[3] = {d_face_u, d_face_v, d_face_w};
    for (int d = 0; d < 3; ++d) { a.vel[d] = vel[d]; a.velo[d] = vel[d]; a.bc[d] = bc[d]; a.face[d] = face[d]; }
    a.p = d_pPrime;
    launch_correct_vel(a, c.s);
    c.last_cv = a; c.have_cv = true;
    c.launches++;
    int rc = 0;
    if (c.vg_on && c.nGhost > 0) {   // GCM_vel_set_bc_internal (IBM/CORE_FRAC_STEP_ROUTINES.F90:373)
        CK(cudaMemsetAsync(c.d_iters, 0, sizeof(int), c.s));
        CK(cudaMemsetAsync(c.d_maxd, 0, sizeof(unsigned long long), c.s));
        GhostArgs g{c.nGhost, c.gidx, c.sidx, c.gsg, c.gg_ptr, c.gg_idx};
        launch_vel_ghosts(d_u, d_v, d_w, g, c.vg_coeff, c.vg_bi_set ? c.vg_bi : nullptr, c.vg_bw, c.vg_iw, c.vg_scr,
                          c.p.iterMax_ad, c.p.restol_ad, c.d_iters, c.d_maxd, c.s);
        c.launches++;
        int h_iters = 0;
        unsigned long long h_maxd = 0;
        CK(cudaMemcpyAsync(&h_iters, c.d_iters, sizeof(int), cudaMemcpyDeviceToHost, c.s));
        CK(cudaMemcpyAsync(&h_maxd, c.d_maxd, sizeof(h_maxd), cudaMemcpyDeviceToHost, c.s));
        CK(cudaStreamSynchronize(c.s));
        c.vg_last_iters = h_iters;
        double maxd;
        std::memcpy(&maxd, &h_maxd, sizeof(maxd));
        // the reference prints its non-convergence message and continues
        if (h_iters >= c.p.iterMax_ad && maxd > c.p.restol_ad) rc = 2;
    }
    CK(cudaStreamSynchronize(c.s));
    return rc;
}

int fsi_mg_set_bc(void *handle, const fsi_mg_bc_values *values, double *d_u, double *d_v, double *d_w,
                  double *const d_bc[9], double *correction_vel)
{
    if (!handle || !values || !d_u || !d_v || !d_w || !d_bc) return fail(-1, "null argument");
    for (int q = 0; q < 9; ++q)
        if (!d_bc[q]) return fail(-1, "set_bc needs all nine boundary-value arrays");
    Ctx &c = *(Ctx *)handle;
    TRY(step_ready(c));
    SetBcArgs a{};
    bool zero_gradient = false;
    const double pi = 4.0 * std::atan(1.0);   // IBM/MAIN.F90:264
    for (int s = 0; s < 6; ++s) {
        const int t = c.p.bc[s];
        if (t == 6) return fail(-1, "user-specified (Blasius) velocity boundaries are not supported");
        if (t != 1 && t != 2 && t != 3 && t != 4 && t != 7)
            return fail(-1, "velocity boundary type must be 1, 2, 3, 4 or 7");
        a.type[s] = t;
        zero_gradient |= (t == BC_ZERO_GRADIENT);
        for (int q = 0; q < 3; ++q) {
            const double amp = values->vel[s][q];
            double v = amp;
            if (t == 3) {   // pulsatile inflow: amp sin(2 pi freq time); x2 u gust switch (IBM/CORE_SET_BC.F90:96-106)
                const double arg = 2.0 * pi * values->freq[s][q] * values->time;
                v = amp * std::sin(arg);
                if (s == 1 && q == 0) v = (values->time > values->tstart_gust) ? amp * std::fabs(std::sin(arg)) : 0.0;
            }
            a.val[s][q] = v;
        }
    }
    if (zero_gradient && !(c.p.outflow_area > 0.0)) return fail(-1, "outflow_area must be > 0 with zero-gradient BCs");
    double *vel[3] = {d_u, d_v, d_w};
    for (int d = 0; d < 3; ++d) { a.vel[d] = vel[d]; a.xn[d] = c.d_xn[d]; a.dx[d] = c.d_dx[d]; }
    for (int q = 0; q < 9; ++q) a.bc[q] = d_bc[q];
    a.fl = c.L1.fl;
    a.d = c.L1.d;
    a.xout = values->xout;
    a.yout = values->yout;
    a.outflow_area = c.p.outflow_area;
    a.sums = (const double *)c.result;
    launch_set_bc_planes(a, c.s);
    c.launches++;
    if (zero_gradient) {
        TRY(ensure_step_partials(c));
        launch_bc_massflux(a, c.step_partials, c.step_cap, (double *)c.result, c.s);
        c.launches += 2;
    }
    for (int axis = 0; axis < 3; ++axis) launch_outer_ghost_vel(a, axis, zero_gradient, c.s);
    c.launches += 3;
    if (zero_gradient) CK(cudaMemcpyAsync(c.h_result, c.result, sizeof(double), cudaMemcpyDeviceToHost, c.s));
    CK(cudaStreamSynchronize(c.s));
    if (correction_vel) *correction_vel = zero_gradient ? -*(const double *)c.h_result / c.p.outflow_area : 0.0;
    return 0;
}

int fsi_mg_rhs_advec_diff(void *handle, int advec_scheme, int frac_step_type, double dt,
                          const fsi_mg_rhs_ad_fields *fl)
{
    if (!handle || !fl) return fail(-1, "null argument");
    if (advec_scheme < 1 || advec_scheme > 3) return fail(-1, "advec_scheme must be 1 (AB2), 2 or 3 (Crank-Nicolson)");
    if (frac_step_type != 0 && frac_step_type != 1) return fail(-1, "frac_step_type must be 0 (NO_VAN_KAN) or 1 (VAN_KAN)");
    if (!(dt > 0.0)) return fail(-1, "dt must be positive");
    Ctx &c = *(Ctx *)handle;
    TRY(step_ready(c));
    const bool three_d = (c.p.ndim == 3);
    if (!fl->u || !fl->v || !fl->face_u || !fl->face_v || !fl->viscTot || !fl->nlu || !fl->nlv ||
        (three_d && (!fl->w || !fl->face_w || !fl->nlw)))
        return fail(-1, "null field");
    if (advec_scheme == 1 && (!fl->nluOld || !fl->nlvOld || (three_d && !fl->nlwOld)))
        return fail(-1, "ADAMS_BASHFORTH2 needs nluOld, nlvOld (and nlwOld in 3D)");
    if (frac_step_type == 1 && (!fl->p || !fl->nlw)) return fail(-1, "VAN_KAN needs p and nlw");
    RhsAdArgs a{};
    a.vel[0] = fl->u; a.vel[1] = fl->v; a.vel[2] = fl->w;
    a.face[0] = fl->face_u; a.face[1] = fl->face_v; a.face[2] = fl->face_w;
    for (int q = 0; q < 9; ++q) a.bc[q] = fl->bc[q];
    a.visc = fl->viscTot;
    for (int q = 0; q < 3; ++q) a.bcvisc[q] = fl->bcvisc[q];
    a.ew = fl->exp_weight;
    a.nlold[0] = fl->nluOld; a.nlold[1] = fl->nlvOld; a.nlold[2] = fl->nlwOld;
    a.p = fl->p;
    a.nl[0] = fl->nlu; a.nl[1] = fl->nlv; a.nl[2] = fl->nlw;
    a.fl = c.L1.fl;
    for (int d = 0; d < 3; ++d) {
        a.fx[d] = c.d_fx[d]; a.gx[d] = c.d_gx[d]; a.dxinv[d] = c.d_dxinv[d];
        a.cm[d] = c.d_adm[d]; a.cp[d] = c.d_adp[d]; a.cb[d] = c.d_adb[d];
    }
    a.d = c.L1.d;
    a.dt = dt;
    a.ab2 = (advec_scheme == 1) ? 1 : 0;
    a.vankan = (frac_step_type == 1) ? 1 : 0;
    a.alfa = c.p.alfa;
    a.hybrid = (std::fabs(c.p.alfa) > 1.0e-3) ? 1 : 0;   // Hybrid (IBM/MAIN.F90:649-652)
    a.three_d = three_d ? 1 : 0;
    launch_rhs_advec_diff(a, c.s);
    c.last_ad = a; c.have_ad = true;
    c.launches++;
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

static int ad_coef_args(Ctx &c, int advec_scheme, double dt, const fsi_mg_rhs_ad_fields *fl, AdCoefArgs &a)
{
    if (advec_scheme < 1 || advec_scheme > 3)
        return fail(-1, "advec_scheme must be 1 (AB2), 2 (CRANK_NICOLSON1) or 3 (CRANK_NICOLSON2)");
    if (!(dt > 0.0)) return fail(-1, "dt must be positive");
    TRY(step_ready(c));
    const bool three_d = (c.p.ndim == 3);
    if (!fl || !fl->face_u || !fl->face_v || !fl->face_w || !fl->viscTot) return fail(-1, "null field");
    const long long n = c.L1.d.sxy * (c.nz + 2);
    if (!c.ad_co) TRY(c.alloc(&c.ad_co, (size_t)(8 * n)));
    a = AdCoefArgs{};
    a.face[0] = fl->face_u; a.face[1] = fl->face_v; a.face[2] = fl->face_w;
    a.visc = fl->viscTot;
    for (int q = 0; q < 3; ++q) a.bcvisc[q] = fl->bcvisc[q];
    for (int q = 0; q < 7; ++q) a.co[q] = c.ad_co + q * n;
    a.fl = c.L1.fl;
    for (int d = 0; d < 3; ++d) {
        a.fx[d] = c.d_fx[d]; a.gx[d] = c.d_gx[d]; a.dxinv[d] = c.d_dxinv[d];
        a.cm[d] = c.d_adm[d]; a.cp[d] = c.d_adp[d]; a.cb[d] = c.d_adb[d];
    }
    a.d = c.L1.d;
    a.dt = dt;
    a.half_dt = (advec_scheme == 1) ? 0.0 : 0.5 * dt;
    a.three_d = three_d ? 1 : 0;
    return 0;
}

int fsi_mg_rhs_adjust_bc(void *handle, int advec_scheme, double dt, const fsi_mg_rhs_ad_fields *fl)
{
    if (!handle || !fl) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    AdCoefArgs a;
    TRY(ad_coef_args(c, advec_scheme, dt, fl, a));
    if (!fl->nlu || !fl->nlv || !fl->nlw) return fail(-1, "null nlu/nlv/nlw");
    double *nl[3] = {fl->nlu, fl->nlv, fl->nlw};
    launch_rhs_adjust_bc(a, fl->bc, nl, c.s);
    c.launches++;
    CK(cudaStreamSynchronize(c.s));
    return 0;
}

int fsi_mg_solve_ad(void *handle, int advec_scheme, double dt, const fsi_mg_rhs_ad_fields *fl, double *d_u,
                    double *d_v, double *d_w, int *iters, double *maxres)
{
    if (!handle || !fl || !d_u || !d_v) return fail(-1, "null argument");
    Ctx &c = *(Ctx *)handle;
    AdCoefArgs a;
    TRY(ad_coef_args(c, advec_scheme, dt, fl, a));
    const bool three_d = (c.p.ndim == 3);
    const bool gcm_vel = (c.p.boundary_formulation == GCM_METHOD) && c.vg_on && c.nGhost > 0;
    if ((three_d || gcm_vel) && !d_w) return fail(-1, "null w (3D, or ghost-cell velocities)");
    if (!fl->nlu || !fl->nlv || (three_d && !fl->nlw)) return fail(-1, "null nlu/nlv/nlw");
    // the GCM branch's GCM_GhostCell_Vel re-balances zero-gradient outflow every
    // iteration (GCM_enforce_global_mass_consv); the branch without a body has no such step
    bool zero_gradient = false;
    for (int q = 0; q < 6; ++q) zero_gradient |= (c.p.bc[q] == BC_ZERO_GRADIENT);
    const bool mass_consv = zero_gradient && c.p.boundary_formulation == GCM_METHOD;
    // CRANK_NICOLSON2 re-evaluates face_vel of the current velocities after each set of
    // sweeps (IBM/CORE_SOLVE_AD.F90:155-157 and :236)
    const bool cn2 = (advec_scheme == 3);
    const long long n = c.L1.d.sxy * (c.nz + 2);
    StepArgs fv{};
    ZgArgs zg{};
    if (mass_consv)
        for (int q = 0; q < 9; ++q)
            if (!fl->bc[q]) return fail(-1, "solve_ad with zero-gradient sides and a GCM body needs all nine bc arrays");
    if (cn2 || mass_consv) {
        if (fl->p) return fail(-1, "solve_ad re-evaluates face_vel (CRANK_NICOLSON2, or zero-gradient sides with a "
                                   "GCM body), which is restated for NO_VAN_KAN only (fields.p must be NULL)");
        if (!d_w) return fail(-1, "null w");
        if (!c.zg_div) TRY(c.alloc(&c.zg_div, (size_t)n));
        TRY(ensure_step_partials(c));
        // face_vel into the step's faces (a missing bc array reads as 0); the divergence goes to
        // scratch, and with dt = 1 its sum is the net face flux of the outflow balance
        fv = step_args(c, 1.0);
        const double *vl[3] = {d_u, d_v, d_w};
        double *fc[3] = {const_cast<double *>(fl->face_u), const_cast<double *>(fl->face_v),
                         const_cast<double *>(fl->face_w)};
        for (int d = 0; d < 3; ++d) { fv.vel[d] = vl[d]; fv.bc[d] = fl->bc[4 * d]; fv.face[d] = fc[d]; }
        fv.nlu0 = c.zg_div;
    }
    if (mass_consv) {
        if (!(c.p.outflow_area > 0.0)) return fail(-1, "outflow_area must be > 0 with zero-gradient BCs");
        zg.nl[0] = fl->nlu; zg.nl[1] = fl->nlv; zg.nl[2] = fl->nlw;   // nlw may be NULL in 2D
        for (int q = 0; q < 9; ++q) zg.bc[q] = const_cast<double *>(fl->bc[q]);
        zg.fl = c.L1.fl;
        for (int d = 0; d < 3; ++d) { zg.cm[d] = c.d_adm[d]; zg.cp[d] = c.d_adp[d]; zg.cb[d] = c.d_adb[d]; }
        zg.sums = (const double *)c.result;
        for (int q = 0; q < 6; ++q) zg.type[q] = c.p.bc[q];
        zg.hdr = 0.50 * dt * fl->reinv;
        zg.outflow_area = c.p.outflow_area;
        zg.three_d = three_d ? 1 : 0;
        zg.d = c.L1.d;
    }
    double *gam = c.ad_co + 7 * n;
    launch_ad_coef(a, c.s);
    c.launches++;
    double *vel[3] = {d_u, d_v, d_w};
    const double *rr[3] = {fl->nlu, fl->nlv, fl->nlw};
    const int ncomp = three_d ? 3 : 2;
    auto residual = [&](double &mr) -> int {
        CK(cudaMemsetAsync(c.d_maxd, 0, sizeof(unsigned long long), c.s));
        launch_ad_residual_all(a, vel, rr, ncomp, c.d_maxd, c.s);
        c.launches++;
        unsigned long long bits = 0;
        CK(cudaMemcpyAsync(&bits, c.d_maxd, sizeof(bits), cudaMemcpyDeviceToHost, c.s));
        CK(cudaStreamSynchronize(c.s));
        std::memcpy(&mr, &bits, sizeof(mr));
        return 0;
    };
    double mr = 0.0;
    TRY(residual(mr));
    const bool gcm = (c.p.boundary_formulation == GCM_METHOD);
    if (gcm) mr = 1.0e10;   // the GCM branch starts its loop unconditionally (IBM/CORE_SOLVE_AD.F90:235)
    int it = 0, rc = 0;
    while (it < c.p.iterMax_ad && mr > c.p.restol_ad) {
        for (int q = 0; q < ncomp; ++q)
            for (int dir = 0; dir < (three_d ? 3 : 2); ++dir)
                for (int col = 0; col < 2; ++col) {
                    launch_ad_line(dir, col, a, vel[q], rr[q], gam, c.s);
                    c.launches++;
                }
        if (gcm && c.vg_on && c.nGhost > 0) {   // GCM_GhostCell_Vel
            CK(cudaMemsetAsync(c.d_iters, 0, sizeof(int), c.s));
            CK(cudaMemsetAsync(c.d_maxd, 0, sizeof(unsigned long long), c.s));
            GhostArgs g{c.nGhost, c.gidx, c.sidx, c.gsg, c.gg_ptr, c.gg_idx};
            launch_vel_ghosts(d_u, d_v, d_w, g, c.vg_coeff, c.vg_bi_set ? c.vg_bi : nullptr,
                              c.vg_bw, c.vg_iw, c.vg_scr, c.p.iterMax_ad, c.p.restol_ad, c.d_iters, c.d_maxd, c.s);
            c.launches++;
        }
        if (mass_consv) {   // GCM_enforce_global_mass_consv
            launch_face_vel_rhs(fv, false, c.step_partials, c.step_cap, (double *)c.result, c.s);
            launch_zg_rhs_terms(zg, c.s);
            launch_zg_planes(zg, c.s);
            c.launches += 5;
            if (advec_scheme == 2) {   // the Crank-Nicolson terms of the rows follow the new faces
                launch_ad_coef(a, c.s);
                c.launches++;
            }
        }
        if (cn2) {   // face_vel of the current velocities; the rows' convective terms follow it
            launch_face_vel_rhs(fv, false, c.step_partials, c.step_cap, (double *)c.result, c.s);
            launch_ad_coef(a, c.s);
            c.launches += 3;
        }
        TRY(residual(mr));
        ++it;
    }
    if (it >= c.p.iterMax_ad && mr > c.p.restol_ad) rc = 1;   // the reference prints and continues
    if (iters) *iters = it;
    if (maxres) *maxres = mr;
    return rc;
}

int fsi_mg_set_velocity_ghosts(void *handle, const double *coeffGCMD, const double *uBI, const double *vBI,
                               const double *wBI, double bodyInterceptWeight, double imagePointWeight)
{
    if (!handle) return fail(-1, "null handle");
    Ctx &c = *(Ctx *)handle;
    if (!c.geometry) return fail(-2, "fsi_mg_set_geometry has not been called");
    if (!coeffGCMD) { c.vg_on = false; return 0; }
    if (c.p.boundary_formulation != GCM_METHOD) return fail(-1, "velocity ghosts need boundary_formulation GCM");
    if ((uBI == nullptr) != (vBI == nullptr) || (uBI == nullptr) != (wBI == nullptr))
        return fail(-1, "uBI, vBI, wBI must be all given or all NULL");
    const int n = c.nGhost;
    if (n == 0) { c.vg_on = true; return 0; }
    if (c.vg_cap < c.ghost_cap) {   // grow-only, sized like the pressure ghost buffers
        for (void *q : {(void *)c.vg_coeff, (void *)c.vg_bi, (void *)c.vg_scr}) {
            auto it = std::find(c.allocs.begin(), c.allocs.end(), q);
            if (q && it != c.allocs.end()) { cudaFree(q); c.allocs.erase(it); }
        }
        TRY(c.alloc(&c.vg_coeff, 8 * (size_t)c.ghost_cap));
        TRY(c.alloc(&c.vg_bi, 3 * (size_t)c.ghost_cap));
        TRY(c.alloc(&c.vg_scr, 6 * (size_t)c.ghost_cap));
        c.vg_cap = c.ghost_cap;
    }
    CK(cudaMemcpyAsync(c.vg_coeff, coeffGCMD, 8 * (size_t)n * 8, cudaMemcpyHostToDevice, c.s));
    c.vg_bi_set = (uBI != nullptr);
    if (c.vg_bi_set) {
        CK(cudaMemcpyAsync(c.vg_bi, uBI, (size_t)n * 8, cudaMemcpyHostToDevice, c.s));
        CK(cudaMemcpyAsync(c.vg_bi + n, vBI, (size_t)n * 8, cudaMemcpyHostToDevice, c.s));
        CK(cudaMemcpyAsync(c.vg_bi + 2 * (size_t)n, wBI, (size_t)n * 8, cudaMemcpyHostToDevice, c.s));
    }
    CK(cudaStreamSynchronize(c.s));
    c.vg_bw = bodyInterceptWeight;
    c.vg_iw = imagePointWeight;
    c.vg_on = true;
    return 0;
}

int fsi_mg_update_pressure(void *handle, int frac_step_type, const double *d_pPrime, double *d_p)
{
    if (!handle || !d_pPrime || !d_p) return fail(-1, "null argument");
    if (frac_step_type != 0 && frac_step_type != 1) return fail(-1, "frac_step_type must be 0 (NO_VAN_KAN) or 1 (VAN_KAN)");
    Ctx &c = *(Ctx *)handle;
    TRY(step_ready(c));
    launch_update_pressure(d_p, d_pPrime, c.L1.d.sxy * (c.nz + 2), frac_step_type == 1, c.s);
    c.last_up_p = d_p; c.last_up_pp = d_pPrime; c.last_up_vk = (frac_step_type == 1); c.have_up = true;
    c.launches++;
    if (c.p.boundary_formulation == GCM_METHOD && c.nGhost > 0) {
        GhostArgs g{c.nGhost, c.gidx, c.sidx, c.gsg, c.gg_ptr, c.gg_idx};
        launch_ghost_rows<double>(d_p, g, c.gco64, c.ggc64, c.gscr64, c.p.iterMax_ad, c.p.restol_ad, 0.0, c.d_iters, c.d_maxd,
                                  c.s);
        c.launches++;
    }
    CK(cudaStreamSynchronize(c.s));
    return 0;
}
} // extern "C"
