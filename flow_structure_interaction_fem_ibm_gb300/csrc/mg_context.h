// Handle state of the native library (one Ctx per fsi_mg_create) and the
// error helpers shared by its host translation units: the multigrid solve
// (fsi_mg.cu) and the fractional-step entry points (step_api.cu).
#pragma once

#include "fsi_mg.h"
#include "mg_kernels.cuh"

#include <algorithm>
#include <string>
#include <vector>

namespace fsimg {

// message of the last failed call on this thread (fsi_mg_last_error)
extern thread_local std::string g_err;
// records msg as the last error and returns code
int fail(int code, const std::string &msg);

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(-10, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

enum { BC_ZERO_GRADIENT = 2, BC_PERIODIC = 5, PBC_DIRICHLET = 1, PBC_NEUMANN = 2, GCM_METHOD = 2 };

struct Level {
    Dims d{};
    int lev[3] = {1, 1, 1};
    uint8_t *fl = nullptr;
    double *binv64[3] = {}, *gam64[3] = {};
    float *binv32[3] = {}, *gam32[3] = {};
    double *cm64[3] = {}, *cp64[3] = {};
    float *cm32[3] = {}, *cp32[3] = {};
    double *v64 = nullptr, *r64 = nullptr;
    float *v32 = nullptr, *r32 = nullptr;
    int dlo[3] = {}, dhi[3] = {};   // finest-level Dirichlet ends per line direction
    double *wpf[3] = {};            // factored partition tables of the FP64 smoother (or null)
};

// Transfer tables between level n and n+1 of one cycle direction.  Level 1 is
// shared by the three cycles, so its tables live per direction (Ctx::T1).
struct Transfer {
    // restriction weights (per coarse index along the cycle direction)
    double *rw1_64 = nullptr, *rw2_64 = nullptr;
    float *rw1_32 = nullptr, *rw2_32 = nullptr;
    // prolongation from level n+1 (per fine index along the cycle direction)
    int *pcA = nullptr, *pcB = nullptr;
    int8_t *pmode = nullptr;
    double *pwA64 = nullptr, *pwB64 = nullptr;
    float *pwA32 = nullptr, *pwB32 = nullptr;
};

struct Ctx {
    fsi_mg_params p{};
    int nx = 0, ny = 0, nz = 0, nd = 3;
    cudaStream_t s = nullptr;
    std::vector<void *> allocs;
    size_t bytes = 0;
    long long launches = 0;

    // host grid metrics (0:n+1)
    std::vector<double> x[3], xc[3], dx[3], dxinv[3], dxc[3], dxcinv[3];
    // MG metrics per axis: [lev-1][i]
    int nlev[3] = {1, 1, 1};
    std::vector<int> mgrid[3];
    std::vector<std::vector<double>> xMG[3], xcMG[3], dxMG[3], dxinvMG[3], dxcMG[3], dxcinvMG[3];

    Level L1;
    std::vector<Level> C[3];   // C[d][n] for n = 2..nlev (index n)
    std::vector<Transfer> T[3];   // T[d][n]: tables between level n and n+1 of cycle d

    // level-1 fields (full layout)
    double *p64 = nullptr, *b64 = nullptr, *nlw0 = nullptr;
    float *e32 = nullptr, *r32 = nullptr;
    double *U64 = nullptr;
    float *U32 = nullptr;
    double *stage = nullptr;   // host-transfer staging (full layout)

    // ghost rows
    int nGhost = 0, ghost_cap = 0;
    long long *gidx = nullptr, *sidx = nullptr;
    int *gsg = nullptr;   // stencil in the ghost-buffer encoding (GhostArgs::sg)
    int *gg_ptr = nullptr, *gg_idx = nullptr;   // ghost-ghost couplings (CSR)
    int gg_cap = 0;
    double *ggc64 = nullptr;
    float *ggc32 = nullptr;
    double *gco64 = nullptr, *gscr64 = nullptr;
    float *gco32 = nullptr, *gscr32 = nullptr;
    int *d_iters = nullptr;
    unsigned long long *d_maxd = nullptr;

    // reductions
    int nred = 0;
    MaxLoc *partials = nullptr, *result = nullptr, *h_result = nullptr;
    double *sums = nullptr;

    // boundary
    double *pgrad = nullptr;
    size_t npgrad = 0;
    bool compat_active = false, nlw0_nonzero = false;
    // FGMRES with the compatibility correction: n1 = nlw0 of a unit shift of the zero-gradient
    // planes (per precision), the unit planes themselves and the flux scalar of phi . z
    double *pg_unit = nullptr, *n1_64 = nullptr, *kflux = nullptr;
    float *n1_32 = nullptr;
    bool n1_ready = false;
    int side_raw[6] = {1, 1, 1, 1, 1, 1};
    int sign[6] = {1, 1, 1, 1, 1, 1};
    double *d_dx[3] = {}, *d_dxinv[3] = {}, *d_dxcinv[3] = {};
    double *d_xn[3] = {};   // node coordinates x(0:n+1) (shear boundary profiles)
    double *d_fx[3] = {};   // face interpolation weights fx(1:n) (IBM/CORE_GRID.F90:163-175)
    double *d_gx[3] = {};   // 1 - fx, as the reference forms it
    // diffusion coefficient tables of rhs_diff: dcinv(i) dinv(i), dcinv(i+1) dinv(i), (2 dinv(i)) dinv(i)
    double *d_adm[3] = {}, *d_adp[3] = {}, *d_adb[3] = {};
    double *step_partials = nullptr;   // one partial sum per CTA of face_vel_rhs
    int step_cap = 0;
    double *vtilde = nullptr;   // uTilde, vTilde, wTilde of the VAN_KAN face_vel (allocated on first use)
    double *zg_div = nullptr;   // divergence scratch of the face_vel inside solve_ad (zero-gradient sides, GCM)
    double ghost32_reltol = 1.0e-6;   // FP32 ghost rows stop at max|dp| <= this x max|p_g|
    // ghost-cell velocities (GCM_vel_set_bc_internal), registered by fsi_mg_set_velocity_ghosts
    bool vg_on = false;
    int vg_cap = 0;
    double *vg_coeff = nullptr, *vg_bi = nullptr, *vg_scr = nullptr;
    bool vg_bi_set = false;
    double vg_bw = 0.0, vg_iw = 0.0;
    int vg_last_iters = 0;
    // arguments of the last step calls, replayed by fsi_mg_time_kernel (which 6, 7, 8)
    StepArgs last_fv{}, last_cv{};
    RhsAdArgs last_ad{};
    bool have_ad = false;
    double *ad_co = nullptr;   // 7 coefficient fields of the implicit momentum operator + gam scratch
    bool have_fv = false, have_cv = false, have_up = false, last_fv_vk = false, last_up_vk = false;
    double *last_up_p = nullptr;
    const double *last_up_pp = nullptr;

    uint8_t *fresh = nullptr;   // fresh_cell (level-1 layout) of a moving body
    bool fresh_on = false;
    bool geometry = false;
    bool bound_device = false;   // p64/b64 point at caller memory

    // graphs
    cudaGraphExec_t graph = nullptr;
    long long graph_kernels = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    double last_e2e = 0;
    double *graph_p = nullptr;
    const double *graph_b = nullptr;

    // FGMRES state (outer_krylov > 0)
    int km = 0;
    std::vector<double *> KV, KZ;          // Arnoldi basis (m+1) and preconditioned directions (m), FP64
    std::vector<float *> KV32, KZ32;       // the same in FP32 (mixed precision)
    double *kw = nullptr, *kzp = nullptr, *kzr = nullptr;
    float *kw32 = nullptr;
    double *kpart = nullptr, *kdots = nullptr, *h_kdots = nullptr;
    cudaGraphExec_t pgraph = nullptr;      // MG preconditioner on fixed buffers
    long long pgraph_kernels = 0;

    // optional event timing of the level-1 line launches inside the solve graphs:
    // pairs [lt_base, lt_base + 2*lt_pairs) of lt_ev belong to the graph being captured
    bool lt_on = false;
    std::vector<cudaEvent_t> lt_ev;
    int lt_next = 0;
    std::vector<int8_t> lt_f32;            // precision of each pair
    int graph_lt0 = 0, graph_lt1 = 0;      // pair range of the outer-iteration graph
    int pgraph_lt0 = 0, pgraph_lt1 = 0;    // pair range of the preconditioner graph
    double lt_ms[2] = {0, 0};              // [FP64, FP32] summed launch durations
    long long lt_n[2] = {0, 0};

    // stats
    std::vector<double> hist;   // max-norm residual after each outer iteration of the last solve
    int last_iters = 0;
    double last_maxres = 0, last_time = 0, last_wall = 0;
    long long ghost_sweeps = 0;

    ~Ctx()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (pgraph) cudaGraphExecDestroy(pgraph);
        if (h_kdots) cudaFreeHost(h_kdots);
        for (cudaEvent_t e : lt_ev) cudaEventDestroy(e);
        for (cudaEvent_t e : {ev0, ev1, ev2, ev3})
            if (e) cudaEventDestroy(e);
        for (void *a : allocs) cudaFree(a);
        if (h_result) cudaFreeHost(h_result);
        if (s) cudaStreamDestroy(s);
    }

    template <typename T>
    int alloc(T **ptr, size_t count)
    {
        void *q = nullptr;
        size_t b = std::max<size_t>(count, 1) * sizeof(T);
        cudaError_t e = cudaMalloc(&q, b);
        if (e != cudaSuccess) return fail(-11, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        cudaMemsetAsync(q, 0, b, s);
        allocs.push_back(q);
        bytes += b;
        *ptr = (T *)q;
        return 0;
    }
};

#define TRY(x)                \
    do {                      \
        int rc_ = (x);        \
        if (rc_ != 0) return rc_; \
    } while (0)

} // namespace fsimg
