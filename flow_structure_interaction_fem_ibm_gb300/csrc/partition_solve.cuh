// The warp-per-line partition solver of tridiagonal line systems, shared by
// the pressure smoother (MG_itsolv, IBM/CORE_MG.F90:1883-2270) and the
// implicit momentum sweeps (itsolv_ad, IBM/CORE_SOLVE_AD.F90): the arithmetic
// role of tdma (IBM/CORE_TDMA.F90:10-34) with one warp per line.  Internal
// linkage, like device_util.cuh.
#pragma once

#include "device_util.cuh"

namespace fsimg {

namespace {

// lines per CTA of the partition solvers (one warp each)
constexpr int WP_LINES = 8;

template <int S> __host__ __device__ constexpr int wp_pitch() { return 32 * (S + 1) + 4; }

// Reciprocal used by the partition solver: IEEE division in FP64; the fast
// approximate reciprocal (about 1 ulp) in FP32, where the smoother only
// produces a correction inside FP64 refinement.
template <typename T> __device__ __forceinline__ T wp_rcp(T x);
template <> __device__ __forceinline__ float wp_rcp<float>(float x) { return __fdividef(1.0f, x); }
template <> __device__ __forceinline__ double wp_rcp<double>(double x) { return 1.0 / x; }

// One parallel-cyclic-reduction step over the warp at distance h.  Each lane
// keeps its row (A, B, C, D) and 1/B.  Outside the system the neighbour is an
// identity row (A = C = D = 0, B = 1): its multiplier is zero, and the lane's
// own (finite) values that the shuffle returns there only ever meet that zero.
template <typename T>
__device__ __forceinline__ void pcr_step(T &A, T &B, T &C, T &D, T &iB, int lane, int h)
{
    const T Am = __shfl_up_sync(0xffffffffu, A, h), iBm = __shfl_up_sync(0xffffffffu, iB, h);
    const T Cm = __shfl_up_sync(0xffffffffu, C, h), Dm = __shfl_up_sync(0xffffffffu, D, h);
    const T Ap = __shfl_down_sync(0xffffffffu, A, h), iBp = __shfl_down_sync(0xffffffffu, iB, h);
    const T Cp = __shfl_down_sync(0xffffffffu, C, h), Dp = __shfl_down_sync(0xffffffffu, D, h);
    const T k1 = (lane < h) ? T(0) : A * iBm;
    const T k2 = (lane + h > 31) ? T(0) : C * iBp;
    const T nA = -k1 * Am, nC = -k2 * Cp;
    const T nB = B - k1 * Cm - k2 * Ap;
    const T nD = D - k1 * Dm - k2 * Dp;
    A = nA; B = nB; C = nC; D = nD;
    iB = wp_rcp(nB);
}

// One row of a line's tridiagonal system in shared memory, (a, b, c, d)
// packed so that staging writes and the solve reads it with one vector access.
template <typename T>
struct alignas(4 * sizeof(T)) WpRow {
    T a, b, c, d;
};

// Row slots of one line: S rows per lane plus one pad slot per lane segment
// (lane l's segment starts at l (S+1), so the per-lane vector reads of the
// solve hit distinct bank groups), plus one slot so that consecutive lines
// start on different banks (the y/z staging writes 8 lines side by side).
template <int S> __host__ __device__ constexpr int wp_rows_pitch() { return 32 * (S + 1) + 1; }

// Partition solve of one line (the calling warp) staged as WpRow rows in
// shared memory (row r at r + r/S): lane l eliminates its S consecutive rows
// in registers, expressing the interior unknowns through the previous lane's
// last unknown XL and its own last unknown XR; the 32 interface unknowns are
// solved by PCR over shuffles; the solution of row r goes to x[r + r/S].  x
// may alias the line's own rows: every lane has read its rows before the
// first shuffle, and the solution is written after the last.  Rows beyond L
// (or an invalid line) are identity rows and write nothing.
template <typename T, int S>
__device__ __forceinline__ void wp_solve_line(const WpRow<T> *rows, T *x, int L, bool valid, int lane)
{
    T a[S], b[S], c[S], dv[S];
#pragma unroll
    for (int s2 = 0; s2 < S; ++s2) {
        const int r = lane * S + s2;
        if (valid && r < L) {
            const WpRow<T> w = rows[r + r / S];
            a[s2] = w.a; b[s2] = w.b; c[s2] = w.c; dv[s2] = w.d;
        } else {
            a[s2] = T(0); b[s2] = T(1); c[s2] = T(0); dv[s2] = T(0);
        }
    }
    // segment elimination: rows 0..S-2 in terms of XL (previous lane's last) and XR (own last)
    T y[S], u[S], w[S], gg[S];
    {
        T gp = T(0), yp = T(0), up = T(0), wp = T(0);
#pragma unroll
        for (int s2 = 0; s2 < S - 1; ++s2) {
            const T inv = wp_rcp(b[s2] - a[s2] * gp);
            y[s2] = (dv[s2] - a[s2] * yp) * inv;
            u[s2] = ((s2 == 0 ? -a[0] : T(0)) - a[s2] * up) * inv;
            w[s2] = ((s2 == S - 2 ? -c[S - 2] : T(0)) - a[s2] * wp) * inv;
            gg[s2] = c[s2] * inv;
            gp = gg[s2]; yp = y[s2]; up = u[s2]; wp = w[s2];
        }
#pragma unroll
        for (int s2 = S - 3; s2 >= 0; --s2) {
            y[s2] = y[s2] - gg[s2] * y[s2 + 1];
            u[s2] = u[s2] - gg[s2] * u[s2 + 1];
            w[s2] = w[s2] - gg[s2] * w[s2 + 1];
        }
    }
    const T y0 = (S >= 2) ? y[0] : T(0), u0 = (S >= 2) ? u[0] : T(0), w0 = (S >= 2) ? w[0] : T(1);
    const T yl = (S >= 2) ? y[S - 2 < 0 ? 0 : S - 2] : T(0);
    const T ul = (S >= 2) ? u[S - 2 < 0 ? 0 : S - 2] : T(1);
    const T wl = (S >= 2) ? w[S - 2 < 0 ? 0 : S - 2] : T(0);
    const T y0n = __shfl_down_sync(0xffffffffu, y0, 1);
    const T u0n = __shfl_down_sync(0xffffffffu, u0, 1);
    const T w0n = __shfl_down_sync(0xffffffffu, w0, 1);
    const T an = a[S - 1], bn = b[S - 1], cn = c[S - 1];
    T RA = an * ul;
    T RB = bn + an * wl + cn * u0n;
    T RC = cn * w0n;
    T RD = dv[S - 1] - an * yl - cn * y0n;
    if (lane == 31) { RB = bn + an * wl; RC = T(0); RD = dv[S - 1] - an * yl; }
    T iRB = wp_rcp(RB);
#pragma unroll
    for (int h = 1; h < 32; h <<= 1) pcr_step(RA, RB, RC, RD, iRB, lane, h);
    const T XR = RD * iRB;
    T XL = __shfl_up_sync(0xffffffffu, XR, 1);
    if (lane == 0) XL = T(0);
    __syncwarp();
#pragma unroll
    for (int s2 = 0; s2 < S; ++s2) {
        const int r = lane * S + s2;
        if (valid && r < L) {
            const T xv = (s2 < S - 1) ? (y[s2 < S - 1 ? s2 : 0] + XL * u[s2 < S - 1 ? s2 : 0] + XR * w[s2 < S - 1 ? s2 : 0]) : XR;
            x[r + r / S] = xv;
        }
    }
}

} // namespace

} // namespace fsimg
