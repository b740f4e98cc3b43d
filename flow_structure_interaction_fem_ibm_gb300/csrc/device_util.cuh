// Device helpers shared by the kernel translation units: launch sizing, the
// axis permutations of a line sweep, interior-cell decoding and the
// deterministic block sums.  All have internal linkage, so each unit that
// includes this header holds its own copy.
#pragma once

#include "mg_kernels.cuh"

namespace fsimg {

namespace {

constexpr int TPB = 256;

inline int nblk(long long n, int tpb = TPB)
{
    long long b = (n + tpb - 1) / tpb;
    return (int)(b < 1 ? 1 : b);
}

template <int DIR> struct Axes;
template <> struct Axes<0> { static constexpr int a = 0, b = 1, c = 2; static constexpr bool c_first = false; };
template <> struct Axes<1> { static constexpr int a = 1, b = 0, c = 2; static constexpr bool c_first = false; };
template <> struct Axes<2> { static constexpr int a = 2, b = 0, c = 1; static constexpr bool c_first = true; };

// (i, j, k), 1-based, of interior cell t of an n0 x n1 x n2 box in column-major
// order; 32-bit arithmetic (every level holds fewer than 2^31 cells)
__device__ __forceinline__ void cell_of(unsigned t, unsigned n0, unsigned n1, int &i, int &j, int &k)
{
    const unsigned q = t / n0;
    i = 1 + (int)(t - q * n0);
    const unsigned kk = q / n1;
    j = 1 + (int)(q - kk * n1);
    k = 1 + (int)kk;
}

// x == 0 (either sign) from its bit pattern: integer instructions only, which
// keeps the all-zero-row test off the FP64 pipe
__device__ __forceinline__ bool is_zero(float x) { return (__float_as_uint(x) << 1) == 0u; }
__device__ __forceinline__ bool is_zero(double x)
{
    return ((unsigned long long)__double_as_longlong(x) << 1) == 0ull;
}

__device__ __forceinline__ long long stride_of(const Dims &d, int axis)
{
    return axis == 0 ? 1LL : (axis == 1 ? d.sx : d.sxy);
}

// ---------------------------------------------------------------------------
// Deterministic block-partial sums (fixed order), shared by the fluid-volume
// mean (IBM/CORE_POISSON.F90:433-443) and the compatibility flux
// (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:290-331).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_sum(double x)
{
    // sized for the largest block that calls it (1024 threads = 32 warps)
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    __shared__ double s[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) s[wid] = x;
    __syncthreads();
    double tot = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s[w];
    return tot;
}

__global__ void k_sum_final(double *partials, int n, int stride, double *out)
{
    // out[c] = sum_t partials[stride*t + c] for c < stride, fixed order per thread then tree
    for (int c = 0; c < stride; ++c) {
        double x = 0.0;
        for (int t = threadIdx.x; t < n; t += blockDim.x) x += partials[(long long)stride * t + c];
        const double tot = block_sum(x);
        if (threadIdx.x == 0) out[c] = tot;
        __syncthreads();
    }
}

} // namespace

} // namespace fsimg
