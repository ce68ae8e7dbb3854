// Shared definitions for the sm_103a kernels of the lens-population characteristic function
// and its inversion.  Host and device code.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include <algorithm>
#include <atomic>

#include "sgl_gb300.h"

namespace sgl {

// two FP32 lanes in one 64-bit register for the packed FMA (fma.rn.f32x2 rounds each lane like fmaf)
__device__ __forceinline__ unsigned long long f32x2_pack(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 f32x2_unpack(unsigned long long v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ void f32x2_fma(unsigned long long& acc, unsigned long long a, unsigned long long b) {
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(a), "l"(b));
}


// ------------------------------------------------------------------ launch geometry
constexpr int kNumSMs = 152;          // GB300: 2 dies x 76 SMs

// ------------------------------------------------------------------ float-float helpers
// A value v is carried as hi + lo with hi = (float)v, lo = (float)(v - hi): ~48 significant
// bits on the FP32 pipes, which is what the phase k * kappa needs before range reduction.
struct ff { float hi, lo; };

__host__ __device__ inline ff ff_from_double(double v) {
    ff r; r.hi = (float)v; r.lo = (float)(v - (double)r.hi); return r;
}

// sin r and cos r for a reduced argument |r| <= pi/4 (+ rounding slack) from their Taylor series
// to r^9 and r^10, written as r + r^3 P(r^2) and 1 + r^2 Q(r^2) so that the last FMA adds a small
// correction to an exact leading term.  On |r| <= 0.8 the truncation error is below 1e-9 relative
// and the FP32 evaluation stays within 0.73 ulp (sin) and 0.88 ulp (cos) of the exact values,
// without bias (checked against FP64 sin / cos over the whole interval).
__device__ __forceinline__ void sincos_reduced(float r, float& s, float& c) {
    const float r2 = r * r;
    float p = fmaf(r2, -1.f / 5040.f, 1.f / 120.f);
    p = fmaf(r2, p, -1.f / 6.f);
    p = fmaf(r2 * r2 * r2, 1.f / 362880.f, p);
    s = fmaf(r * r2, p, r);
    float q = fmaf(r2, -1.f / 3628800.f, 1.f / 40320.f);
    q = fmaf(r2, q, -1.f / 720.f);
    q = fmaf(r2, q, 1.f / 24.f);
    q = fmaf(r2, q, -0.5f);
    c = fmaf(r2, q, 1.f);
}

// Mixed path: ph = k * kap in float-float, half angle reduced mod pi/2 (three float parts of
// pi/2 with FMA-exact products).  Returns the reduced argument r, the quadrant q mod 4 and ph
// (float-float head + tail): scale * ph = r + q pi/2.
// scale = 0.5 reduces ph/2 (the default), scale = 1 reduces ph itself.
__device__ __forceinline__ void halfangle_reduce_ff(ff k, ff kap, float& r, int& quad, float& ph_hi, float& ph_lo,
                                                    float scale = 0.5f) {
    const float p = k.hi * kap.hi;
    const float e = fmaf(k.hi, kap.hi, -p);
    const float t = fmaf(k.hi, kap.lo, fmaf(k.lo, kap.hi, e));
    ph_hi = p; ph_lo = t;
    const float xh = scale * p, xl = scale * t;
    const float q = rintf(xh * 0.636619772367581343f);   // 2/pi; exact integer for |q| < 2^24
    // x - q pi/2 with pi/2 = C1 + C2 + C3 (float parts); the roundings of q*C1 and q*C2 are
    // recovered exactly with FMA and xh - q*C1 is exact (Sterbenz), so the reduction holds for
    // every |q| < 2^24 (phases up to ~2.6e7)
    constexpr float C1 = 1.57079637050628662109375f;
    constexpr float C2 = -4.371138828673792886547744274139404296875e-08f;
    constexpr float C3 = -1.7151245100058819e-15f;
    const float p1 = q * C1, e1 = fmaf(q, C1, -p1);
    const float p2 = q * C2, e2 = fmaf(q, C2, -p2);
    float rr = xh - p1;
    rr -= e1;
    rr -= p2;
    rr -= e2;
    rr = fmaf(-q, C3, rr);
    r = rr + xl;
    quad = ((int)q) & 3;
}

// sin(ph/2), cos(ph/2) and ph: the reduction above, the reduced sin / cos and the quadrant fix-up.
__device__ inline void halfangle_sincos_ff(ff k, ff kap, float& s, float& c, float& ph_hi, float& ph_lo) {
    float r;
    int qi;
    halfangle_reduce_ff(k, kap, r, qi, ph_hi, ph_lo);
    float sr, cr;
    sincos_reduced(r, sr, cr);
    switch (qi) {
        case 0: s = sr;  c = cr;  break;
        case 1: s = cr;  c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
}

// sin(k kap) and cos(k kap) in FP32 from the float-float phase, reduced exactly (full angle).
__device__ inline void sincos_ff(ff k, ff kap, float& s, float& c) {
    float r, ph_hi, ph_lo;
    int qi;
    halfangle_reduce_ff(k, kap, r, qi, ph_hi, ph_lo, 1.f);
    float sr, cr;
    sincos_reduced(r, sr, cr);
    switch (qi) {
        case 0: s = sr;  c = cr;  break;
        case 1: s = cr;  c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
}

// ------------------------------------------------------------------ J0(x) - 1
// Small-argument series below 1e-3 exactly as the reference forms it (-x^2/4 (1 - x^2/16));
// above, CUDA's double-precision j0 minus 1.
__device__ inline double j0m1_d(double x) {
    if (x < 1e-3) { double x2 = x * x; return -x2 * 0.25 * (1.0 - x2 * (1.0 / 16.0)); }
    return j0(x) - 1.0;
}

// ------------------------------------------------------------------ block reductions
template <typename T>
__device__ inline T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Deterministic block sum (fixed tree); every thread gets the total.  `sh` holds >= 32 T.
template <typename T>
__device__ inline T block_sum(T v, T* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    T t = (threadIdx.x < nw) ? sh[threadIdx.x] : T(0);
    if (wid == 0) t = warp_sum(t);
    if (threadIdx.x == 0) sh[0] = t;
    __syncthreads();
    T r = sh[0];
    __syncthreads();
    return r;
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Number of kernels this library has launched (reported by sgl_stats_json).
std::atomic<long long>& launch_counter();
#define SGL_COUNT(n) (::sgl::launch_counter() += (n))

}  // namespace sgl
