// One-dimensional compensated compound-Poisson CF sweep over a large cell list:
//   Lambda(k_n) = sum_c w_c (e^{i k_n kap_c} - 1 - i k_n kap_c)
// (the kappa part of Psi_1, reference _sep_lam_kernel's A1 term, sgl_full.py:2596-2617), for cell
// lists of any size (16.8M cells x 16384 k in the synthetic plane x mass x impact-parameter sweep).
//
// CTA (k tile of 256 rows, cell chunk): each thread owns one k; the chunk's cells stream through
// shared memory in tiles of 512 (coalesced loads, broadcast reads).  FP64 path: FP64 sincos of the
// half angle; mixed path: float-float phase, exact reduction mod pi/2, FP32 sin / cos of the reduced
// half angle (Taylor polynomials), Kahan-compensated FP32 accumulation within the chunk, FP64 across
// chunks (fixed order: deterministic).
//
// Also: FMA-throughput probes used as the measured FP64 / FP32 peaks of the CF-sweep roofline.
#include "kernels.cuh"

namespace sgl {

constexpr int kSwRows = 256;
constexpr int kSwTile = 512;

template <int MODE>
__global__ void __launch_bounds__(kSwRows)
k_sweep1d(const double* __restrict__ kk, int nk, const double* __restrict__ kap, const double* __restrict__ w,
          const float* __restrict__ kh, const float* __restrict__ kl, const float* __restrict__ wf,
          long long nc, long long per_chunk, double2* __restrict__ part) {
    __shared__ double s_k[MODE == SGL_FP64 ? kSwTile : 1];
    __shared__ double s_w[MODE == SGL_FP64 ? kSwTile : 1];
    __shared__ float4 s_c[MODE == SGL_FP64 ? 1 : kSwTile];     // (kappa head, kappa tail, w, -)
    const int n = blockIdx.x * kSwRows + threadIdx.x;
    const double k = n < nk ? kk[n] : 0.0;
    const ff kf = ff_from_double(k);
    const long long c0 = (long long)blockIdx.y * per_chunk;
    const long long c1 = c0 + per_chunk < nc ? c0 + per_chunk : nc;
    double ar = 0.0, ai = 0.0;
    float far = 0.f, fai = 0.f, car = 0.f, cai = 0.f;
    for (long long base = c0; base < c1; base += kSwTile) {
        const int cnt = (int)((c1 - base) < kSwTile ? (c1 - base) : kSwTile);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += kSwRows) {
            if (MODE == SGL_FP64) { s_k[e] = kap[base + e]; s_w[e] = w[base + e]; }
            else s_c[e] = make_float4(kh[base + e], kl[base + e], wf[base + e], 0.f);
        }
        __syncthreads();
        if (MODE == SGL_FP64) {
            for (int e = 0; e < cnt; ++e) {
                const double ph = k * s_k[e];
                double s, c;
                sincos(0.5 * ph, &s, &c);
                const double cm1 = -2.0 * s * s;
                double smp;
                if (fabs(ph) < 1e-2) {
                    const double p2 = ph * ph;
                    smp = -ph * p2 / 6.0 * (1.0 - p2 / 20.0 * (1.0 - p2 / 42.0));
                } else {
                    smp = 2.0 * s * c - ph;
                }
                ar = fma(s_w[e], cm1, ar);
                ai = fma(s_w[e], smp, ai);
            }
        } else {
            for (int e = 0; e < cnt; ++e) {
                const float4 cv = s_c[e];
                ff kapf; kapf.hi = cv.x; kapf.lo = cv.y;
                float r, ph_hi, ph_lo;
                int qi;
                halfangle_reduce_ff(kf, kapf, r, qi, ph_hi, ph_lo);
                float sr, cr;
                sincos_reduced(r, sr, cr);
                // only sin^2(ph/2) and sin(ph/2) cos(ph/2) enter: the quadrant picks sin or cos
                // for the square and the sign of the product
                const bool odd = qi & 1;
                const float a = odd ? cr : sr;
                const float cm1 = -2.f * a * a;
                const float sn = (odd ? -2.f : 2.f) * sr * cr;
                const float ph = ph_hi + ph_lo;
                float smp;
                if (fabsf(ph) < 1e-2f) {
                    const float p2 = ph * ph;
                    smp = -ph * p2 * (1.f / 6.f) * (1.f - p2 * (1.f / 20.f) * (1.f - p2 * (1.f / 42.f)));
                } else {
                    smp = (sn - ph_hi) - ph_lo;
                }
                const float wv = cv.z;
                float y = fmaf(wv, cm1, -car); float t = far + y; car = (t - far) - y; far = t;
                y = fmaf(wv, smp, -cai); t = fai + y; cai = (t - fai) - y; fai = t;
            }
        }
    }
    if (n < nk) {
        if (MODE == SGL_FP64) part[(long long)blockIdx.y * nk + n] = make_double2(ar, ai);
        else part[(long long)blockIdx.y * nk + n] = make_double2((double)far - (double)car, (double)fai - (double)cai);
    }
}

__global__ void k_sweep1d_reduce(const double2* __restrict__ part, int nchunks, int nk, double* __restrict__ re,
                                 double* __restrict__ im) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nk) return;
    double r = 0.0, i = 0.0;
    for (int c = 0; c < nchunks; ++c) { const double2 v = part[(long long)c * nk + n]; r += v.x; i += v.y; }
    re[n] = r;
    im[n] = i;
}

int sweep1d_chunks(int nk, long long nc) {
    // ~4 CTAs per SM over (k tiles x chunks), at least 16 k... cells per chunk
    const int ktiles = ceil_div(nk, kSwRows);
    long long nch = (4LL * kNumSMs + ktiles - 1) / ktiles;
    nch = nch < 1 ? 1 : nch;
    const long long maxch = (nc + kSwTile - 1) / kSwTile;
    if (nch > maxch) nch = maxch > 0 ? maxch : 1;
    return (int)nch;
}

void launch_sweep1d(int precision, const double* kk, int nk, const double* kap, const double* w, const float* kh,
                    const float* kl, const float* wf, long long nc, int nchunks, double2* part, double* re,
                    double* im, cudaStream_t st) {
    const long long per = (nc + nchunks - 1) / nchunks;
    dim3 grid(ceil_div(nk, kSwRows), nchunks);
    if (precision == SGL_FP64) { k_sweep1d<SGL_FP64><<<grid, kSwRows, 0, st>>>(kk, nk, kap, w, kh, kl, wf, nc, per, part); SGL_COUNT(1); }
    else { k_sweep1d<SGL_MIXED><<<grid, kSwRows, 0, st>>>(kk, nk, kap, w, kh, kl, wf, nc, per, part); SGL_COUNT(1); }
    { k_sweep1d_reduce<<<ceil_div(nk, 256), 256, 0, st>>>(part, nchunks, nk, re, im); SGL_COUNT(1); }
}

// ------------------------------------------------------------------ FMA throughput probes
// 8 independent FMA chains per thread, iters iterations; the result is stored so nothing is elided.
template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, int iters, T seed) {
    T a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = seed + (T)(threadIdx.x + j);
    const T m = (T)0.999999, c = (T)1e-7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fma(a[j], m, c);
    }
    T s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

void launch_fma_probe(int fp64, void* out, int blocks, int iters, cudaStream_t st) {
    if (fp64) { k_fma_probe<double><<<blocks, 256, 0, st>>>((double*)out, iters, 1.0); SGL_COUNT(1); }
    else { k_fma_probe<float><<<blocks, 256, 0, st>>>((float*)out, iters, 1.f); SGL_COUNT(1); }
}

}  // namespace sgl
