// Poisson part Psi_1 of ln Phi:  sum_c w_c (e^{i kk kap_c} J0(kg gam_c) - 1 - i kk kap_c).
//
//  * k_psi1_direct   -- dense direct sum for small grids and the k-reach probes
//                       (reference: _lam_worker_block, sgl_full.py:2682-2704)
//  * k_sep_sweep     -- separable evaluation, the part exact in kappa
//                       (reference: _sep_lam_kernel, sgl_full.py:2586-2619)
//  * table builders  -- J0-1 on gamma nodes x Chebyshev k_gamma points, the barycentric
//                       Chebyshev-Lobatto interpolation matrix (sgl_full.py:2665-2680)
#include "kernels.cuh"

namespace sgl {

// ------------------------------------------------------------------ phase helpers
// e^{i ph} - 1 - i ph without cancellation: cos(ph) - 1 = -2 sin^2(ph/2); sin(ph) - ph by its
// 3-term series below |ph| = 1e-2 (the reference's threshold and series).
__device__ inline void compensated_fp64(double ph, double& cm1, double& smp, double& sn) {
    double s, c;
    sincos(0.5 * ph, &s, &c);
    cm1 = -2.0 * s * s;
    sn = 2.0 * s * c;
    if (fabs(ph) < 1e-2) {
        const double p2 = ph * ph;
        smp = -ph * p2 / 6.0 * (1.0 - p2 / 20.0 * (1.0 - p2 / 42.0));
    } else {
        smp = sn - ph;
    }
}

// float-float arithmetic (Dekker / Knuth error-free transforms with FMA)
__device__ __forceinline__ ff ff_fast_sum(float a, float b) {      // |a| >= |b|
    ff r; r.hi = a + b; r.lo = b - (r.hi - a); return r;
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const float s = a.hi + b.hi, bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (b.hi - bb);
    return ff_fast_sum(s, e + (a.lo + b.lo));
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return ff_fast_sum(p, e);
}
__device__ __forceinline__ ff ff_div_f(ff a, float b) {
    const float q1 = a.hi / b;
    const float p = q1 * b, e = fmaf(q1, b, -p);
    const float r = ((a.hi - p) - e) + a.lo;
    return ff_fast_sum(q1, r / b);
}

// J0(a b) - 1 for the mixed path's FP32 tables, from the float-float product x = a b:
//  * x < 2: the power series sum_k (-y)^k / (k!)^2, y = x^2 / 4, as -y + (y^2/4) T(y) with y kept
//    as float-float, so the leading term carries no rounding of its own (<= 1.34 ulp);
//  * 2 <= x < 12: the same power series term by term in float-float arithmetic (32 terms; the
//    largest term is ~4e3 at x = 12, and float-float's ~48 bits leave the sum within 1e-10
//    relative, so the FP32 result is correctly rounded to within 0.5001 ulp);
//  * x >= 12: Hankel's asymptotic expansion J0 = sqrt(2/(pi x)) (P cos chi - Q sin chi),
//    chi = x - pi/4, with the first three terms of P and Q (Abramowitz & Stegun 9.2.5, 9.2.9,
//    9.2.10 at nu = 0) and x reduced mod pi/2 exactly from the float-float product (<= 1.06 ulp).
// The bounds were checked against FP64 J0 - 1 over the whole range; the errors are unbiased.
__device__ float j0m1_mixed(double a, double b) {
    const ff A = ff_from_double(a), B = ff_from_double(b);
    const float xh = A.hi * B.hi;
    const float xe = fmaf(A.hi, B.hi, -xh);
    const float xl = fmaf(A.hi, B.lo, fmaf(A.lo, B.hi, xe));
    if (xh < 2.f) {
        const float x2 = xh * xh;
        const float yh = 0.25f * x2;
        const float ye = fmaf(0.5f * xh, xl, 0.25f * fmaf(xh, xh, -x2));
        float T = 1.f;
#pragma unroll
        for (int k = 12; k > 2; --k) T = fmaf(-yh * (1.f / (float)(k * k)), T, 1.f);
        const float corr = (0.25f * yh * yh) * T;
        return (corr - ye) - yh;
    }
    if (xh < 12.f) {
        // y = x^2 / 4 in float-float; t_k = t_{k-1} (-y) / k^2, S = sum t_k
        const float p = xh * xh;
        const ff y = ff_fast_sum(p, fmaf(2.f * xh, xl, fmaf(xh, xh, -p)));
        const ff ny = {-0.25f * y.hi, -0.25f * y.lo};
        ff t = {1.f, 0.f}, S = {0.f, 0.f};
#pragma unroll 4
        for (int k = 1; k <= 32; ++k) {
            t = ff_div_f(ff_mul(t, ny), (float)(k * k));
            S = ff_add(S, t);
        }
        return S.hi + S.lo;
    }
    float r, ph_hi, ph_lo;
    int qi;
    halfangle_reduce_ff(A, B, r, qi, ph_hi, ph_lo, 1.f);
    float sr, cr;
    sincos_reduced(r, sr, cr);
    constexpr float kRsqrt2 = 0.70710678118654752f;
    const float c = (cr + sr) * kRsqrt2, s = (sr - cr) * kRsqrt2;    // cos, sin of r - pi/4
    float C, S;                                                          // cos, sin of chi
    switch (qi) {
        case 0: C = c;  S = s;  break;
        case 1: C = -s; S = c;  break;
        case 2: C = -c; S = -s; break;
        default: C = s; S = -c; break;
    }
    const float iz = 1.f / (8.f * xh), iz2 = iz * iz;
    float P = fmaf(iz2, -108056025.f / 720.f, 11025.f / 24.f);
    P = fmaf(iz2, P, -4.5f);
    P = fmaf(iz2, P, 1.f);
    float Q = fmaf(iz2, -893025.f / 120.f, 225.f / 6.f);
    Q = fmaf(iz2, Q, -1.f) * iz;
    const float amp = sqrtf(0.636619772367581343f / xh);
    return amp * fmaf(P, C, -Q * S) - 1.f;
}

// ------------------------------------------------------------------ direct sum
// CTA (output point, cell chunk); threads stride over the chunk's cells; deterministic block sum
// into part[chunk, point]; a second kernel sums the chunks in a fixed order.
constexpr int kDirectChunkCells = 4096;

__global__ void __launch_bounds__(256)
k_psi1_direct(const double* __restrict__ kk, int nk, const double* __restrict__ kg, int nkg,
              const double* __restrict__ k0, const double* __restrict__ g0,
              const double* __restrict__ w0, int64_t nc, double2* __restrict__ part) {
    __shared__ double sh[32];
    const int pt = blockIdx.x;
    const int n = pt / nkg, m = pt % nkg;
    const double k = kk[n], g = kg[m];
    const int64_t c0 = (int64_t)blockIdx.y * kDirectChunkCells;
    const int64_t c1 = c0 + kDirectChunkCells < nc ? c0 + kDirectChunkCells : nc;
    double re = 0.0, im = 0.0;
    if (g == 0.0) {
        // k_gamma = 0 (the kappa-axis probes): J0 = 1, J0 - 1 = 0
        for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
            const double w = w0[c];
            double cm1, smp, sn;
            compensated_fp64(k * k0[c], cm1, smp, sn);
            re += w * cm1;
            im += w * smp;
        }
    } else if (k == 0.0) {
        // k_kappa = 0 (the gamma-axis probes): the phase terms vanish
        for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
            const double x = g * g0[c];
            double B;
            if (x < 1e-3) { const double x2 = x * x; B = -x2 * 0.25 * (1.0 - x2 * (1.0 / 16.0)); }
            else B = j0(x) - 1.0;
            re += w0[c] * B;
        }
    } else {
        for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
            const double w = w0[c];
            const double ph = k * k0[c];
            const double x = g * g0[c];
            double cm1, smp, sn;
            compensated_fp64(ph, cm1, smp, sn);
            const double J = j0(x);
            double B;
            if (x < 1e-3) { const double x2 = x * x; B = -x2 * 0.25 * (1.0 - x2 * (1.0 / 16.0)); }
            else B = J - 1.0;
            // (cos-1) J + (J-1) and (sin-ph) J + ph (J-1): every term O(A) or O(B)
            re += w * fma(cm1, J, B);
            im += w * fma(smp, J, ph * B);
        }
    }
    re = block_sum(re, sh);
    im = block_sum(im, sh);
    if (threadIdx.x == 0) part[(long long)blockIdx.y * gridDim.x + pt] = make_double2(re, im);
}

// Mixed direct sum for the k-reach probes (and other small grids): the terms in FP32 from the
// float-float phase (exact reduction) and the FP32 J0 - 1 of the tables, accumulated in FP64.  On
// the two probe lines one of the factors is exactly 1 (k_gamma = 0: J0 = 1; k_kappa = 0: no
// phase), and only that factor's work is done.
__global__ void __launch_bounds__(256)
k_psi1_direct_mixed(const double* __restrict__ kk, int nk, const double* __restrict__ kg, int nkg,
                    const double* __restrict__ k0, const double* __restrict__ g0,
                    const double* __restrict__ w0, int64_t nc, double2* __restrict__ part) {
    __shared__ double sh[32];
    const int pt = blockIdx.x;
    const int n = pt / nkg, m = pt % nkg;
    const double k = kk[n], g = kg[m];
    const ff kf = ff_from_double(k);
    const int64_t c0 = (int64_t)blockIdx.y * kDirectChunkCells;
    const int64_t c1 = c0 + kDirectChunkCells < nc ? c0 + kDirectChunkCells : nc;
    double re = 0.0, im = 0.0;
    for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const double w = w0[c];
        float cm1 = 0.f, smp = 0.f, ph = 0.f;
        if (k != 0.0) {
            float r, ph_hi, ph_lo;
            int qi;
            halfangle_reduce_ff(kf, ff_from_double(k0[c]), r, qi, ph_hi, ph_lo);
            float sr, cr;
            sincos_reduced(r, sr, cr);
            const bool odd = qi & 1;
            const float a = odd ? cr : sr;
            cm1 = -2.f * a * a;
            const float sn = (odd ? -2.f : 2.f) * sr * cr;
            ph = ph_hi + ph_lo;
            if (fabsf(ph) < 1e-2f) {
                const float p2 = ph * ph;
                smp = -ph * p2 * (1.f / 6.f) * (1.f - p2 * (1.f / 20.f) * (1.f - p2 * (1.f / 42.f)));
            } else {
                smp = (sn - ph_hi) - ph_lo;
            }
        }
        if (g == 0.0) {
            re = fma(w, (double)cm1, re);
            im = fma(w, (double)smp, im);
        } else {
            const float B = j0m1_mixed(g, g0[c]);
            // (cos-1) J + (J-1) and (sin-ph) J + ph (J-1), J = 1 + B
            re = fma(w, (double)fmaf(cm1, 1.f + B, B), re);
            im = fma(w, (double)fmaf(smp, 1.f + B, ph * B), im);
        }
    }
    re = block_sum(re, sh);
    im = block_sum(im, sh);
    if (threadIdx.x == 0) part[(long long)blockIdx.y * gridDim.x + pt] = make_double2(re, im);
}

__global__ void k_direct_reduce(const double2* __restrict__ part, int nchunks, int npt, double* __restrict__ re,
                                double* __restrict__ im) {
    const int pt = blockIdx.x * blockDim.x + threadIdx.x;
    if (pt >= npt) return;
    double r = 0.0, i = 0.0;
    for (int c = 0; c < nchunks; ++c) { const double2 v = part[(long long)c * npt + pt]; r += v.x; i += v.y; }
    re[pt] = r;
    im[pt] = i;
}

int psi1_direct_chunks(int64_t nc) { return (int)((nc + kDirectChunkCells - 1) / kDirectChunkCells); }

void launch_psi1_direct(const double* kk, int nk, const double* kg, int nkg, const double* k0,
                        const double* g0, const double* w0, int64_t nc, double* re, double* im,
                        double2* part, cudaStream_t st, int precision) {
    const int npt = nk * nkg;
    if (npt == 0) return;
    const int nch = psi1_direct_chunks(nc) > 0 ? psi1_direct_chunks(nc) : 1;
    dim3 grid(npt, nch);
    if (precision == SGL_MIXED) { k_psi1_direct_mixed<<<grid, 256, 0, st>>>(kk, nk, kg, nkg, k0, g0, w0, nc, part); SGL_COUNT(1); }
    else { k_psi1_direct<<<grid, 256, 0, st>>>(kk, nk, kg, nkg, k0, g0, w0, nc, part); SGL_COUNT(1); }
    { k_direct_reduce<<<ceil_div(npt, 256), 256, 0, st>>>(part, nch, npt, re, im); SGL_COUNT(1); }
}

// ------------------------------------------------------------------ separable sweep
// Cells are sorted by gamma-node group; each group g owns columns [gcol0[g], gcol0[g] + gncol[g])
// of T (gncol = 8 Chebyshev nodes, or 1 exact node for a cell whose bin needs more than smax
// sub-bins).  A chunk is a range of whole groups.  CTA (row tile, chunk): each thread owns one
// k_kappa row and walks the chunk's cells, which are staged in shared memory and broadcast.
//   A_part[chunk, n] = sum_{c in chunk} w_c (e^{i k_n kap_c} - 1 - i k_n kap_c)
//   Tt[col, n] = Re sum wl e^{i k kap},  Tt[col, nk + n] = Im  (node-major: coalesced stores)
constexpr int kSweepRows = 128;
constexpr int kSweepStage = 64;

// FP64 sweep (the parity path).
__global__ void __launch_bounds__(kSweepRows, 4)
k_sep_sweep_f64(const double* __restrict__ kk, int nk, SepDevice sd, double* __restrict__ Tt,
                double2* __restrict__ A_part) {
    __shared__ double s_wl[kSweepStage][8];
    __shared__ double s_w[kSweepStage];
    __shared__ double s_k0[kSweepStage];
    __shared__ int s_grp[kSweepStage];
    const int n = blockIdx.x * kSweepRows + threadIdx.x;
    const bool live = n < nk;
    const double k = live ? kk[n] : 0.0;
    const int c_begin = sd.chunk_begin[blockIdx.y], c_end = sd.chunk_begin[blockIdx.y + 1];
    const long long ld = 2LL * nk;
    double ar = 0.0, ai = 0.0;
    double tr[8], ti[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) { tr[j] = 0.0; ti[j] = 0.0; }
    int cur = -1;
    auto flush = [&](int g) {
        if (g >= 0 && live) {
            const int col0 = sd.gcol0[g], nc = sd.gncol[g];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (j < nc) {
                    Tt[(long long)(col0 + j) * ld + n] = tr[j];
                    Tt[(long long)(col0 + j) * ld + nk + n] = ti[j];
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) { tr[j] = 0.0; ti[j] = 0.0; }
    };
    for (int base = c_begin; base < c_end; base += kSweepStage) {
        const int cnt = min(kSweepStage, c_end - base);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += kSweepRows) {
            s_k0[e] = sd.kap[base + e];
            s_w[e] = sd.w[base + e];
            s_grp[e] = sd.grp[base + e];
        }
        for (int e = threadIdx.x; e < cnt * 8; e += kSweepRows) s_wl[e >> 3][e & 7] = sd.wl[(long long)base * 8 + e];
        __syncthreads();
        for (int e = 0; e < cnt; ++e) {
            const int g = s_grp[e];
            if (g != cur) { flush(cur); cur = g; }
            const double w = s_w[e];
            const double ph = k * s_k0[e];
            double cm1, smp, sn;
            compensated_fp64(ph, cm1, smp, sn);
            ar = fma(w, cm1, ar);
            ai = fma(w, smp, ai);
            const double cr = cm1 + 1.0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                tr[j] = fma(s_wl[e][j], cr, tr[j]);
                ti[j] = fma(s_wl[e][j], sn, ti[j]);
            }
        }
    }
    flush(cur);
    if (live) A_part[(long long)blockIdx.y * nk + n] = make_double2(ar, ai);
}

// Mixed sweep: float-float phase, FP32 sin / cos of the reduced half angle, Kahan-compensated
// FP32 sums for A.  The inner loop is issue-bound, so it is kept short:
//  * each staged cell is packed as three float4 (kappa head, kappa tail, w, group | 8 weights),
//    read with three broadcast 16-byte shared loads;
//  * only sin^2(ph/2) and sin(ph/2) cos(ph/2) are needed, so the quadrant fix-up reduces to
//    choosing sin or cos for the square and the sign of the product (odd quadrants);
//  * warps whose rows are all past nk skip the arithmetic (they still stage and synchronise).
__global__ void __launch_bounds__(kSweepRows, 8)
k_sep_sweep_mixed(const double* __restrict__ kk, int nk, SepDevice sd, float* __restrict__ Tt,
                  double2* __restrict__ A_part) {
    __shared__ float4 s_c[kSweepStage][3];
    const int n = blockIdx.x * kSweepRows + threadIdx.x;
    const bool live = n < nk;
    const bool warp_live = blockIdx.x * kSweepRows + (threadIdx.x & ~31) < nk;
    const ff kf = ff_from_double(live ? kk[n] : 0.0);
    const int c_begin = sd.chunk_begin[blockIdx.y], c_end = sd.chunk_begin[blockIdx.y + 1];
    const long long ld = 2LL * nk;
    float far = 0.f, fai = 0.f, car = 0.f, cai = 0.f;  // Kahan-compensated FP32
    // the 8 node sums of the current group in weight pairs: tr2[q] = (tr[2q], tr[2q + 1]) for the
    // packed FMA (each lane rounds like fmaf)
    unsigned long long tr2[4], ti2[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) { tr2[q] = 0ull; ti2[q] = 0ull; }
    int cur = -1;
    auto flush = [&](int g) {
        if (g >= 0 && live) {
            const int col0 = sd.gcol0[g], nc = sd.gncol[g];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float2 r2 = f32x2_unpack(tr2[q]), i2 = f32x2_unpack(ti2[q]);
                const float rv[2] = {r2.x, r2.y}, iv[2] = {i2.x, i2.y};
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int j = 2 * q + h;
                    if (j < nc) {
                        Tt[(long long)(col0 + j) * ld + n] = rv[h];
                        Tt[(long long)(col0 + j) * ld + nk + n] = iv[h];
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) { tr2[q] = 0ull; ti2[q] = 0ull; }
    };
    for (int base = c_begin; base < c_end; base += kSweepStage) {
        const int cnt = min(kSweepStage, c_end - base);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += kSweepRows)
            s_c[e][0] = make_float4(sd.kap_hi[base + e], sd.kap_lo[base + e], sd.w_f[base + e],
                                    __int_as_float(sd.grp[base + e]));
        for (int e = threadIdx.x; e < cnt * 2; e += kSweepRows) {
            const float* w8 = sd.wl_f + (long long)(base + (e >> 1)) * 8 + (e & 1) * 4;
            s_c[e >> 1][1 + (e & 1)] = make_float4(w8[0], w8[1], w8[2], w8[3]);
        }
        __syncthreads();
        if (!warp_live) continue;
        for (int e = 0; e < cnt; ++e) {
            const float4 h = s_c[e][0];
            const int g = __float_as_int(h.w);
            if (g != cur) { flush(cur); cur = g; }
            ff kapf; kapf.hi = h.x; kapf.lo = h.y;
            float r, ph_hi, ph_lo;
            int qi;
            halfangle_reduce_ff(kf, kapf, r, qi, ph_hi, ph_lo);
            float sr, cr;
            sincos_reduced(r, sr, cr);
            const bool odd = qi & 1;
            const float a = odd ? cr : sr;                    // |sin(ph/2)|
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
            const float wf = h.z;
            float y = fmaf(wf, cm1, -car); float t = far + y; car = (t - far) - y; far = t;
            y = fmaf(wf, smp, -cai); t = fai + y; cai = (t - fai) - y; fai = t;
            const float crr = cm1 + 1.f;
            const float4 w0 = s_c[e][1], w1 = s_c[e][2];
            const unsigned long long wp[4] = {f32x2_pack(w0.x, w0.y), f32x2_pack(w0.z, w0.w), f32x2_pack(w1.x, w1.y),
                                              f32x2_pack(w1.z, w1.w)};
            const unsigned long long cp = f32x2_pack(crr, crr), sp = f32x2_pack(sn, sn);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                f32x2_fma(tr2[q], wp[q], cp);
                f32x2_fma(ti2[q], wp[q], sp);
            }
        }
    }
    flush(cur);
    if (live) A_part[(long long)blockIdx.y * nk + n] = make_double2((double)far - (double)car, (double)fai - (double)cai);
}

// A1[n] = sum over chunks (fixed order) of A_part[chunk, n]
__global__ void k_reduce_chunks(const double2* __restrict__ A_part, int nchunks, int nk, double2* __restrict__ A1) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nk) return;
    double r = 0.0, i = 0.0;
    for (int c = 0; c < nchunks; ++c) { const double2 v = A_part[(long long)c * nk + n]; r += v.x; i += v.y; }
    A1[n] = make_double2(r, i);
}

void launch_sep_sweep(int precision, const double* kk, int nk, const SepDevice& s, void* Tt,
                      double2* A_part, double2* A1, cudaStream_t st) {
    dim3 grid(ceil_div(nk, kSweepRows), s.nchunks);
    if (precision == SGL_FP64)
        { k_sep_sweep_f64<<<grid, kSweepRows, 0, st>>>(kk, nk, s, (double*)Tt, A_part); SGL_COUNT(1); }
    else
        { k_sep_sweep_mixed<<<grid, kSweepRows, 0, st>>>(kk, nk, s, (float*)Tt, A_part); SGL_COUNT(1); }
    { k_reduce_chunks<<<ceil_div(nk, 256), 256, 0, st>>>(A_part, s.nchunks, nk, A1); SGL_COUNT(1); }
}

// ------------------------------------------------------------------ tables
// B[r, j] = J0(node_r * x_j) - 1 (row-major, ld = nx), in TT.
template <typename TT>
__global__ void k_j0m1_table(const double* __restrict__ nodes, int nn, const double* __restrict__ x, int nx,
                             TT* __restrict__ B) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nn * nx) return;
    const int r = (int)(e / nx), j = (int)(e % nx);
    B[e] = (TT)j0m1_d(nodes[r] * x[j]);
}

__global__ void k_j0m1_table_mixed(const double* __restrict__ nodes, int nn, const double* __restrict__ x, int nx,
                                   float* __restrict__ B) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nn * nx) return;
    const int r = (int)(e / nx), j = (int)(e % nx);
    B[e] = j0m1_mixed(nodes[r], x[j]);
}

void launch_j0m1_table(int precision, const double* nodes, int nn, const double* x, int nx, void* B, cudaStream_t st) {
    const long long tot = (long long)nn * nx;
    if (tot == 0) return;
    if (precision == SGL_FP64) { k_j0m1_table<double><<<ceil_div(tot, 256), 256, 0, st>>>(nodes, nn, x, nx, (double*)B); SGL_COUNT(1); }
    else { k_j0m1_table_mixed<<<ceil_div(tot, 256), 256, 0, st>>>(nodes, nn, x, nx, (float*)B); SGL_COUNT(1); }
}

// Barycentric Chebyshev-Lobatto interpolation matrix L (nx x N): points t_j = K/2 (1 - cos(j pi/(N-1))),
// weights (-1)^j halved at both ends; a point within 1e-14 K of a node gets the exact unit row.
// One CTA per row.
// The points t_j come precomputed (k_cheb_points, the same expression); each row keeps its terms
// wb / (x - t_j) in shared memory between the sum and the normalisation (the first kChebSmem of
// them; any beyond are recomputed).
constexpr int kChebSmem = 4096;

template <typename TT>
__global__ void __launch_bounds__(256)
k_cheb_matrix(double K, int N, const double* __restrict__ tpts, const double* __restrict__ x, int nx,
              TT* __restrict__ L) {
    __shared__ double sh[32];
    __shared__ double s_q[kChebSmem];
    __shared__ int s_hit;
    const int m = blockIdx.x;
    const double xm = x[m];
    if (threadIdx.x == 0) s_hit = -1;
    __syncthreads();
    double part = 0.0;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double d = xm - tpts[j];
        const bool at = fabs(d) <= 1e-14 * K;
        if (at) atomicMax(&s_hit, j);
        double wb = (j & 1) ? -1.0 : 1.0;
        if (j == 0 || j == N - 1) wb *= 0.5;
        const double q = wb / (at ? 1.0 : d);
        if (j < kChebSmem) s_q[j] = q;
        part += q;
    }
    const double tot = block_sum(part, sh);
    const int hit = s_hit;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        double v;
        if (hit >= 0) v = (j == hit) ? 1.0 : 0.0;
        else if (j < kChebSmem) v = s_q[j] / tot;
        else {
            double wb = (j & 1) ? -1.0 : 1.0;
            if (j == 0 || j == N - 1) wb *= 0.5;
            v = (wb / (xm - tpts[j])) / tot;
        }
        L[(long long)m * N + j] = (TT)v;
    }
}

void launch_cheb_matrix(int precision, double K, int N, const double* tpts, const double* x, int nx, void* L,
                        cudaStream_t st) {
    if (precision == SGL_FP64) { k_cheb_matrix<double><<<nx, 256, 0, st>>>(K, N, tpts, x, nx, (double*)L); SGL_COUNT(1); }
    else { k_cheb_matrix<float><<<nx, 256, 0, st>>>(K, N, tpts, x, nx, (float*)L); SGL_COUNT(1); }
}

__global__ void k_cheb_points(double K, int N, double* __restrict__ t) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < N) t[j] = 0.5 * K * (1.0 - cos(j * M_PI / (N - 1)));
}

void launch_cheb_points(double K, int N, double* t, cudaStream_t st) {
    { k_cheb_points<<<ceil_div(N, 256), 256, 0, st>>>(K, N, t); SGL_COUNT(1); }
}

}  // namespace sgl
