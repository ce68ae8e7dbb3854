// Composition of ln Phi on the full grid and the GEMM launchers.
//
// ln Phi(n, m) = [separable GEMM output](n, m) + A1[n] - 1/2 kk_n^2 V + Q(n, m)
// where Q is the not-a-knot bicubic spline of the coarse-grid xi_lin term (reference:
// Lam._Q_interpolated, sgl_full.py:2998-3022): with coefficients C = Mk Qc Mg^T on the knot
// vectors of s = linspace(0, 1, n), Q(n, m) = sum_a sum_b Bk[n, a] C[lk + a, lg + b] Bg[m, b],
// B the cubic B-spline basis (de Boor's recursion) at s = sqrt(clip(k / kmax, 0, 1)).
#include "kernels.cuh"

namespace sgl {

std::atomic<long long>& launch_counter() {
    static std::atomic<long long> n{0};      // contexts may run on several host threads
    return n;
}

// ------------------------------------------------------------------ GEMM launchers
// The layout kernel's shared memory (operand tiles + running sums) is above the 48 KB static
// limit: opted in once per instantiation.
template <bool AK, bool BJ>
void launch_f32_layout(const GemmDesc<float>* d_descs, int nprob, int tiles, cudaStream_t st) {
    static const bool opted = cudaFuncSetAttribute(gemm_f32_layout_kernel<AK, BJ>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   kF32LayoutSmem) == cudaSuccess;
    (void)opted;
    gemm_f32_layout_kernel<AK, BJ><<<tiles, 256, kF32LayoutSmem, st>>>(d_descs, nprob);
    SGL_COUNT(1);
}

// layout (FP32): bit 0 = every A is k-contiguous, bit 1 = every B is j-contiguous, -1 = mixed.
// layout kSmallTiles (FP64): the descriptors were planned with 16 x 16 tiles.
template <typename T>
void launch_grouped_gemm(const GemmDesc<T>* d_descs, int nprob, int tiles, int layout, cudaStream_t st) {
    if (tiles <= 0) return;
    if constexpr (sizeof(T) == 8) {
        if (layout == kSmallTiles) {
            gemm_f64_small_kernel<16><<<tiles, 256, 0, st>>>(d_descs, nprob);
            SGL_COUNT(1);
            return;
        }
    }
    if constexpr (sizeof(T) == 4) {
        switch (layout) {
            case 0: launch_f32_layout<false, false>(d_descs, nprob, tiles, st); return;
            case 1: launch_f32_layout<true, false>(d_descs, nprob, tiles, st); return;
            case 2: launch_f32_layout<false, true>(d_descs, nprob, tiles, st); return;
            case 3: launch_f32_layout<true, true>(d_descs, nprob, tiles, st); return;
            default: break;
        }
    }
    { grouped_gemm_kernel<T><<<tiles, 256, 0, st>>>(d_descs, nprob); SGL_COUNT(1); }
}
template void launch_grouped_gemm<double>(const GemmDesc<double>*, int, int, int, cudaStream_t);
template void launch_grouped_gemm<float>(const GemmDesc<float>*, int, int, int, cudaStream_t);

// out(i, j) = sum_s ws[s, i, j] (+ beta out(i, j)); ws slices are dense rows x cols, out has row
// stride ldo.  Grid (column blocks, rows).  FP64 slices are summed in FP64.  FP32 slices are summed
// in float-float (Knuth's TwoSum, errors accumulated in a second float): about 48 significant
// bits, as accurate as an FP64 sum for a float result, with no FP64 arithmetic.
template <typename T>
__global__ void k_sum_slices(const T* __restrict__ ws, int ns, int rows, int cols, T* __restrict__ out, long long ldo,
                             T beta) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    const long long n = (long long)rows * cols;
    for (int i = blockIdx.y; i < rows; i += gridDim.y) {
        const long long e = (long long)i * cols + j;
        T* o = out + (long long)i * ldo + j;
        if constexpr (sizeof(T) == 8) {
            double acc = 0.0;
            for (int s = 0; s < ns; ++s) acc += ws[(long long)s * n + e];
            *o = (beta != T(0)) ? acc + beta * *o : acc;
        } else {
            float hi = 0.f, lo = 0.f;
            auto add = [&](float v) {
                const float t = hi + v, bp = t - hi;
                lo += (hi - (t - bp)) + (v - bp);
                hi = t;
            };
            for (int s = 0; s < ns; ++s) add(ws[(long long)s * n + e]);
            if (beta != 0.f) {
                const float ov = *o, p = beta * ov;
                lo += fmaf(beta, ov, -p);
                add(p);
            }
            *o = hi + lo;
        }
    }
}

template <typename T>
void launch_sum_slices(const T* ws, int ns, int rows, int cols, T* out, long long ldo, T beta, cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return;
    dim3 grid(ceil_div(cols, 128), std::min(rows, 65535));
    { k_sum_slices<T><<<grid, 128, 0, st>>>(ws, ns, rows, cols, out, ldo, beta); SGL_COUNT(1); }
}
template void launch_sum_slices<double>(const double*, int, int, int, double*, long long, double, cudaStream_t);
template void launch_sum_slices<float>(const float*, int, int, int, float*, long long, float, cudaStream_t);

// ------------------------------------------------------------------ spline basis
// Knots t[0..ncoef+3]; find l in [3, ncoef-1] with t[l] <= s < t[l+1] (s = t[ncoef] -> last
// interval), then the 4 nonzero cubic basis values B_{l-3..l}(s).
__global__ void k_spline_basis(const double* __restrict__ x, int n, double xmax, const double* __restrict__ t,
                               int ncoef, int* __restrict__ lout, double* __restrict__ bout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = x[i] / xmax;
    s = fmin(fmax(s, 0.0), 1.0);
    s = sqrt(s);
    int lo = 3, hi = ncoef - 1;          // search the interval
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (t[mid] <= s) lo = mid; else hi = mid - 1;
    }
    const int l = lo;
    double N[4], left[4], right[4];
    N[0] = 1.0;
    for (int j = 1; j <= 3; ++j) {
        left[j] = s - t[l + 1 - j];
        right[j] = t[l + j] - s;
        double saved = 0.0;
        for (int r = 0; r < j; ++r) {
            const double temp = N[r] / (right[r + 1] + left[j - r]);
            N[r] = saved + right[r + 1] * temp;
            saved = left[j - r] * temp;
        }
        N[j] = saved;
    }
    lout[i] = l - 3;
    for (int a = 0; a < 4; ++a) bout[4 * i + a] = N[a];
}

void launch_spline_basis(const double* x, int n, double xmax, const double* knots, int ncoef, int* l, double* b,
                         cudaStream_t st) {
    { k_spline_basis<<<ceil_div(n, 128), 128, 0, st>>>(x, n, xmax, knots, ncoef, l, b); SGL_COUNT(1); }
}

// ------------------------------------------------------------------ finalize
// G: GEMM output planes (rows 0..nk-1 real, nk..2nk-1 imaginary), ld = nkg.
// write_phi = 0: out = ln Phi (double planes); 1: out = Phi = exp(ln Phi) (TT planes).
template <typename TT, int WRITE_PHI>
__global__ void k_finalize(const TT* __restrict__ G, int nk, int nkg, const double2* __restrict__ A1,
                           const double* __restrict__ kk, double V, const double* __restrict__ Cre,
                           const double* __restrict__ Cim, int ncg, SplineAxis sk, SplineAxis sg,
                           void* __restrict__ out_re, void* __restrict__ out_im, long long ld_out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (m >= nkg) return;
    const long long e = (long long)n * nkg + m;
    const double k = kk[n];
    double re = (double)G[e] + A1[n].x - 0.5 * (k * k * V);
    double im = (double)G[(long long)nk * nkg + e] + A1[n].y;
    if (Cre != nullptr) {
        const int lk = sk.l[n], lg = sg.l[m];
        double qr = 0.0, qi = 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const double ba = sk.b[4 * n + a];
            double rr = 0.0, ri = 0.0;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const double bb = sg.b[4 * m + b];
                const long long ci = (long long)(lk + a) * ncg + (lg + b);
                rr = fma(bb, Cre[ci], rr);
                ri = fma(bb, Cim[ci], ri);
            }
            qr = fma(ba, rr, qr);
            qi = fma(ba, ri, qi);
        }
        re += qr;
        im += qi;
    }
    const long long eo = (long long)n * ld_out + m;
    if (WRITE_PHI == 0) {
        ((double*)out_re)[eo] = re;
        ((double*)out_im)[eo] = im;
    } else {
        const double mag = exp(re);
        double s, c;
        sincos(im, &s, &c);
        ((TT*)out_re)[eo] = (TT)(mag * c);
        ((TT*)out_im)[eo] = (TT)(mag * s);
    }
}

__global__ void k_to_float(const double* __restrict__ src, float* __restrict__ dst, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}

void launch_to_float(const double* src, float* dst, long long n, cudaStream_t st) {
    if (n > 0) { k_to_float<<<ceil_div(n, 256), 256, 0, st>>>(src, dst, n); SGL_COUNT(1); }
}

// Mixed path with FP32 spline: the xi term's bicubic spline is a convex combination of its
// coefficients (B-spline weights >= 0, summing to 1), so FP32 evaluation adds ~1e-7 of |Q| to
// ln Phi (at most ~4e-8 of Phi, as Phi <= e^{-|Q|}); the sum of the large terms of ln Phi and
// the reduction of its phase stay FP64.
__global__ void k_finalize_mixed(const float* __restrict__ G, int nk, int nkg, const double2* __restrict__ A1,
                                 const double* __restrict__ kk, double V, const float* __restrict__ Cre,
                                 const float* __restrict__ Cim, int ncg, SplineAxis sk, SplineAxis sg,
                                 float* __restrict__ out_re, float* __restrict__ out_im, long long ld_out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (m >= nkg) return;
    const long long e = (long long)n * nkg + m;
    const double k = kk[n];
    double re = (double)G[e] + A1[n].x - 0.5 * (k * k * V);
    double im = (double)G[(long long)nk * nkg + e] + A1[n].y;
    if (Cre != nullptr) {
        const int lk = sk.l[n], lg = sg.l[m];
        const float4 bk = *reinterpret_cast<const float4*>(sk.bf + 4 * n);
        const float4 bg = *reinterpret_cast<const float4*>(sg.bf + 4 * m);
        const float bka[4] = {bk.x, bk.y, bk.z, bk.w}, bgb[4] = {bg.x, bg.y, bg.z, bg.w};
        float qr = 0.f, qi = 0.f;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            float rr = 0.f, ri = 0.f;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const long long ci = (long long)(lk + a) * ncg + (lg + b);
                rr = fmaf(bgb[b], Cre[ci], rr);
                ri = fmaf(bgb[b], Cim[ci], ri);
            }
            qr = fmaf(bka[a], rr, qr);
            qi = fmaf(bka[a], ri, qi);
        }
        re += (double)qr;
        im += (double)qi;
    }
    const double two_pi = 6.283185307179586;
    const double qn = rint(im * (1.0 / two_pi));
    const float r = (float)fma(-qn, two_pi, im);
    float s, c;
    sincosf(r, &s, &c);
    const float mag = expf((float)re);
    const long long eo = (long long)n * ld_out + m;
    out_re[eo] = mag * c;
    out_im[eo] = mag * s;
}

// Mixed path exp: the phase is reduced mod 2 pi in FP64, the rest is FP32.
template <>
__global__ void k_finalize<float, 1>(const float* __restrict__ G, int nk, int nkg, const double2* __restrict__ A1,
                                     const double* __restrict__ kk, double V, const double* __restrict__ Cre,
                                     const double* __restrict__ Cim, int ncg, SplineAxis sk, SplineAxis sg,
                                     void* __restrict__ out_re, void* __restrict__ out_im, long long ld_out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    if (m >= nkg) return;
    const long long e = (long long)n * nkg + m;
    const double k = kk[n];
    double re = (double)G[e] + A1[n].x - 0.5 * (k * k * V);
    double im = (double)G[(long long)nk * nkg + e] + A1[n].y;
    if (Cre != nullptr) {
        const int lk = sk.l[n], lg = sg.l[m];
        double qr = 0.0, qi = 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const double ba = sk.b[4 * n + a];
            double rr = 0.0, ri = 0.0;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const double bb = sg.b[4 * m + b];
                const long long ci = (long long)(lk + a) * ncg + (lg + b);
                rr = fma(bb, Cre[ci], rr);
                ri = fma(bb, Cim[ci], ri);
            }
            qr = fma(ba, rr, qr);
            qi = fma(ba, ri, qi);
        }
        re += qr;
        im += qi;
    }
    const double two_pi = 6.283185307179586;
    const double qn = rint(im * (1.0 / two_pi));
    const float r = (float)fma(-qn, two_pi, im);
    float s, c;
    sincosf(r, &s, &c);
    const float mag = expf((float)re);
    const long long eo = (long long)n * ld_out + m;
    ((float*)out_re)[eo] = mag * c;
    ((float*)out_im)[eo] = mag * s;
}

void launch_finalize(int precision, int write_phi, const void* G, int nk, int nkg, const double2* A1, const double* kk,
                     double V, const double* C_re, const double* C_im, int ncg, SplineAxis sk, SplineAxis sg,
                     void* out_re, void* out_im, long long ld_out, cudaStream_t st, const float* Cf, long long nq) {
    dim3 grid(ceil_div(nkg, 128), nk);
    if (precision == SGL_MIXED && write_phi && (C_re == nullptr || (Cf && sk.bf && sg.bf))) {
        k_finalize_mixed<<<grid, 128, 0, st>>>((const float*)G, nk, nkg, A1, kk, V, C_re ? Cf : nullptr,
                                               C_re ? Cf + nq : nullptr, ncg, sk, sg, (float*)out_re,
                                               (float*)out_im, ld_out);
        SGL_COUNT(1);
        return;
    }
    if (precision == SGL_FP64) {
        if (write_phi) { k_finalize<double, 1><<<grid, 128, 0, st>>>((const double*)G, nk, nkg, A1, kk, V, C_re, C_im, ncg, sk, sg, out_re, out_im, ld_out); SGL_COUNT(1); }
        else { k_finalize<double, 0><<<grid, 128, 0, st>>>((const double*)G, nk, nkg, A1, kk, V, C_re, C_im, ncg, sk, sg, out_re, out_im, ld_out); SGL_COUNT(1); }
    } else {
        if (write_phi) { k_finalize<float, 1><<<grid, 128, 0, st>>>((const float*)G, nk, nkg, A1, kk, V, C_re, C_im, ncg, sk, sg, out_re, out_im, ld_out); SGL_COUNT(1); }
        else { k_finalize<float, 0><<<grid, 128, 0, st>>>((const float*)G, nk, nkg, A1, kk, V, C_re, C_im, ncg, sk, sg, out_re, out_im, ld_out); SGL_COUNT(1); }
    }
}

}  // namespace sgl
