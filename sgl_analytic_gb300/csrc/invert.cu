// Inversion Phi(k_kappa, k_gamma) -> P3(kappa, gamma) -> P_s(ln mu)
// (reference: sgl.P_vector_joint sgl.py:1127-1156, sgl_full.invert sgl_full.py:272-360).
//
//   Hankel   F[n, j]   = sum_m Phi[n, m] k_g[m] w_g[m] J0(gam_j k_g[m])         (GEMM, M matrix)
//   kappa    P3[i, j]  = 1/(2 pi^2) sum_n w_k[n] Re(e^{-i kap_i k_n} F[n, j])   (GEMM, CS matrix)
//   E-M      P3       += a(kap) + b(kap) gam^2 from Phi[:, 0], Phi[:, 1]        (2 extra F columns)
//   path     P_i(xi)   = pi / mu^2 int P3(kap, gam(kap; mu)) dkap  (+ gamma-parametrised tail)
#include "kernels.cuh"

namespace sgl {

// M[m, j] = k_g[m] w_g[m] J0(gam_j k_g[m]),  w_g = dk_g (halved at both ends); row stride ld.
// FP32 (mixed path): M = M_hi + M_lo, both FP32, M_lo written nkg * ld elements after M_hi --
// the Hankel sum's rounding of M would otherwise dominate the PDF tail error.
template <typename TT>
__global__ void k_hankel_matrix(const double* __restrict__ kg, int nkg, double dkg, const double* __restrict__ gam,
                                int ngam, int ld, TT* __restrict__ M) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nkg * ngam) return;
    const int m = (int)(e / ngam), j = (int)(e % ngam);
    double w = dkg;
    if (m == 0 || m == nkg - 1) w *= 0.5;
    const double v = (kg[m] * w) * j0(gam[j] * kg[m]);
    const TT hi = (TT)v;
    M[(long long)m * ld + j] = hi;
    if (sizeof(TT) == 4) M[(long long)nkg * ld + (long long)m * ld + j] = (TT)(v - (double)hi);
}

void launch_hankel_matrix(int precision, const double* kg, int nkg, double dkg, const double* gam, int ngam, int ld,
                          void* M, cudaStream_t st) {
    const long long tot = (long long)nkg * ngam;
    if (precision == SGL_FP64) { k_hankel_matrix<double><<<ceil_div(tot, 256), 256, 0, st>>>(kg, nkg, dkg, gam, ngam, ld, (double*)M); SGL_COUNT(1); }
    else { k_hankel_matrix<float><<<ceil_div(tot, 256), 256, 0, st>>>(kg, nkg, dkg, gam, ngam, ld, (float*)M); SGL_COUNT(1); }
}

// CS[i, n] = cos(kap_i k_n) w_k[n],  CS[i, nk + n] = sin(kap_i k_n) w_k[n]
template <typename TT>
__global__ void k_kappa_matrix(const double* __restrict__ kk, int nk, double dkk, const double* __restrict__ kap,
                               int nkap, TT* __restrict__ CS) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nkap * nk) return;
    const int i = (int)(e / nk), n = (int)(e % nk);
    double w = dkk;
    if (n == 0 || n == nk - 1) w *= 0.5;
    double s, c;
    sincos(kap[i] * kk[n], &s, &c);
    CS[(long long)i * 2 * nk + n] = (TT)(c * w);
    CS[(long long)i * 2 * nk + nk + n] = (TT)(s * w);
}

// Mixed path: the same matrix with no FP64 transcendental (float-float phase, exact reduction,
// FP32 sin / cos of the reduced argument).  One CTA per kappa row.
__global__ void k_kappa_matrix_ff(const double* __restrict__ kk, int nk, double dkk, const double* __restrict__ kap,
                                  float* __restrict__ CS) {
    const int i = blockIdx.x;
    const ff kf = ff_from_double(kap[i]);
    const float wf = (float)dkk, wh = (float)(0.5 * dkk);
    float* row = CS + (long long)i * 2 * nk;
    for (int n = threadIdx.x; n < nk; n += blockDim.x) {
        float s, c;
        sincos_ff(ff_from_double(kk[n]), kf, s, c);
        const float w = (n == 0 || n == nk - 1) ? wh : wf;
        row[n] = c * w;
        row[nk + n] = s * w;
    }
}

void launch_kappa_matrix(int precision, const double* kk, int nk, double dkk, const double* kap, int nkap, void* CS,
                         cudaStream_t st) {
    const long long tot = (long long)nkap * nk;
    if (precision == SGL_FP64) { k_kappa_matrix<double><<<ceil_div(tot, 256), 256, 0, st>>>(kk, nk, dkk, kap, nkap, (double*)CS); SGL_COUNT(1); }
    else if (nkap > 0) { k_kappa_matrix_ff<<<nkap, 256, 0, st>>>(kk, nk, dkk, kap, (float*)CS); SGL_COUNT(1); }
}

// Euler-Maclaurin endpoint columns (sgl_full.py:277-298): from Phi0 = Phi[:, 0], Phi1 = Phi[:, 1],
// Phi2 = (Phi1 - Phi0)/dkg^2, va = dkg^2/12 Phi0 - dkg^4/120 Phi2, vb = dkg^4/480 Phi0, written into
// columns col (va) and col + 1 (vb) of F (real rows then imaginary rows).
template <typename TT>
__global__ void k_em_columns(const TT* __restrict__ Phi, int nk, int nkg, double dkg, TT* __restrict__ F, int ldF,
                             int col) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nk) return;
    const long long im_off = (long long)nk * nkg;
    const double p0r = (double)Phi[(long long)n * nkg], p0i = (double)Phi[im_off + (long long)n * nkg];
    const double p1r = (double)Phi[(long long)n * nkg + 1], p1i = (double)Phi[im_off + (long long)n * nkg + 1];
    const double d2 = dkg * dkg, d4 = d2 * d2;
    const double p2r = (p1r - p0r) / d2, p2i = (p1i - p0i) / d2;
    F[(long long)n * ldF + col] = (TT)((d2 / 12.0) * p0r - (d4 / 120.0) * p2r);
    F[(long long)(nk + n) * ldF + col] = (TT)((d2 / 12.0) * p0i - (d4 / 120.0) * p2i);
    F[(long long)n * ldF + col + 1] = (TT)((d4 / 480.0) * p0r);
    F[(long long)(nk + n) * ldF + col + 1] = (TT)((d4 / 480.0) * p0i);
}

void launch_em_columns(int precision, const void* Phi, int nk, int nkg, double dkg, void* F, int ldF, int col,
                       cudaStream_t st) {
    if (precision == SGL_FP64) { k_em_columns<double><<<ceil_div(nk, 128), 128, 0, st>>>((const double*)Phi, nk, nkg, dkg, (double*)F, ldF, col); SGL_COUNT(1); }
    else { k_em_columns<float><<<ceil_div(nk, 128), 128, 0, st>>>((const float*)Phi, nk, nkg, dkg, (float*)F, ldF, col); SGL_COUNT(1); }
}

// Phi[i, j] *= wk[i] wg[j] on both planes (positive-definite box window, sgl_full.py:83-94)
template <typename TT>
__global__ void k_window(TT* __restrict__ Phi, int nk, int nkg, const double* __restrict__ wk,
                         const double* __restrict__ wg) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long npt = (long long)nk * nkg;
    if (e >= npt) return;
    const double w = wk[e / nkg] * wg[e % nkg];
    Phi[e] = (TT)((double)Phi[e] * w);
    Phi[npt + e] = (TT)((double)Phi[npt + e] * w);
}

// out[e] = (float)in[e]: a caller's FP64 Phi planes taken into the mixed path's FP32 layout
__global__ void k_phi_to_f32(const double* __restrict__ in, long long n, float* __restrict__ out) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) out[e] = (float)in[e];
}

void launch_phi_to_f32(const double* in, long long n, float* out, cudaStream_t st) {
    if (n <= 0) return;
    k_phi_to_f32<<<ceil_div(n, 256), 256, 0, st>>>(in, n, out);
    SGL_COUNT(1);
}

void launch_window(int precision, void* Phi, int nk, int nkg, const double* wk, const double* wg, cudaStream_t st) {
    const long long tot = (long long)nk * nkg;
    if (precision == SGL_FP64) { k_window<double><<<ceil_div(tot, 256), 256, 0, st>>>((double*)Phi, nk, nkg, wk, wg); SGL_COUNT(1); }
    else { k_window<float><<<ceil_div(tot, 256), 256, 0, st>>>((float*)Phi, nk, nkg, wk, wg); SGL_COUNT(1); }
}

// P3[i, j] = P3ext[i, j] + P3ext[i, ngam] + P3ext[i, ngam + 1] gam_j^2  (already scaled by 1/(2 pi^2))
// The mixed path also writes a float copy P3f (the values carry FP32 accuracy already: P3ext is
// FP32 there) for the FP32 path integral.
template <typename TT>
__global__ void k_p3_finish(const TT* __restrict__ P3ext, int nkap, int ngam, int ld, const double* __restrict__ gam,
                            double* __restrict__ P3, float* __restrict__ P3f) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nkap * ngam) return;
    const int i = (int)(e / ngam), j = (int)(e % ngam);
    const TT* row = P3ext + (long long)i * ld;
    const double g = gam[j];
    const double v = (double)row[j] + (double)row[ngam] + (double)row[ngam + 1] * (g * g);
    P3[e] = v;
    if (P3f) P3f[e] = (float)v;
}

void launch_p3_finish(int precision, const void* P3ext, int nkap, int ngam, int ld, const double* gam, double* P3,
                      float* P3f, cudaStream_t st) {
    const long long tot = (long long)nkap * ngam;
    if (precision == SGL_FP64) { k_p3_finish<double><<<ceil_div(tot, 256), 256, 0, st>>>((const double*)P3ext, nkap, ngam, ld, gam, P3, P3f); SGL_COUNT(1); }
    else { k_p3_finish<float><<<ceil_div(tot, 256), 256, 0, st>>>((const float*)P3ext, nkap, ngam, ld, gam, P3, P3f); SGL_COUNT(1); }
}

// ------------------------------------------------------------------ path integral
// Uniform axis a_i = a0 + i h (numpy linspace); RegularGridInterpolator linear semantics: cell
// i = floor((x - a0) / h) clipped to [0, n-2], weight t = (x - a0) / h - i, and 0 outside [a0, a1].
// GB300's FP64 pipe is ~1/74 of FP32, so the per-point work is kept to a few FP64 operations:
// no divisions (reciprocal steps precomputed), one sqrt per path point, and the blend written
// as v00 + t_x (v10 - v00) + t_y (v01 - v00 + t_x (v11 - v10 - v01 + v00)).  Against the
// reference's node-exact interval search this moves P by ~1e-16 relative.
struct Axis { double a0, a1, h, inv_h; int n; };

__device__ __forceinline__ double bilinear(const double* __restrict__ P3, const Axis& K, const Axis& G, double x,
                                           double y) {
    if (!(x >= K.a0 && x <= K.a1 && y >= G.a0 && y <= G.a1)) return 0.0;
    const double fx = (x - K.a0) * K.inv_h, fy = (y - G.a0) * G.inv_h;
    const int i = min(max((int)fx, 0), K.n - 2), j = min(max((int)fy, 0), G.n - 2);
    const double tx = fx - (double)i, ty = fy - (double)j;
    const double* p = P3 + (long long)i * G.n + j;
    const double v00 = __ldg(p), v01 = __ldg(p + 1), v10 = __ldg(p + G.n), v11 = __ldg(p + G.n + 1);
    const double d10 = v10 - v00, d01 = v01 - v00;
    return fma(tx, d10, v00) + ty * fma(tx, (v11 - v10) - d01, d01);
}

// The gamma-parametrised tail of the path (FP64 on P3), shared by both precisions.
__device__ double path_tail(const double* __restrict__ P3, const Axis& K, const Axis& G, double mu, double hi,
                            double lo, double c1, double pref, double gmax, double g_def, double* sh) {
    double total = 0.0;
    if (gmax > g_def && lo > K.a0) {
        const double gb = fmin(gmax, sqrt(fmax((hi - K.a0) * (c1 - K.a0), 0.0)));
        if (gb > g_def) {
            const int n = (int)ceil((gb - g_def) / (0.5 * G.h)) + 1;
            const double gstep = (gb - g_def) / (double)(n - 1);
            const double imu = 1.0 / mu;
            double acc2 = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const double ga = (i == n - 1) ? gb : fma((double)i, gstep, g_def);
                const double ra = sqrt(fma(ga, ga, imu));
                const double ka = fmin(fmax(1.0 - ra, K.a0), K.a1);
                const double v = bilinear(P3, K, G, ka, ga) * (ga / ra);
                acc2 += (i == 0 || i == n - 1) ? 0.5 * v : v;
            }
            total = pref * gstep * block_sum(acc2, sh);
        }
    }
    return total;
}

// One CTA per xi.  Body: n_k_int points kappa in [lo, hi], gamma = sqrt((hi - k)(1 - k + 1/sqrt(mu))),
// trapezoid in kappa (uniform step: endpoints halved); tail (gamma in (g_def, gb]) parametrised in
// gamma with weight gamma / r.
__global__ void __launch_bounds__(256)
k_path_integral(const double* __restrict__ P3, Axis K, Axis G, const double* __restrict__ xi, double gmax,
                double g_def, int n_k_int, double* __restrict__ out) {
    __shared__ double sh[32];
    const double x = xi[blockIdx.x];
    const double mu = exp(x);
    const double rm = 1.0 / sqrt(mu);
    const double hi = 1.0 - rm;
    const double lo = fmax(K.a0, 1.0 - sqrt(1.0 / mu + g_def * g_def));
    const double pref = M_PI / (mu * mu);
    if (!(hi > lo)) { if (threadIdx.x == 0) out[blockIdx.x] = 0.0; return; }
    const double step = (hi - lo) / (double)(n_k_int - 1);
    const double c1 = 1.0 + rm;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n_k_int; i += blockDim.x) {
        const double k0 = (i == n_k_int - 1) ? hi : fma((double)i, step, lo);
        const double g0 = sqrt(fmax((hi - k0) * (c1 - k0), 0.0));
        const double v = bilinear(P3, K, G, k0, g0);
        acc += (i == 0 || i == n_k_int - 1) ? 0.5 * v : v;
    }
    double total = pref * step * block_sum(acc, sh);
    total += path_tail(P3, K, G, mu, hi, lo, c1, pref, gmax, g_def, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = total;
}

// Mixed path tail in FP32 on P3f: gamma_a = g_def + i gstep, r = sqrt(gamma^2 + 1/mu) and
// kappa = 1 - r formed as (1 - 1/mu - gamma^2) / (1 + r), with 1 - 1/mu from FP64 and gamma^2
// exact by FMA, so kappa keeps ~1e-7 relative accuracy where 1 - r cancels; the cell positions
// take one FP64 FMA each.
__device__ double path_tail_f32(const float* __restrict__ P3f, const Axis& K, const Axis& G, double mu, double hi,
                                double lo, double c1, double pref, double gmax, double g_def, double* sh) {
    if (!(gmax > g_def && lo > K.a0)) return 0.0;
    const double gb = fmin(gmax, sqrt(fmax((hi - K.a0) * (c1 - K.a0), 0.0)));
    if (!(gb > g_def)) return 0.0;
    const int n = (int)ceil((gb - g_def) / (0.5 * G.h)) + 1;
    const double gstep = (gb - g_def) / (double)(n - 1);
    const double om = 1.0 - 1.0 / mu;
    const float om_hi = (float)om, om_lo = (float)(om - (double)om_hi);
    const float imu = (float)(1.0 / mu), gs = (float)gstep, gd = (float)g_def, gbf = (float)gb;
    const float ginv = (float)G.inv_h, k_lo = (float)K.a0, k_hi = (float)K.a1;
    const double kx0 = -K.a0 * K.inv_h;
    const int nK = K.n, nG = G.n;
    float acc = 0.f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float ga = (i == n - 1) ? gbf : fmaf((float)i, gs, gd);
        const float ra = sqrtf(fmaf(ga, ga, imu));
        const float p = ga * ga, pe = fmaf(ga, ga, -p);
        const float ka = fminf(fmaxf(((om_hi - p) + (om_lo - pe)) / (1.f + ra), k_lo), k_hi);
        // kappa is clamped to the box and gamma <= gb <= the box edge, as in the FP64 form: the
        // positions are clamped to the grid rather than tested
        const double fx = fmin(fmax(fma((double)ka, K.inv_h, kx0), 0.0), (double)(nK - 1));
        const float fy = fminf(ga * ginv, (float)(nG - 1));
        const int ix = min((int)fx, nK - 2), j = min((int)fy, nG - 2);
        const float t = (float)(fx - (double)ix), ty = fy - (float)j;
        const float* q = P3f + (long long)ix * nG + j;
        const float v00 = __ldg(q), v01 = __ldg(q + 1), v10 = __ldg(q + nG), v11 = __ldg(q + nG + 1);
        const float d10 = v10 - v00, d01 = v01 - v00;
        const float v = (fmaf(t, d10, v00) + ty * fmaf(t, (v11 - v10) - d01, d01)) * (ga / ra);
        acc += (i == 0 || i == n - 1) ? 0.5f * v : v;
    }
    return pref * gstep * block_sum((double)acc, sh);
}

// Mixed path: the body's points in FP32 on the float copy of P3.  The FP64 constants of each xi
// are formed once per CTA.  Per point, hi - k = (n - 1 - i) step and c1 - k = 2 rm + (hi - k)
// avoid the cancellation of forming k, and the kappa cell position (lo - a0)/h + i step/h is
// carried as an integer plus a float-float fraction (the products made exact with FMA), so the
// interpolation weights keep ~1e-7 of a cell at every point.  The tail stays FP64.
__global__ void __launch_bounds__(256)
k_path_integral_f32(const float* __restrict__ P3f, const double* __restrict__ P3, Axis K, Axis G,
                    const double* __restrict__ xi, double gmax, double g_def, int n_k_int, double* __restrict__ out) {
    __shared__ double sh[32];
    __shared__ double cd[8];
    __shared__ float cf[6];
    __shared__ int ci[2];
    if (threadIdx.x == 0) {
        const double x = xi[blockIdx.x];
        const double mu = exp(x), rm = 1.0 / sqrt(mu);
        const double hi = 1.0 - rm;
        const double lo = fmax(K.a0, 1.0 - sqrt(1.0 / mu + g_def * g_def));
        const double step = (hi - lo) / (double)(n_k_int - 1);
        const double base = (lo - K.a0) * K.inv_h, bfl = floor(base);
        const double ss = step * K.inv_h;
        cd[0] = mu; cd[1] = hi; cd[2] = lo; cd[3] = 1.0 + rm; cd[4] = M_PI / (mu * mu); cd[5] = step;
        ci[0] = hi > lo; ci[1] = (int)bfl;
        cf[0] = (float)(base - bfl);
        cf[1] = (float)ss; cf[2] = (float)(ss - (double)cf[1]);
        cf[3] = (float)step; cf[4] = (float)(2.0 * rm); cf[5] = (float)G.inv_h;
    }
    __syncthreads();
    if (!ci[0]) { if (threadIdx.x == 0) out[blockIdx.x] = 0.0; return; }
    const int bi = ci[1], nK = K.n, nG = G.n;
    const float bf = cf[0], sh_hi = cf[1], sh_lo = cf[2], step_f = cf[3], two_rm = cf[4], ginv = cf[5];
    float acc = 0.f;
    for (int i = threadIdx.x; i < n_k_int; i += blockDim.x) {
        const float fi = (float)i;
        const float d = (float)(n_k_int - 1 - i) * step_f;               // hi - k
        const float g = sqrtf(fmaxf(d * (two_rm + d), 0.f));
        // kappa cell: bf + fi * ss as (integer cell, fraction t)
        const float p = fi * sh_hi;
        const float e = fmaf(fi, sh_hi, -p) + fi * sh_lo;
        const float s = bf + p, bp = s - bf;
        const float e2 = (bf - (s - bp)) + (p - bp);
        float cell = floorf(s);
        float t = (s - cell) + (e + e2);
        if (t < 0.f) { cell -= 1.f; t += 1.f; } else if (t >= 1.f) { cell += 1.f; t -= 1.f; }
        int ix = bi + (int)cell;
        const float fy = g * ginv;
        float v = 0.f;
        if (ix >= 0 && (ix < nK - 1 || (ix == nK - 1 && t == 0.f)) && fy <= (float)(nG - 1)) {
            if (ix == nK - 1) { ix = nK - 2; t = 1.f; }
            const int j = min((int)fy, nG - 2);
            const float ty = fy - (float)j;
            const float* q = P3f + (long long)ix * nG + j;
            const float v00 = __ldg(q), v01 = __ldg(q + 1), v10 = __ldg(q + nG), v11 = __ldg(q + nG + 1);
            const float d10 = v10 - v00, d01 = v01 - v00;
            v = fmaf(t, d10, v00) + ty * fmaf(t, (v11 - v10) - d01, d01);
        }
        acc += (i == 0 || i == n_k_int - 1) ? 0.5f * v : v;
    }
    double total = cd[4] * cd[5] * block_sum((double)acc, sh);
    total += path_tail_f32(P3f, K, G, cd[0], cd[1], cd[2], cd[3], cd[4], gmax, g_def, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = total;
}

void launch_path_integral(const double* P3, const float* P3f, int nkap, int ngam, double kap0, double kap1,
                          double gam1, const double* xi, int nxi, double gmax, double g_def, int n_k_int, double* out,
                          cudaStream_t st) {
    const double hk = (kap1 - kap0) / (nkap - 1), hg = gam1 / (ngam - 1);
    Axis K{kap0, kap1, hk, 1.0 / hk, nkap};
    Axis G{0.0, gam1, hg, 1.0 / hg, ngam};
    if (nxi <= 0) return;
    if (P3f) { k_path_integral_f32<<<nxi, 256, 0, st>>>(P3f, P3, K, G, xi, gmax, g_def, n_k_int, out); SGL_COUNT(1); }
    else { k_path_integral<<<nxi, 256, 0, st>>>(P3, K, G, xi, gmax, g_def, n_k_int, out); SGL_COUNT(1); }
}

}  // namespace sgl
