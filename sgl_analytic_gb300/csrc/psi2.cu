// xi_lin (Gauss-Poisson pair) term Psi_2 of ln Phi (reference: Lam._Qxi_gauss,
// sgl_full.py:2869-2951):
//   Psi_2 = sum_groups sign_m / 2 sum_r G_r^2,
//   G_r(k, q) = sum_p e^{i k kap_p} sum_q' H[r, p, q'] J_m(q gam_q')  (+ residual terms)
// evaluated group by group as
//   stage A   T_g[p, r, j]  = sum_{entries (p, q')} rows[r, e] J_m(gam_q' kg_j)   (sparse rows)
//   stage B   G_g[i, r, j]  = sum_p E[i, p] T_g[p, r, j],  E = [cos; sin](kk kap_p)  (grouped GEMM)
//   stage C   Psi_2(n, j)   = sum_g sign/2 sum_r (Gr + i Gi)^2 with the residual terms  (reduce)
// plus the two 1-D fast paths used by the k-reach probes (k_gamma = 0, k_kappa = 0).
#include "kernels.cuh"

namespace sgl {

// J2 from its power series below x = 2 (14 terms: (x/2)^{2k} / (k! (k+2)!) < 1e-18 there) and
// from the recurrence J2 = 2 J1 / x - J0 above (stable for x >= n).
__device__ inline double bessel_j2(double x) {
    if (x < 2.0) {
        const double h = 0.5 * x, h2 = h * h;
        double term = 0.5;          // 1 / 2!
        double sum = term;
        for (int k = 1; k < 14; ++k) { term *= -h2 / (double(k) * double(k + 2)); sum += term; }
        return sum * h2;
    }
    return 2.0 * j1(x) / x - j0(x);
}

__device__ inline double bessel_jm(int m, double x) {
    return m == 0 ? j0(x) : (m == 1 ? j1(x) : bessel_j2(x));
}

// J[m][q][j] = J_m(gmc[q] * kg[j]), m = 0, 1, 2
template <typename TT>
__global__ void k_bessel_tables(const double* __restrict__ gmc, int n_gmc, const double* __restrict__ kg, int nkg,
                                TT* __restrict__ J) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n_gmc * nkg;
    if (e >= 3 * per) return;
    const int m = (int)(e / per);
    const long long r = e % per;
    const int q = (int)(r / nkg), j = (int)(r % nkg);
    J[e] = (TT)bessel_jm(m, gmc[q] * kg[j]);
}

void launch_bessel_tables(int precision, const double* gmc, int n_gmc, const double* kg, int nkg, void* J, cudaStream_t st) {
    const long long tot = 3LL * n_gmc * nkg;
    if (precision == SGL_FP64) { k_bessel_tables<double><<<ceil_div(tot, 256), 256, 0, st>>>(gmc, n_gmc, kg, nkg, (double*)J); SGL_COUNT(1); }
    else { k_bessel_tables<float><<<ceil_div(tot, 256), 256, 0, st>>>(gmc, n_gmc, kg, nkg, (float*)J); SGL_COUNT(1); }
}

__device__ inline int find_group(const long long* prefix, int ng, long long v) {
    int lo = 0, hi = ng - 1;      // largest g with prefix[g] <= v
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// stage A: one CTA per (group, local p); threads over (r, j)
template <typename TT>
__global__ void __launch_bounds__(256)
k_xi_stageA(XiDevice x, const long long* __restrict__ p_prefix, const long long* __restrict__ T_off,
            const long long* __restrict__ rowel_off, const TT* __restrict__ J, int nkg, TT* __restrict__ T) {
    const long long P = blockIdx.x;
    const int g = find_group(p_prefix, x.n_groups, P);
    const int p = (int)(P - p_prefix[g]);
    const int r = x.g_r[g], m = x.g_m[g];
    const int e0 = x.p_ptr[P], e1 = x.p_ptr[P + 1];
    const long long ent0 = x.g_ent_off[g];
    const TT* Jm = J + (long long)m * x.n_gmc * nkg;
    TT* Tg = T + T_off[g] + (long long)p * r * nkg;
    const double* rows = x.rows + rowel_off[g];
    for (int t = threadIdx.x; t < r * nkg; t += blockDim.x) {
        const int rr = t / nkg, j = t % nkg;
        double acc = 0.0;
        for (int e = e0; e < e1; ++e) {
            const long long el = e - ent0;
            acc = fma(rows[el * r + rr], (double)Jm[(long long)x.ent_qg[e] * nkg + j], acc);
        }
        Tg[t] = (TT)acc;
    }
}

void launch_xi_stageA(int precision, const XiDevice& x, const long long* d_p_prefix, int total_p, const long long* T_off,
                      const void* J, int nkg, void* T, cudaStream_t st) {
    // rowel_off is stored right after p_prefix in the same device block (see capi)
    const long long* rowel_off = d_p_prefix + (x.n_groups + 1);
    if (precision == SGL_FP64)
        { k_xi_stageA<double><<<total_p, 256, 0, st>>>(x, d_p_prefix, T_off, rowel_off, (const double*)J, nkg, (double*)T); SGL_COUNT(1); }
    else
        { k_xi_stageA<float><<<total_p, 256, 0, st>>>(x, d_p_prefix, T_off, rowel_off, (const float*)J, nkg, (float*)T); SGL_COUNT(1); }
}

// E_g[i, p] = cos(kk_i kap_p) (i < nk) / sin(kk_{i-nk} kap_p): one CTA per global p
template <typename TT>
__global__ void k_xi_E(XiDevice x, const double* __restrict__ kk, int nk, const long long* __restrict__ E_off,
                       const long long* __restrict__ p_prefix, TT* __restrict__ E) {
    const long long P = blockIdx.x;
    const int g = find_group(p_prefix, x.n_groups, P);
    const int p = (int)(P - p_prefix[g]);
    const int nP = x.g_nP[g];
    const double kap = x.kmc[x.idx_p[P]];
    TT* Eg = E + E_off[g];
    for (int i = threadIdx.x; i < nk; i += blockDim.x) {
        double s, c;
        sincos(kk[i] * kap, &s, &c);
        Eg[(long long)i * nP + p] = (TT)c;
        Eg[(long long)(nk + i) * nP + p] = (TT)s;
    }
}

void launch_xi_E(int precision, const XiDevice& x, const double* kk, int nk, const long long* E_off,
                 const long long* d_p_prefix, int total_p, void* E, cudaStream_t st) {
    if (precision == SGL_FP64) { k_xi_E<double><<<total_p, 128, 0, st>>>(x, kk, nk, E_off, d_p_prefix, (double*)E); SGL_COUNT(1); }
    else { k_xi_E<float><<<total_p, 128, 0, st>>>(x, kk, nk, E_off, d_p_prefix, (float*)E); SGL_COUNT(1); }
}

// stage C: one thread per output (n, j); groups and rows in a fixed order (deterministic)
template <typename TT>
__global__ void k_xi_square(XiDevice x, const long long* __restrict__ G_off, const TT* __restrict__ G,
                            const double* __restrict__ kk, int nk, const double* __restrict__ kg, int nkg,
                            double* __restrict__ out_re, double* __restrict__ out_im) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nk * nkg) return;
    const int n = (int)(e / nkg), j = (int)(e % nkg);
    const double k = kk[n], q = kg[j];
    double re = 0.0, im = 0.0;
    for (int g = 0; g < x.n_groups; ++g) {
        const int r = x.g_r[g], m = x.g_m[g];
        const double sign = (m == 0) ? 1.0 : ((m & 1) ? -2.0 : 2.0);
        const TT* Gg = G + G_off[g];
        const long long ldg = (long long)r * nkg;
        const double* res = x.res + x.g_row_off[g];
        const double* srow = x.sum_rows + x.g_row_off[g];
        double gre = 0.0, gim = 0.0;
        for (int rr = 0; rr < r; ++rr) {
            double a = (double)Gg[(long long)n * ldg + (long long)rr * nkg + j];
            double b = (double)Gg[(long long)(nk + n) * ldg + (long long)rr * nkg + j];
            if (m == 0) { a -= srow[rr]; b = fma(k, res[rr], b); }
            else if (m == 1) { a = fma(0.5 * q, res[rr], a); }
            gre += a * a - b * b;
            gim += a * b;
        }
        re = fma(0.5 * sign, gre, re);
        im = fma(0.5 * sign, 2.0 * gim, im);
    }
    out_re[e] = re;
    out_im[e] = im;
}

void launch_xi_square(int precision, const XiDevice& x, const long long* G_off, const void* G, const double* kk, int nk,
                      const double* kg, int nkg, double* out_re, double* out_im, cudaStream_t st) {
    const long long tot = (long long)nk * nkg;
    if (precision == SGL_FP64)
        { k_xi_square<double><<<ceil_div(tot, 128), 128, 0, st>>>(x, G_off, (const double*)G, kk, nk, kg, nkg, out_re, out_im); SGL_COUNT(1); }
    else
        { k_xi_square<float><<<ceil_div(tot, 128), 128, 0, st>>>(x, G_off, (const float*)G, kk, nk, kg, nkg, out_re, out_im); SGL_COUNT(1); }
}

// ---- 1-D path along k_kappa (k_gamma = 0): G_R = sum_p e^{i k kap_p} W0[R, p] - sum0_R + i k res0_R
__global__ void __launch_bounds__(256)
k_xi_line_k(XiDevice x, const double* __restrict__ kk, double* __restrict__ out_re, double* __restrict__ out_im) {
    extern __shared__ double sm[];
    double* ec = sm;
    double* es = sm + x.n_kmc;
    double* red = sm + 2 * x.n_kmc;
    const int n = blockIdx.x;
    const double k = kk[n];
    for (int p = threadIdx.x; p < x.n_kmc; p += blockDim.x) sincos(k * x.kmc[p], &es[p], &ec[p]);
    __syncthreads();
    double re = 0.0, im = 0.0;
    for (int R = threadIdx.x; R < x.R0; R += blockDim.x) {
        const double* w = x.W0 + (long long)R * x.n_kmc;
        double a = 0.0, b = 0.0;
        for (int p = 0; p < x.n_kmc; ++p) { a = fma(ec[p], w[p], a); b = fma(es[p], w[p], b); }
        a -= x.sum0[R];
        b = fma(k, x.res0[R], b);
        re += a * a - b * b;
        im += 2.0 * a * b;
    }
    re = block_sum(re, red);
    im = block_sum(im, red);
    if (threadIdx.x == 0) { out_re[n] = 0.5 * re; out_im[n] = 0.5 * im; }
}

void launch_xi_line_k(const XiDevice& x, const double* kk, int nk, double* out_re, double* out_im, cudaStream_t st) {
    const size_t sm = (2 * (size_t)x.n_kmc + 32) * sizeof(double);
    { k_xi_line_k<<<nk, 256, sm, st>>>(x, kk, out_re, out_im); SGL_COUNT(1); }
}

// ---- 1-D path along k_gamma (k_kappa = 0): per m, G_R = sum_q U_m[R, q] J_m(gam_q kg) (+ residuals)
__global__ void __launch_bounds__(256)
k_xi_line_g(XiDevice x, const double* __restrict__ kg, double* __restrict__ out_re, double* __restrict__ out_im) {
    extern __shared__ double sm[];
    double* Jq = sm;                 // [n_gmc]
    double* red = sm + x.n_gmc;
    const int j = blockIdx.x;
    const double q = kg[j];
    double tot = 0.0;
    for (int m = 0; m < 3; ++m) {
        if (x.Rm[m] == 0) continue;
        __syncthreads();
        for (int c = threadIdx.x; c < x.n_gmc; c += blockDim.x) Jq[c] = bessel_jm(m, x.gmc[c] * q);
        __syncthreads();
        double acc = 0.0;
        for (int R = threadIdx.x; R < x.Rm[m]; R += blockDim.x) {
            const double* u = x.U[m] + (long long)R * x.n_gmc;
            double a = 0.0;
            for (int c = 0; c < x.n_gmc; ++c) a = fma(u[c], Jq[c], a);
            if (m == 0) a -= x.summ[m][R];
            else if (m == 1) a = fma(0.5 * q, x.resm[m][R], a);
            acc += a * a;
        }
        acc = block_sum(acc, red);
        const double sign = (m == 0) ? 1.0 : ((m & 1) ? -2.0 : 2.0);
        tot += 0.5 * sign * acc;
    }
    if (threadIdx.x == 0) { out_re[j] = tot; out_im[j] = 0.0; }
}

void launch_xi_line_g(const XiDevice& x, const double* kg, int nkg, double* out_re, double* out_im, cudaStream_t st) {
    const size_t sm = ((size_t)x.n_gmc + 32) * sizeof(double);
    { k_xi_line_g<<<nkg, 256, sm, st>>>(x, kg, out_re, out_im); SGL_COUNT(1); }
}

}  // namespace sgl
