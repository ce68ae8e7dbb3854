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
                        double2* part, cudaStream_t st) {
    const int npt = nk * nkg;
    if (npt == 0) return;
    const int nch = psi1_direct_chunks(nc) > 0 ? psi1_direct_chunks(nc) : 1;
    dim3 grid(npt, nch);
    { k_psi1_direct<<<grid, 256, 0, st>>>(kk, nk, kg, nkg, k0, g0, w0, nc, part); SGL_COUNT(1); }
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

template <int MODE, typename TT>
__global__ void __launch_bounds__(kSweepRows, MODE == SGL_FP64 ? 4 : 8)
k_sep_sweep(const double* __restrict__ kk, int nk, SepDevice sd, TT* __restrict__ Tt,
            double2* __restrict__ A_part) {
    // FP64 path stages (kappa, w, wl) as doubles; the mixed path stages float-float kappa and
    // float weights (prepared once per plan), so its inner loop issues no FP64 instruction.
    __shared__ TT s_wl[kSweepStage][8];
    __shared__ TT s_w[kSweepStage];
    __shared__ TT s_k0[kSweepStage];
    __shared__ float s_k1[kSweepStage];
    __shared__ int s_grp[kSweepStage];
    const int n = blockIdx.x * kSweepRows + threadIdx.x;
    const bool live = n < nk;
    const double k = live ? kk[n] : 0.0;
    const ff kf = ff_from_double(k);
    const int c_begin = sd.chunk_begin[blockIdx.y], c_end = sd.chunk_begin[blockIdx.y + 1];
    const long long ld = 2LL * nk;

    double ar = 0.0, ai = 0.0;                       // FP64 path
    float far = 0.f, fai = 0.f, car = 0.f, cai = 0.f;  // mixed path: Kahan-compensated FP32
    TT tr[8], ti[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) { tr[j] = TT(0); ti[j] = TT(0); }
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
        for (int j = 0; j < 8; ++j) { tr[j] = TT(0); ti[j] = TT(0); }
    };

    for (int base = c_begin; base < c_end; base += kSweepStage) {
        const int cnt = min(kSweepStage, c_end - base);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += kSweepRows) {
            if (MODE == SGL_FP64) { s_k0[e] = (TT)sd.kap[base + e]; s_w[e] = (TT)sd.w[base + e]; }
            else { s_k0[e] = (TT)sd.kap_hi[base + e]; s_k1[e] = sd.kap_lo[base + e]; s_w[e] = (TT)sd.w_f[base + e]; }
            s_grp[e] = sd.grp[base + e];
        }
        for (int e = threadIdx.x; e < cnt * 8; e += kSweepRows) {
            if (MODE == SGL_FP64) s_wl[e >> 3][e & 7] = (TT)sd.wl[(long long)base * 8 + e];
            else s_wl[e >> 3][e & 7] = (TT)sd.wl_f[(long long)base * 8 + e];
        }
        __syncthreads();
        for (int e = 0; e < cnt; ++e) {
            const int g = s_grp[e];
            if (g != cur) { flush(cur); cur = g; }
            if (MODE == SGL_FP64) {
                const double w = (double)s_w[e];
                const double ph = k * (double)s_k0[e];
                double cm1, smp, sn;
                compensated_fp64(ph, cm1, smp, sn);
                ar = fma(w, cm1, ar);
                ai = fma(w, smp, ai);
                const double cr = cm1 + 1.0;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const double wj = (double)s_wl[e][j];
                    tr[j] = (TT)fma(wj, cr, (double)tr[j]);
                    ti[j] = (TT)fma(wj, sn, (double)ti[j]);
                }
            } else {
                ff kapf; kapf.hi = (float)s_k0[e]; kapf.lo = s_k1[e];
                float s, c, ph_hi, ph_lo;
                halfangle_sincos_ff(kf, kapf, s, c, ph_hi, ph_lo);
                const float cm1 = -2.f * s * s;
                const float sn = 2.f * s * c;
                const float ph = ph_hi + ph_lo;
                float smp;
                if (fabsf(ph) < 1e-2f) {
                    const float p2 = ph * ph;
                    smp = -ph * p2 * (1.f / 6.f) * (1.f - p2 * (1.f / 20.f) * (1.f - p2 * (1.f / 42.f)));
                } else {
                    smp = (sn - ph_hi) - ph_lo;
                }
                const float wf = (float)s_w[e];
                float y = fmaf(wf, cm1, -car); float t = far + y; car = (t - far) - y; far = t;
                y = fmaf(wf, smp, -cai); t = fai + y; cai = (t - fai) - y; fai = t;
                const float cr = cm1 + 1.f;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const float wj = (float)s_wl[e][j];
                    tr[j] = (TT)fmaf(wj, cr, (float)tr[j]);
                    ti[j] = (TT)fmaf(wj, sn, (float)ti[j]);
                }
            }
        }
    }
    flush(cur);
    if (live) {
        if (MODE == SGL_FP64) A_part[(long long)blockIdx.y * nk + n] = make_double2(ar, ai);
        else A_part[(long long)blockIdx.y * nk + n] = make_double2((double)far - (double)car, (double)fai - (double)cai);
    }
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
        { k_sep_sweep<SGL_FP64, double><<<grid, kSweepRows, 0, st>>>(kk, nk, s, (double*)Tt, A_part); SGL_COUNT(1); }
    else
        { k_sep_sweep<SGL_MIXED, float><<<grid, kSweepRows, 0, st>>>(kk, nk, s, (float*)Tt, A_part); SGL_COUNT(1); }
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

void launch_j0m1_table(int precision, const double* nodes, int nn, const double* x, int nx, void* B, cudaStream_t st) {
    const long long tot = (long long)nn * nx;
    if (tot == 0) return;
    if (precision == SGL_FP64) { k_j0m1_table<double><<<ceil_div(tot, 256), 256, 0, st>>>(nodes, nn, x, nx, (double*)B); SGL_COUNT(1); }
    else { k_j0m1_table<float><<<ceil_div(tot, 256), 256, 0, st>>>(nodes, nn, x, nx, (float*)B); SGL_COUNT(1); }
}

// Barycentric Chebyshev-Lobatto interpolation matrix L (nx x N): points t_j = K/2 (1 - cos(j pi/(N-1))),
// weights (-1)^j halved at both ends; a point within 1e-14 K of a node gets the exact unit row.
// One CTA per row.
template <typename TT>
__global__ void __launch_bounds__(256)
k_cheb_matrix(double K, int N, const double* __restrict__ x, int nx, TT* __restrict__ L) {
    __shared__ double sh[32];
    __shared__ int s_hit;
    const int m = blockIdx.x;
    const double xm = x[m];
    if (threadIdx.x == 0) s_hit = -1;
    __syncthreads();
    double part = 0.0;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double t = 0.5 * K * (1.0 - cos(j * M_PI / (N - 1)));
        const double d = xm - t;
        if (fabs(d) <= 1e-14 * K) atomicMax(&s_hit, j);
        double wb = (j & 1) ? -1.0 : 1.0;
        if (j == 0 || j == N - 1) wb *= 0.5;
        part += wb / (fabs(d) <= 1e-14 * K ? 1.0 : d);
    }
    const double tot = block_sum(part, sh);
    const int hit = s_hit;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        double v;
        if (hit >= 0) v = (j == hit) ? 1.0 : 0.0;
        else {
            const double t = 0.5 * K * (1.0 - cos(j * M_PI / (N - 1)));
            double wb = (j & 1) ? -1.0 : 1.0;
            if (j == 0 || j == N - 1) wb *= 0.5;
            v = (wb / (xm - t)) / tot;
        }
        L[(long long)m * N + j] = (TT)v;
    }
}

void launch_cheb_matrix(int precision, double K, int N, const double* x, int nx, void* L, cudaStream_t st) {
    if (precision == SGL_FP64) { k_cheb_matrix<double><<<nx, 256, 0, st>>>(K, N, x, nx, (double*)L); SGL_COUNT(1); }
    else { k_cheb_matrix<float><<<nx, 256, 0, st>>>(K, N, x, nx, (float*)L); SGL_COUNT(1); }
}

__global__ void k_cheb_points(double K, int N, double* __restrict__ t) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < N) t[j] = 0.5 * K * (1.0 - cos(j * M_PI / (N - 1)));
}

void launch_cheb_points(double K, int N, double* t, cudaStream_t st) {
    { k_cheb_points<<<ceil_div(N, 256), 256, 0, st>>>(K, N, t); SGL_COUNT(1); }
}

}  // namespace sgl
