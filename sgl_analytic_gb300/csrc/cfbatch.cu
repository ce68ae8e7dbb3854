// Batched plain CF solver over many uneven instances in one persistent launch.
//
// An instance is a lens population split into planes (plane p has cells [plane_cells[p],
// plane_cells[p + 1])) with its own uniform k grid k_n = n dk, n < nk.  Its log-CF is
//   gauss: ln Phi(k) = sum_c w_c (e^{i k kap_c} - 1 - i k kap_c) - V k^2 / 2
//   vp:    ln Phi(k) = sum_p Lambda_p(k) + ln E exp( sum_p (lam_p(U_p) - 1) Lambda_p(k) )
//          with Lambda_p the plane's compensated sum and U_p a stationary Markov chain on nstate
//          latent states (weights w, transition K): the one-dimensional form of the positive Cox
//          closure (pos_closure.py:184-240, 453-491; one group per plane).
// Work items are (instance, tile of KT k-points), sorted by cost (longest first).  A persistent grid
// of CTAs takes items from a device counter until none is left; each item stages its instance's
// cells through shared memory (all threads of the CTA work on the same instance) and writes its
// k-points' ln Phi.  Per-term arithmetic is that of the 1-D sweep: FP64 sincos (SGL_FP64), or the
// float-float phase with exact reduction and FP32 polynomial sin / cos, Kahan-compensated FP32
// partial sums folded into FP64 every tile of cells (SGL_MIXED).
//
// Then per instance Phi = exp(ln Phi) times the trapezoid weights, and the inversion to
//   dP/dln mu = (1 - kappa) / 2 * (1/pi) sum_n w_n Re[Phi(k_n) e^{-i k_n kappa}],  kappa = 1 - mu^-1/2
// at the caller's ln mu points: one thread per (instance, ln mu point), the instance's Phi staged
// in shared memory, the phase rotated step by step and re-seeded exactly every 32 steps (FP32
// rotation from a float-float phase in mixed precision, FP64 rotation from an FP64 phase in FP64).
#include "kernels.cuh"

namespace sgl {

constexpr int kCfbTile = 512;                 // cells per shared-memory tile
constexpr int kCfbMaxStates = 8;

struct CfbArgs {
    const CfbInst* inst;
    const int2* items;                        // (instance, tile)
    int n_items;
    int* counter;
    const long long* plane_cells;
    const double* kap; const double* w;       // FP64 cells
    const float* kh; const float* kl; const float* wf;    // mixed cells
    const double* vp_D;                       // [plane][nstate] lam - 1
    const double* vp_K;                       // [slot][nstate][nstate]
    const double* vp_w;                       // [slot][nstate]
    int nstate;
    double2* out;                             // ln Phi per (instance, k)
};

// compensated sum over cells [c0, c1) for one k (thread), cells staged cooperatively
template <int MODE, int KT>
__device__ __forceinline__ double2 cfb_cells(const CfbArgs& a, long long c0, long long c1, double k, ff kf,
                                             float4* s_c, double* s_k, double* s_w) {
    double ar = 0.0, ai = 0.0;
    for (long long base = c0; base < c1; base += kCfbTile) {
        const int cnt = (int)((c1 - base) < kCfbTile ? (c1 - base) : kCfbTile);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += KT) {
            if (MODE == SGL_FP64) { s_k[e] = a.kap[base + e]; s_w[e] = a.w[base + e]; }
            else s_c[e] = make_float4(a.kh[base + e], a.kl[base + e], a.wf[base + e], 0.f);
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
            float far = 0.f, fai = 0.f, car = 0.f, cai = 0.f;
            for (int e = 0; e < cnt; ++e) {
                const float4 cv = s_c[e];
                ff kapf; kapf.hi = cv.x; kapf.lo = cv.y;
                float r, ph_hi, ph_lo;
                int qi;
                halfangle_reduce_ff(kf, kapf, r, qi, ph_hi, ph_lo);
                float sr, cr;
                sincos_reduced(r, sr, cr);
                const bool odd = qi & 1;
                const float av = odd ? cr : sr;
                const float cm1 = -2.f * av * av;
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
            ar += (double)far - (double)car;
            ai += (double)fai - (double)cai;
        }
    }
    return make_double2(ar, ai);
}

template <int MODE, int KT>
__global__ void __launch_bounds__(KT)
k_cfb_persistent(CfbArgs a) {
    __shared__ float4 s_c[MODE == SGL_FP64 ? 1 : kCfbTile];
    __shared__ double s_k[MODE == SGL_FP64 ? kCfbTile : 1];
    __shared__ double s_w[MODE == SGL_FP64 ? kCfbTile : 1];
    __shared__ double s_K[kCfbMaxStates * kCfbMaxStates];
    __shared__ int s_item;
    const int S = a.nstate;
    for (;;) {
        __syncthreads();                          // the previous item's readers of s_item are done
        if (threadIdx.x == 0) s_item = atomicAdd(a.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= a.n_items) break;
        const int2 wi = a.items[it];
        const CfbInst I = a.inst[wi.x];
        const int n = wi.y * KT + threadIdx.x;
        const bool live = n < I.nk;
        const double k = live ? (I.geom ? exp(I.k0 + (double)n * I.dk) : I.k0 + (double)n * I.dk) : 0.0;
        const ff kf = ff_from_double(k);
        double2 lp;
        if (I.closure == 0) {
            const double2 s = cfb_cells<MODE, KT>(a, I.c0, I.c1, k, kf, s_c, s_k, s_w);
            lp = make_double2(s.x - 0.5 * I.V * k * k, s.y);
        } else if (MODE == SGL_FP64) {
            // Poisson sum plus the chain: alpha_t = (sum_s alpha_s K_st) e^{z_t}, z_t = D_pt Lambda_p,
            // rescaled by its largest modulus each plane (the scale kept as a logarithm)
            for (int e = threadIdx.x; e < S * S; e += KT) s_K[e] = a.vp_K[(long long)I.vp_slot * S * S + e];
            __syncthreads();
            double ar[kCfbMaxStates], ai[kCfbMaxStates];
            double lnsc = 0.0, sr = 0.0, si = 0.0;
            for (int p = I.p0; p < I.p1; ++p) {
                const double2 L = cfb_cells<MODE, KT>(a, a.plane_cells[p], a.plane_cells[p + 1], k, kf, s_c, s_k, s_w);
                sr += L.x; si += L.y;
                const double* D = a.vp_D + (long long)p * S;
                double br[kCfbMaxStates], bi[kCfbMaxStates];
#pragma unroll
                for (int t = 0; t < kCfbMaxStates; ++t) {
                    double xr = 0.0, xi = 0.0;
                    if (p == I.p0) {
                        xr = t < S ? a.vp_w[(long long)I.vp_slot * S + t] : 0.0;
                    } else {
#pragma unroll
                        for (int s2 = 0; s2 < kCfbMaxStates; ++s2) {
                            if (s2 < S && t < S) {
                                const double Kv = s_K[s2 * S + t];
                                xr = fma(ar[s2], Kv, xr);
                                xi = fma(ai[s2], Kv, xi);
                            }
                        }
                    }
                    br[t] = xr; bi[t] = xi;
                }
                // e^{z_t} with the largest Re z taken out into the scale (no overflow)
                double zmax = -1e300;
#pragma unroll
                for (int t = 0; t < kCfbMaxStates; ++t) if (t < S) zmax = fmax(zmax, D[t] * L.x);
                lnsc += zmax;
                double mx = 0.0;
#pragma unroll
                for (int t = 0; t < kCfbMaxStates; ++t) {
                    ar[t] = 0.0; ai[t] = 0.0;
                    if (t < S) {
                        const double m = exp(D[t] * L.x - zmax);
                        double sn, cs;
                        sincos(D[t] * L.y, &sn, &cs);
                        const double er = m * cs, ei = m * sn;
                        ar[t] = br[t] * er - bi[t] * ei;
                        ai[t] = br[t] * ei + bi[t] * er;
                        mx = fmax(mx, fabs(ar[t]) + fabs(ai[t]));
                    }
                }
                if (mx > 0.0) {
                    const double inv = 1.0 / mx;
#pragma unroll
                    for (int t = 0; t < kCfbMaxStates; ++t) { ar[t] *= inv; ai[t] *= inv; }
                    lnsc += log(mx);
                }
            }
            double tr = 0.0, ti = 0.0;
#pragma unroll
            for (int t = 0; t < kCfbMaxStates; ++t) { tr += ar[t]; ti += ai[t]; }
            lp = make_double2(sr + lnsc + 0.5 * log(tr * tr + ti * ti), si + atan2(ti, tr));
        } else {
            // the same chain in FP32 registers: z_t = D_pt Lambda_p and its largest real part in FP64, Im z
            // reduced mod 2 pi in FP64, then exp / sincos, the transition and the products in FP32; the
            // state is rescaled by a power of two each plane (exact), the exponents summed in FP64
            float* s_Kf = reinterpret_cast<float*>(s_K);
            for (int e = threadIdx.x; e < S * S; e += KT) s_Kf[e] = (float)a.vp_K[(long long)I.vp_slot * S * S + e];
            __syncthreads();
            float ar[kCfbMaxStates], ai[kCfbMaxStates];
            double lnsc = 0.0, sr = 0.0, si = 0.0;
            for (int p = I.p0; p < I.p1; ++p) {
                const double2 L = cfb_cells<MODE, KT>(a, a.plane_cells[p], a.plane_cells[p + 1], k, kf, s_c, s_k, s_w);
                sr += L.x; si += L.y;
                const double* D = a.vp_D + (long long)p * S;
                float br[kCfbMaxStates], bi[kCfbMaxStates];
#pragma unroll
                for (int t = 0; t < kCfbMaxStates; ++t) {
                    float xr = 0.f, xi = 0.f;
                    if (p == I.p0) {
                        xr = t < S ? (float)a.vp_w[(long long)I.vp_slot * S + t] : 0.f;
                    } else {
#pragma unroll
                        for (int s2 = 0; s2 < kCfbMaxStates; ++s2) {
                            if (s2 < S && t < S) {
                                const float Kv = s_Kf[s2 * S + t];
                                xr = fmaf(ar[s2], Kv, xr);
                                xi = fmaf(ai[s2], Kv, xi);
                            }
                        }
                    }
                    br[t] = xr; bi[t] = xi;
                }
                double zmax = -1e300;
#pragma unroll
                for (int t = 0; t < kCfbMaxStates; ++t) if (t < S) zmax = fmax(zmax, D[t] * L.x);
                lnsc += zmax;
                float mx = 0.f;
#pragma unroll
                for (int t = 0; t < kCfbMaxStates; ++t) {
                    ar[t] = 0.f; ai[t] = 0.f;
                    if (t < S) {
                        const double zi = D[t] * L.y;
                        const double red = zi - 6.283185307179586 * rint(zi * 0.15915494309189535);
                        const float m = expf((float)(D[t] * L.x - zmax));
                        float sn, cs;
                        sincosf((float)red, &sn, &cs);
                        const float er = m * cs, ei = m * sn;
                        ar[t] = br[t] * er - bi[t] * ei;
                        ai[t] = br[t] * ei + bi[t] * er;
                        mx = fmaxf(mx, fabsf(ar[t]) + fabsf(ai[t]));
                    }
                }
                if (mx > 0.f) {
                    int ex;
                    frexpf(mx, &ex);                        // mx = f 2^ex, f in [1/2, 1)
                    const float sc = ldexpf(1.f, -ex);
#pragma unroll
                    for (int t = 0; t < kCfbMaxStates; ++t) { ar[t] *= sc; ai[t] *= sc; }
                    lnsc += ex * 0.6931471805599453;
                }
            }
            float tr = 0.f, ti = 0.f;
#pragma unroll
            for (int t = 0; t < kCfbMaxStates; ++t) { tr += ar[t]; ti += ai[t]; }
            const double trd = tr, tid = ti;
            lp = make_double2(sr + lnsc + 0.5 * log(trd * trd + tid * tid), si + atan2(tid, trd));
        }
        if (live) a.out[I.k_off + n] = lp;
    }
}

// Phi(k_n) w_n / pi (trapezoid weights) per (instance, k), FP64 or FP32 planes
template <typename T>
__global__ void k_cfb_phi(const CfbInst* __restrict__ inst, int n_inst, const double2* __restrict__ lnphi,
                          long long total, const long long* __restrict__ k_offs, T* __restrict__ phi) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    int lo = 0, hi = n_inst - 1;                      // the instance whose k range holds e
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (k_offs[mid] <= e) lo = mid; else hi = mid - 1;
    }
    const CfbInst I = inst[lo];
    const long long n = e - I.k_off;
    const double wgt = (n == 0 || n == I.nk - 1 ? 0.5 : 1.0) * I.dk / M_PI;
    const double2 L = lnphi[e];
    const double m = exp(L.x) * wgt;
    double s, c;
    sincos(L.y, &s, &c);
    phi[2 * e] = (T)(m * c);
    phi[2 * e + 1] = (T)(m * s);
}

constexpr int kCfbPdfThreads = 128;
constexpr int kCfbPdfStage = 1024;
constexpr int kCfbReseed = 32;

// dP/dln mu at lnmu[m] for instance blockIdx.y: thread per ln mu point
template <int MODE>
__global__ void __launch_bounds__(kCfbPdfThreads)
k_cfb_pdf(const CfbInst* __restrict__ inst, const void* __restrict__ phi_v, const double* __restrict__ lnmu, int nm,
          double* __restrict__ P) {
    __shared__ double2 s_pd[MODE == SGL_FP64 ? kCfbPdfStage : 1];
    __shared__ float2 s_pf[MODE == SGL_FP64 ? 1 : kCfbPdfStage];
    const int i = blockIdx.y;
    const CfbInst I = inst[i];
    const int m = blockIdx.x * kCfbPdfThreads + threadIdx.x;
    const bool live = m < nm;
    const double kap = live ? 1.0 - exp(-0.5 * lnmu[m]) : 0.0;
    double acc = 0.0;
    const ff kapf = ff_from_double(kap), dkf = ff_from_double(I.dk);
    for (int base = 0; base < I.nk; base += kCfbPdfStage) {
        const int cnt = min(kCfbPdfStage, I.nk - base);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += kCfbPdfThreads) {
            const long long g = I.k_off + base + e;
            if (MODE == SGL_FP64) {
                const double* p = (const double*)phi_v;
                s_pd[e] = make_double2(p[2 * g], p[2 * g + 1]);
            } else {
                const float* p = (const float*)phi_v;
                s_pf[e] = make_float2(p[2 * g], p[2 * g + 1]);
            }
        }
        __syncthreads();
        if (MODE == SGL_FP64) {
            // exact FP64 phase every kCfbReseed steps, FP64 rotation by the step in between
            double sd, cd;
            sincos(I.dk * kap, &sd, &cd);
            for (int e0 = 0; e0 < cnt; e0 += kCfbReseed) {
                double s, c;
                sincos((double)(base + e0) * I.dk * kap, &s, &c);
                const int e1 = min(cnt, e0 + kCfbReseed);
                for (int e = e0; e < e1; ++e) {
                    acc = fma(s_pd[e].x, c, fma(s_pd[e].y, s, acc));
                    const double c2 = fma(c, cd, -s * sd), s2 = fma(s, cd, c * sd);
                    c = c2;
                    s = s2;
                }
            }
        } else {
            // exact phase (float-float n dk kappa, reduced mod pi/2) every kCfbReseed steps, rotation
            // by the step's exact sin / cos in between; FP32 terms, FP64 sum per block of steps
            float sd, cd;
            {
                float r, ph_hi, ph_lo; int q;
                halfangle_reduce_ff(dkf, kapf, r, q, ph_hi, ph_lo);      // half of dk kappa, reduced
                float sr, cr;
                sincos_reduced(r, sr, cr);
                const bool odd = q & 1;
                const float sh = odd ? cr : sr, ch = odd ? sr : cr;          // |sin|, |cos| of the half angle
                const float sgn_s = (q & 2) ? -1.f : 1.f, sgn_c = ((q + 1) & 2) ? -1.f : 1.f;
                const float shs = sgn_s * sh, chs = sgn_c * ch;
                sd = 2.f * shs * chs;
                cd = (chs - shs) * (chs + shs);
            }
            for (int e0 = 0; e0 < cnt; e0 += kCfbReseed) {
                const int n0 = base + e0;
                float s, c;
                {
                    const ff nk = ff_from_double((double)n0 * I.dk);
                    float r, ph_hi, ph_lo; int q;
                    halfangle_reduce_ff(nk, kapf, r, q, ph_hi, ph_lo);
                    float sr, cr;
                    sincos_reduced(r, sr, cr);
                    const bool odd = q & 1;
                    const float sh = odd ? cr : sr, ch = odd ? sr : cr;
                    const float sgn_s = (q & 2) ? -1.f : 1.f, sgn_c = ((q + 1) & 2) ? -1.f : 1.f;
                    const float shs = sgn_s * sh, chs = sgn_c * ch;
                    s = 2.f * shs * chs;
                    c = (chs - shs) * (chs + shs);
                }
                float fa = 0.f;
                const int e1 = min(cnt, e0 + kCfbReseed);
                for (int e = e0; e < e1; ++e) {
                    fa = fmaf(s_pf[e].x, c, fmaf(s_pf[e].y, s, fa));
                    const float c2 = c * cd - s * sd, s2 = s * cd + c * sd;
                    c = c2; s = s2;
                }
                acc += (double)fa;
            }
        }
    }
    if (live) P[(long long)i * nm + m] = acc * (1.0 - kap) * 0.5;
}

void launch_cfb_persistent(int precision, int kt, int ctas, const CfbInst* inst, const int2* items, int n_items,
                           int* counter, const long long* plane_cells, const double* kap, const double* w,
                           const float* kh, const float* kl, const float* wf, const double* vp_D, const double* vp_K,
                           const double* vp_w, int nstate, double2* out, cudaStream_t st) {
    CfbArgs a{inst, items, n_items, counter, plane_cells, kap, w, kh, kl, wf, vp_D, vp_K, vp_w, nstate, out};
    cudaMemsetAsync(counter, 0, sizeof(int), st);
#define SGL_CFB_LAUNCH(M, T) k_cfb_persistent<M, T><<<ctas, T, 0, st>>>(a)
    if (precision == SGL_FP64) {
        if (kt == 64) SGL_CFB_LAUNCH(SGL_FP64, 64); else if (kt == 256) SGL_CFB_LAUNCH(SGL_FP64, 256); else SGL_CFB_LAUNCH(SGL_FP64, 128);
    } else {
        if (kt == 64) SGL_CFB_LAUNCH(SGL_MIXED, 64); else if (kt == 256) SGL_CFB_LAUNCH(SGL_MIXED, 256); else SGL_CFB_LAUNCH(SGL_MIXED, 128);
    }
#undef SGL_CFB_LAUNCH
    SGL_COUNT(1);
}

void launch_cfb_pdf(int precision, const CfbInst* inst, int n_inst, const double2* lnphi, long long total,
                    const long long* k_offs, void* phi, const double* lnmu, int nm, double* P, cudaStream_t st) {
    if (precision == SGL_FP64) {
        k_cfb_phi<double><<<ceil_div(total, 256), 256, 0, st>>>(inst, n_inst, lnphi, total, k_offs, (double*)phi);
        SGL_COUNT(1);
        k_cfb_pdf<SGL_FP64><<<dim3(ceil_div(nm, kCfbPdfThreads), n_inst), kCfbPdfThreads, 0, st>>>(inst, phi, lnmu, nm, P);
    } else {
        k_cfb_phi<float><<<ceil_div(total, 256), 256, 0, st>>>(inst, n_inst, lnphi, total, k_offs, (float*)phi);
        SGL_COUNT(1);
        k_cfb_pdf<SGL_MIXED><<<dim3(ceil_div(nm, kCfbPdfThreads), n_inst), kCfbPdfThreads, 0, st>>>(inst, phi, lnmu, nm, P);
    }
    SGL_COUNT(1);
}

// Cells of planes with a separable template: cell (m, b) of plane p has kap = u[p][m] F[m][b] and
// w = v[p][m] g[b] (nm x nb cells per plane, plane after plane), in the solver's FP64, float-float
// and FP32 forms
__global__ void k_cfb_fill_separable(long long n_cells, int nm, int nb, const double* __restrict__ F,
                                     const double* __restrict__ g, const double* __restrict__ u,
                                     const double* __restrict__ v, double* __restrict__ kap, double* __restrict__ w,
                                     float* __restrict__ kh, float* __restrict__ kl, float* __restrict__ wf) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cells) return;
    const long long per = (long long)nm * nb;
    const long long p = c / per;
    const int r = (int)(c - p * per);
    const int m = r / nb, b = r - m * nb;
    const double k = u[p * nm + m] * F[r];
    const double ww = v[p * nm + m] * g[b];
    kap[c] = k;
    w[c] = ww;
    const ff f = ff_from_double(k);
    kh[c] = f.hi;
    kl[c] = f.lo;
    wf[c] = (float)ww;
}

void launch_cfb_fill_separable(long long n_cells, int nm, int nb, const double* F, const double* g, const double* u,
                               const double* v, double* kap, double* w, float* kh, float* kl, float* wf, cudaStream_t st) {
    k_cfb_fill_separable<<<(unsigned)ceil_div(n_cells, 256), 256, 0, st>>>(n_cells, nm, nb, F, g, u, v, kap, w, kh, kl, wf);
    SGL_COUNT(1);
}

int cfb_resident_ctas(int precision, int kt) {
    int n = 0;
    cudaError_t e;
    if (precision == SGL_FP64) {
        if (kt == 64) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cfb_persistent<SGL_FP64, 64>, 64, 0);
        else if (kt == 256) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cfb_persistent<SGL_FP64, 256>, 256, 0);
        else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cfb_persistent<SGL_FP64, 128>, 128, 0);
    } else {
        if (kt == 64) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cfb_persistent<SGL_MIXED, 64>, 64, 0);
        else if (kt == 256) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cfb_persistent<SGL_MIXED, 256>, 256, 0);
        else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cfb_persistent<SGL_MIXED, 128>, 128, 0);
    }
    return e == cudaSuccess ? n : 0;
}

}  // namespace sgl
