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

// J[m][q][j] = J_m(gmc[q] * kg[j]) for m = 0, 1, 2 and, as table 3, J0 - 1 without cancellation
template <typename TT>
__global__ void k_bessel_tables(const double* __restrict__ gmc, int n_gmc, const double* __restrict__ kg, int nkg,
                                TT* __restrict__ J) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n_gmc * nkg;
    if (e >= 4 * per) return;
    const int m = (int)(e / per);
    const long long r = e % per;
    const int q = (int)(r / nkg), j = (int)(r % nkg);
    const double x = gmc[q] * kg[j];
    J[e] = (TT)(m < 3 ? bessel_jm(m, x) : j0m1_d(x));
}

void launch_bessel_tables(int precision, const double* gmc, int n_gmc, const double* kg, int nkg, void* J, cudaStream_t st) {
    const long long tot = 4LL * n_gmc * nkg;
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

// stage A: one CTA per (group, local p); threads over (r, j).  The p-row's entries (their rows
// and J_m rows) are staged in shared memory; accumulation in TT (FP64 path: double).
constexpr int kStageAEnt = 32;
template <typename TT>
__global__ void __launch_bounds__(256)
k_xi_stageA(XiDevice x, const long long* __restrict__ p_prefix, const long long* __restrict__ T_off,
            const long long* __restrict__ rowel_off, const TT* __restrict__ J, int nkg, TT* __restrict__ T) {
    extern __shared__ unsigned char smraw[];
    TT* s_rows = (TT*)smraw;                                  // [kStageAEnt][r]
    const long long P = blockIdx.x;
    const int g = find_group(p_prefix, x.n_groups, P);
    const int p = (int)(P - p_prefix[g]);
    const int r = x.g_r[g], m = x.g_m[g];
    TT* s_J = s_rows + kStageAEnt * r;                        // [kStageAEnt][nkg]
    const int e0 = x.p_ptr[P], e1 = x.p_ptr[P + 1];
    const long long ent0 = x.g_ent_off[g];
    const TT* Jm = J + (long long)m * x.n_gmc * nkg;
    TT* Tg = T + T_off[g] + (long long)p * r * nkg;
    const double* rows = x.rows + rowel_off[g];
    const float* rows_f = x.rows_f ? x.rows_f + rowel_off[g] : nullptr;
    constexpr int kMaxOut = 24;                               // outputs per thread (r * nkg <= 256 * 24)
    TT acc[kMaxOut];
#pragma unroll
    for (int i = 0; i < kMaxOut; ++i) acc[i] = TT(0);
    const int nout = r * nkg;
    for (int eb = e0; eb < e1; eb += kStageAEnt) {
        const int cnt = min(kStageAEnt, e1 - eb);
        __syncthreads();
        for (int t = threadIdx.x; t < cnt * r; t += blockDim.x) {
            const int e = t / r, rr = t % r;
            const long long el = (long long)(eb + e) - ent0;
            s_rows[e * r + rr] = (sizeof(TT) == 4 && rows_f) ? (TT)rows_f[el * r + rr] : (TT)rows[el * r + rr];
        }
        for (int t = threadIdx.x; t < cnt * nkg; t += blockDim.x) {
            const int e = t / nkg, j = t % nkg;
            s_J[e * nkg + j] = Jm[(long long)x.ent_qg[eb + e] * nkg + j];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < kMaxOut; ++i) {
            const int t = threadIdx.x + i * blockDim.x;
            if (t < nout) {
                const int rr = t / nkg, j = t % nkg;
                TT a = acc[i];
                for (int e = 0; e < cnt; ++e) a = fma(s_rows[e * r + rr], s_J[e * nkg + j], a);
                acc[i] = a;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < kMaxOut; ++i) {
        const int t = threadIdx.x + i * blockDim.x;
        if (t < nout) Tg[t] = acc[i];
    }
}

// Generic stage A (any grid width): no staging, FP64 accumulation.
template <typename TT>
__global__ void __launch_bounds__(256)
k_xi_stageA_generic(XiDevice x, const long long* __restrict__ p_prefix, const long long* __restrict__ T_off,
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
    for (long long t = threadIdx.x; t < (long long)r * nkg; t += blockDim.x) {
        const int rr = (int)(t / nkg), j = (int)(t % nkg);
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
    const int rmax = x.r_max;
    if (nkg > 128 || (long long)rmax * nkg > 256LL * 24) {
        if (precision == SGL_FP64) { k_xi_stageA_generic<double><<<total_p, 256, 0, st>>>(x, d_p_prefix, T_off, rowel_off, (const double*)J, nkg, (double*)T); SGL_COUNT(1); }
        else { k_xi_stageA_generic<float><<<total_p, 256, 0, st>>>(x, d_p_prefix, T_off, rowel_off, (const float*)J, nkg, (float*)T); SGL_COUNT(1); }
        return;
    }
    if (precision == SGL_FP64) {
        const size_t sm = (size_t)kStageAEnt * (rmax + nkg) * sizeof(double);
        k_xi_stageA<double><<<total_p, 256, sm, st>>>(x, d_p_prefix, T_off, rowel_off, (const double*)J, nkg, (double*)T);
        SGL_COUNT(1);
    } else {
        const size_t sm = (size_t)kStageAEnt * (rmax + nkg) * sizeof(float);
        k_xi_stageA<float><<<total_p, 256, sm, st>>>(x, d_p_prefix, T_off, rowel_off, (const float*)J, nkg, (float*)T);
        SGL_COUNT(1);
    }
}

// Mixed-path stage A written straight into the xi GEMM's packed A operand
//   A'(i', p) = T_g[p, i'],  i' = rr * nkg + j,  packed [kb][part][Mpad][16], 2 TF32 parts,
// so the GEMM's bulk copies read it as is (no FP32 T in HBM, no separate pack pass).
// One CTA per (group, 4 consecutive p): for each p, its entries (rows and J_m rows) stream through
// shared memory in chunks of 32 and each thread accumulates 4 rr x 4 j tiles (FP32, float4 operand
// reads); the 4 p results are staged in shared memory and written as (hi, lo) float4 rows of the
// core matrices, with zeros in the padded rows and columns.
constexpr int kSAEnt = 32, kSAThreads = 256, kSAMaxTasks = 2;

bool xi_stageA_pack_fits(int r_max, int nkg) {
    const int tasks = ((r_max + 3) / 4) * ((nkg + 3) / 4);
    const size_t sm = (4ULL * r_max * nkg + (size_t)kSAEnt * (((r_max + 3) & ~3) + ((nkg + 3) & ~3))) * 4;
    return tasks <= kSAThreads * kSAMaxTasks && sm <= 200 * 1024;
}

__device__ __forceinline__ float tf32_rna_sa(float v) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
    return __uint_as_float(r);
}

__global__ void __launch_bounds__(kSAThreads)
k_xi_stageA_pack(XiDevice x, const long long* __restrict__ p_prefix, const long long* __restrict__ rowel_off,
                 const float* __restrict__ J, int nkg, const long long* __restrict__ chunk_prefix,
                 const TcGemmDesc* __restrict__ descs, float* __restrict__ packed) {
    extern __shared__ __align__(16) float sa_sm[];
    const int rmax = x.r_max;
    const int rpm = (rmax + 3) & ~3, nkp = (nkg + 3) & ~3;
    float* s_out = sa_sm;                                   // [4][r * nkg]
    float* s_rows = s_out + 4LL * rmax * nkg;               // [kSAEnt][rp]
    float* s_J = s_rows + kSAEnt * rpm;                     // [kSAEnt][nkp]
    const long long cidx = blockIdx.x;
    const int g = find_group(chunk_prefix, x.n_groups, cidx);
    const int c4 = (int)(cidx - chunk_prefix[g]);
    const TcGemmDesc d = descs[g];
    const int r = x.g_r[g], m = x.g_m[g], nP = x.g_nP[g];
    const int rp = (r + 3) & ~3;
    const int M = r * nkg;
    const int nrb = rp / 4, njb = nkp / 4, ntask = nrb * njb;
    const long long gp0 = p_prefix[g], ent0 = x.g_ent_off[g];
    const float* rowsg = x.rows_f + rowel_off[g];
    const float* Jm = J + (long long)m * x.n_gmc * nkg;
    const int tid = threadIdx.x;
    for (int pp = 0; pp < 4; ++pp) {
        const int p = 4 * c4 + pp;
        float* so = s_out + (long long)pp * M;
        if (p >= nP) {
            for (int i = tid; i < M; i += kSAThreads) so[i] = 0.f;
            continue;
        }
        const long long P = gp0 + p;
        const int e0 = x.p_ptr[P], e1 = x.p_ptr[P + 1];
        float acc[kSAMaxTasks][16];
#pragma unroll
        for (int a = 0; a < kSAMaxTasks; ++a)
#pragma unroll
            for (int b = 0; b < 16; ++b) acc[a][b] = 0.f;
        for (int eb = e0; eb < e1; eb += kSAEnt) {
            const int cnt = min(kSAEnt, e1 - eb);
            __syncthreads();
            for (int t = tid; t < kSAEnt * rp; t += kSAThreads) {
                const int e = t / rp, rr = t % rp;
                s_rows[e * rp + rr] = (e < cnt && rr < r) ? rowsg[((long long)(eb + e) - ent0) * r + rr] : 0.f;
            }
            for (int t = tid; t < kSAEnt * nkp; t += kSAThreads) {
                const int e = t / nkp, j = t % nkp;
                s_J[e * nkp + j] = (e < cnt && j < nkg) ? Jm[(long long)x.ent_qg[eb + e] * nkg + j] : 0.f;
            }
            __syncthreads();
#pragma unroll
            for (int a = 0; a < kSAMaxTasks; ++a) {
                const int task = tid + a * kSAThreads;
                if (task < ntask) {
                    const int rb = task / njb, jb = task % njb;
                    for (int e = 0; e < cnt; ++e) {
                        const float4 ra = *(const float4*)(s_rows + e * rp + 4 * rb);
                        const float4 jv = *(const float4*)(s_J + e * nkp + 4 * jb);
                        const float av[4] = {ra.x, ra.y, ra.z, ra.w}, bv[4] = {jv.x, jv.y, jv.z, jv.w};
#pragma unroll
                        for (int u = 0; u < 4; ++u)
#pragma unroll
                            for (int w = 0; w < 4; ++w) acc[a][u * 4 + w] = fmaf(av[u], bv[w], acc[a][u * 4 + w]);
                    }
                }
            }
        }
#pragma unroll
        for (int a = 0; a < kSAMaxTasks; ++a) {
            const int task = tid + a * kSAThreads;
            if (task < ntask) {
                const int rb = task / njb, jb = task % njb;
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int w = 0; w < 4; ++w) {
                        const int rr = 4 * rb + u, j = 4 * jb + w;
                        if (rr < r && j < nkg) so[rr * nkg + j] = acc[a][u * 4 + w];
                    }
            }
        }
    }
    __syncthreads();
    // packed rows: chunk c of K block kb holds p = 16 kb + 4 c .. + 3
    const int kb = c4 / 4, c = c4 % 4;
    float* Ap = packed + d.a_off;
    const long long pstride = (long long)d.Mpad * 16;
    for (int i = tid; i < d.Mpad; i += kSAThreads) {
        float hv[4], lv[4];
#pragma unroll
        for (int pp = 0; pp < 4; ++pp) {
            const float v = i < M ? s_out[(long long)pp * M + i] : 0.f;
            hv[pp] = tf32_rna_sa(v);
            lv[pp] = tf32_rna_sa(v - hv[pp]);
        }
        const long long o = (long long)(i >> 3) * 128 + c * 32 + (i & 7) * 4;
        *(float4*)(Ap + (2LL * kb) * pstride + o) = make_float4(hv[0], hv[1], hv[2], hv[3]);
        *(float4*)(Ap + (2LL * kb + 1) * pstride + o) = make_float4(lv[0], lv[1], lv[2], lv[3]);
    }
}

// Register-tiled form for groups with at most 256 (4 rr x 4 j) tiles: each thread owns one tile
// for all 4 p of the CTA (64 FP32 accumulators), so the packed (hi, lo) float4 rows are written
// straight from registers.  All entries of the 4 p stream through shared memory together, copied
// with cp.async (warp per entry, no index division) so that a batch costs one memory round trip
// after its gamma-cell indices are known; the usual <= 96 entries are one batch.  Per-p summation
// order is that of the form above: the results are identical.
constexpr int kSA2Ent = 96;

// 4-byte asynchronous global -> shared copy (no register staging, many in flight per thread)
__device__ __forceinline__ void cp_async4(float* sdst, const float* gsrc) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" :: "r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all4() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__global__ void __launch_bounds__(kSAThreads, 3)
k_xi_stageA_pack_reg(XiDevice x, const long long* __restrict__ p_prefix, const long long* __restrict__ rowel_off,
                     const float* __restrict__ J, int nkg, const long long* __restrict__ chunk_prefix,
                     const TcGemmDesc* __restrict__ descs, float* __restrict__ packed) {
    extern __shared__ __align__(16) float sa2_sm[];
    __shared__ int s_q[kSA2Ent];
    const int rpm = (x.r_max + 3) & ~3, nkp = (nkg + 3) & ~3;
    float* s_rows = sa2_sm;                                 // [kSA2Ent][rpm]
    float* s_J = sa2_sm + kSA2Ent * rpm;                    // [kSA2Ent][nkp]
    const long long cidx = blockIdx.x;
    const int g = find_group(chunk_prefix, x.n_groups, cidx);
    const int c4 = (int)(cidx - chunk_prefix[g]);
    const TcGemmDesc d = descs[g];
    const int r = x.g_r[g], m = x.g_m[g], nP = x.g_nP[g];
    const int rp = (r + 3) & ~3;
    const int M = r * nkg;
    const int njb = nkp / 4, ntask = (rp / 4) * njb;
    const long long gp0 = p_prefix[g], ent0 = x.g_ent_off[g];
    const float* rowsg = x.rows_f + rowel_off[g];
    const float* Jm = J + (long long)m * x.n_gmc * nkg;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool has_task = tid < ntask;
    const int rb = has_task ? tid / njb : 0, jb = has_task ? tid % njb : 0;
    int pb[5];                                              // entry bounds of the 4 p (p >= nP: empty)
#pragma unroll
    for (int pp = 0; pp < 5; ++pp) pb[pp] = x.p_ptr[gp0 + min(4 * c4 + pp, nP)];
    float acc[4][16];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 16; ++b) acc[a][b] = 0.f;
    for (int eb = pb[0]; eb < pb[4]; eb += kSA2Ent) {
        const int cnt = min(kSA2Ent, pb[4] - eb);
        __syncthreads();
        for (int e = tid; e < cnt; e += kSAThreads) s_q[e] = x.ent_qg[eb + e];
        __syncthreads();
        // one round trip for the whole batch: every copy is issued before any is waited on
        for (int e = warp; e < cnt; e += kSAThreads / 32) {
            const float* src = rowsg + ((long long)(eb + e) - ent0) * r;
            for (int rr = lane; rr < rp; rr += 32) {
                if (rr < r) cp_async4(s_rows + e * rpm + rr, src + rr);
                else s_rows[e * rpm + rr] = 0.f;
            }
            const float* js = Jm + (long long)s_q[e] * nkg;
            for (int j = lane; j < nkp; j += 32) {
                if (j < nkg) cp_async4(s_J + e * nkp + j, js + j);
                else s_J[e * nkp + j] = 0.f;
            }
        }
        cp_async_wait_all4();
        __syncthreads();
        if (has_task) {
#pragma unroll
            for (int pp = 0; pp < 4; ++pp) {
                const int e_lo = max(pb[pp], eb) - eb, e_hi = min(pb[pp + 1], eb + cnt) - eb;
                for (int e = e_lo; e < e_hi; ++e) {
                    const float4 ra = *(const float4*)(s_rows + e * rpm + 4 * rb);
                    const float4 jv = *(const float4*)(s_J + e * nkp + 4 * jb);
                    const float av[4] = {ra.x, ra.y, ra.z, ra.w}, bv[4] = {jv.x, jv.y, jv.z, jv.w};
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int w = 0; w < 4; ++w) acc[pp][u * 4 + w] = fmaf(av[u], bv[w], acc[pp][u * 4 + w]);
                }
            }
        }
    }
    // packed rows: chunk c of K block kb holds p = 16 kb + 4 c .. + 3
    const int kb = c4 / 4, c = c4 % 4;
    float* Ap = packed + d.a_off;
    const long long pstride = (long long)d.Mpad * 16;
    float* A_hi = Ap + (2LL * kb) * pstride;
    float* A_lo = Ap + (2LL * kb + 1) * pstride;
    if (has_task) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const int rr = 4 * rb + u, j = 4 * jb + w;
                if (rr < r && j < nkg) {
                    const int i = rr * nkg + j;
                    float hv[4], lv[4];
#pragma unroll
                    for (int pp = 0; pp < 4; ++pp) {
                        const float v = acc[pp][u * 4 + w];
                        hv[pp] = tf32_rna_sa(v);
                        lv[pp] = tf32_rna_sa(v - hv[pp]);
                    }
                    const long long o = (long long)(i >> 3) * 128 + c * 32 + (i & 7) * 4;
                    *(float4*)(A_hi + o) = make_float4(hv[0], hv[1], hv[2], hv[3]);
                    *(float4*)(A_lo + o) = make_float4(lv[0], lv[1], lv[2], lv[3]);
                }
            }
    }
    for (int i = M + tid; i < d.Mpad; i += kSAThreads) {
        const long long o = (long long)(i >> 3) * 128 + c * 32 + (i & 7) * 4;
        *(float4*)(A_hi + o) = make_float4(0.f, 0.f, 0.f, 0.f);
        *(float4*)(A_lo + o) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

void launch_xi_stageA_pack(const XiDevice& x, const long long* d_p_prefix, const float* J, int nkg,
                           const long long* d_chunk_prefix, long long nchunks, const TcGemmDesc* d_descs,
                           float* packed, cudaStream_t st) {
    const long long* rowel_off = d_p_prefix + (x.n_groups + 1);
    const int rmax = x.r_max;
    const int rpm = (rmax + 3) & ~3, nkp = (nkg + 3) & ~3;
    if ((rpm / 4) * (nkp / 4) <= kSAThreads) {
        const size_t sm = (size_t)kSA2Ent * (rpm + nkp) * 4;
        cudaFuncSetAttribute(k_xi_stageA_pack_reg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_xi_stageA_pack_reg<<<(unsigned)nchunks, kSAThreads, sm, st>>>(x, d_p_prefix, rowel_off, J, nkg,
                                                                        d_chunk_prefix, d_descs, packed);
        SGL_COUNT(1);
        return;
    }
    const size_t sm = (4ULL * rmax * nkg + (size_t)kSAEnt * (rpm + nkp)) * 4;
    cudaFuncSetAttribute(k_xi_stageA_pack, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_xi_stageA_pack<<<(unsigned)nchunks, kSAThreads, sm, st>>>(x, d_p_prefix, rowel_off, J, nkg, d_chunk_prefix,
                                                                d_descs, packed);
    SGL_COUNT(1);
}

// E_g[i, p] = cos(kk_i kap_p) (i < nk) / sin(kk_{i-nk} kap_p): one CTA per global p
// comp = 1 (mixed path): m = 0 groups get cos - 1 = -2 sin^2(x/2) in place of cos, so that
// G_r = sum (cos - 1) T + sum_q U (J0 - 1) carries no cancellation against sum_rows.
template <typename TT>
__global__ void k_xi_E(XiDevice x, const double* __restrict__ kk, int nk, const long long* __restrict__ E_off,
                       const long long* __restrict__ p_prefix, TT* __restrict__ E, int comp) {
    const long long P = blockIdx.x;
    const int g = find_group(p_prefix, x.n_groups, P);
    const int p = (int)(P - p_prefix[g]);
    const int nP = x.g_nP[g];
    const bool cm1 = comp && x.g_m[g] == 0;
    const double kap = x.kmc[x.idx_p[P]];
    TT* Eg = E + E_off[g];
    for (int i = threadIdx.x; i < nk; i += blockDim.x) {
        double s, c;
        const double ph = kk[i] * kap;
        sincos(ph, &s, &c);
        if (cm1) { const double h = sin(0.5 * ph); c = -2.0 * h * h; }
        Eg[(long long)i * nP + p] = (TT)c;
        Eg[(long long)(nk + i) * nP + p] = (TT)s;
    }
}

// Mixed path: the same table in FP32 with no FP64 transcendental.  The phase k kap is formed in
// float-float and reduced exactly (halfangle_sincos_ff), then, with s = sin(ph/2), c = cos(ph/2):
// cos ph = (c - s)(c + s), sin ph = 2 s c, and for m = 0 groups cos ph - 1 = -2 s^2.
__global__ void k_xi_E_ff(XiDevice x, const double* __restrict__ kk, int nk, const long long* __restrict__ E_off,
                          const long long* __restrict__ p_prefix, float* __restrict__ E) {
    const long long P = blockIdx.x;
    const int g = find_group(p_prefix, x.n_groups, P);
    const int p = (int)(P - p_prefix[g]);
    const int nP = x.g_nP[g];
    const bool cm1 = x.g_m[g] == 0;
    const ff kap = ff_from_double(x.kmc[x.idx_p[P]]);
    float* Eg = E + E_off[g];
    for (int i = threadIdx.x; i < nk; i += blockDim.x) {
        float s, c, ph_hi, ph_lo;
        halfangle_sincos_ff(ff_from_double(kk[i]), kap, s, c, ph_hi, ph_lo);
        Eg[(long long)i * nP + p] = cm1 ? -2.f * s * s : (c - s) * (c + s);
        Eg[(long long)(nk + i) * nP + p] = 2.f * s * c;
    }
}

void launch_xi_E(int precision, const XiDevice& x, const double* kk, int nk, const long long* E_off,
                 const long long* d_p_prefix, int total_p, void* E, cudaStream_t st) {
    if (precision == SGL_FP64) { k_xi_E<double><<<total_p, 128, 0, st>>>(x, kk, nk, E_off, d_p_prefix, (double*)E, 0); SGL_COUNT(1); }
    else { k_xi_E_ff<<<total_p, 128, 0, st>>>(x, kk, nk, E_off, d_p_prefix, (float*)E); SGL_COUNT(1); }
}

// V[g, r, j] = sum_q U_g[r, q] (J0 - 1)(gam_q kg_j) for the m = 0 groups (compensated form),
// U_g = sum over p of the group's rows; one CTA per (group row), threads over j.  FP64.
template <typename VT>
__global__ void k_xi_V(XiDevice x, const double* __restrict__ J0m1, int nkg, VT* __restrict__ V) {
    const int R = blockIdx.x;                     // global row index
    int g = 0;
    {
        int lo = 0, hi = x.n_groups - 1;
        while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (x.g_row_off[mid] <= R) lo = mid; else hi = mid - 1; }
        g = lo;
    }
    if (x.g_m[g] != 0) return;
    const int rr = R - (int)x.g_row_off[g];
    const int nQ = x.g_nQ[g];
    const double* U = x.U0 + x.g_u_off[g] + (long long)rr * nQ;
    const int* qs = x.idx_q + x.g_q_off[g];
    for (int j = threadIdx.x; j < nkg; j += blockDim.x) {
        double a = 0.0;
        for (int q = 0; q < nQ; ++q) a = fma(U[q], J0m1[(long long)qs[q] * nkg + j], a);
        V[(long long)R * nkg + j] = (VT)a;
    }
}

void launch_xi_V(const XiDevice& x, const double* J0m1, int nkg, double* V, int total_rows, cudaStream_t st) {
    if (total_rows > 0) { k_xi_V<double><<<total_rows, 128, 0, st>>>(x, J0m1, nkg, V); SGL_COUNT(1); }
}

// Mixed path: V rounded to FP32 where it is formed (the square kernel adds it in FP32), and the two
// per-row correction terms of the square kernel as float-float tables, formed once in FP64:
//   kres[n][R] = k_n res_R (m = 0 rows: imaginary part)   hq[R][j] = q_j res_R / 2 (m = 1 rows)
// kres_t = 1: kres laid out [R][n] instead (the fused kernel reads it with lanes along n).
__global__ void k_xi_corr_tables(const double* __restrict__ res, int rows, const double* __restrict__ kk, int nk,
                                 const double* __restrict__ kg, int nkg, float2* __restrict__ kres,
                                 float2* __restrict__ hq, int kres_t) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n1 = (long long)nk * rows, n2 = (long long)rows * nkg;
    if (t < n1) {
        const double v = kk[t / rows] * res[t % rows];
        const ff f = ff_from_double(v);
        kres[kres_t ? (t % rows) * nk + t / rows : t] = make_float2(f.hi, f.lo);
    } else if (t < n1 + n2) {
        const long long u = t - n1;
        const double v = (0.5 * kg[u % nkg]) * res[u / nkg];
        const ff f = ff_from_double(v);
        hq[u] = make_float2(f.hi, f.lo);
    }
}

void launch_xi_V_mixed(const XiDevice& x, const double* J0m1, int nkg, float* Vf, int total_rows, const double* kk,
                       int nk, const double* kg, float2* kres, float2* hq, cudaStream_t st, int kres_t) {
    if (total_rows <= 0) return;
    k_xi_V<float><<<total_rows, 128, 0, st>>>(x, J0m1, nkg, Vf);
    SGL_COUNT(1);
    const long long tot = (long long)nk * total_rows + (long long)total_rows * nkg;
    k_xi_corr_tables<<<ceil_div(tot, 256), 256, 0, st>>>(x.res, total_rows, kk, nk, kg, nkg, kres, hq, kres_t);
    SGL_COUNT(1);
}

__global__ void k_xi_square_sum(const double* __restrict__ part, int nsplit, long long npt, double* __restrict__ out_re,
                                double* __restrict__ out_im);

// round(b + (h + l)) in FP32 for a float-float addend (TwoSum of b and h, then the tails)
__device__ __forceinline__ float add_ff(float b, float2 hl) {
    const float s = b + hl.x, bp = s - b;
    const float err = (b - (s - bp)) + (hl.x - bp);
    return s + (err + hl.y);
}

// Mixed square: no FP64 arithmetic per element.  The FP64 form's fma(k, res, b) and
// fma(q/2, res, a) round k res and q res / 2 once in FP64 and add them to the FP32 G value; here
// the same FP64 products come as float-float tables and the sum is rounded once to FP32.
__global__ void k_xi_square_mixed(XiDevice x, const long long* __restrict__ G_off, const float* __restrict__ G,
                                  int nk, int nkg, const float* __restrict__ Vf, const float2* __restrict__ kres,
                                  const float2* __restrict__ hq, int rows, int nsplit, double* __restrict__ part) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long npt = (long long)nk * nkg;
    if (e >= npt) return;
    const int n = (int)(e / nkg), j = (int)(e % nkg);
    const int per = (x.n_groups + nsplit - 1) / nsplit;
    const int g0 = blockIdx.y * per, g1 = min(x.n_groups, g0 + per);
    double re = 0.0, im = 0.0;
    for (int g = g0; g < g1; ++g) {
        const int r = x.g_r[g], m = x.g_m[g];
        const double sign = (m == 0) ? 1.0 : ((m & 1) ? -2.0 : 2.0);
        const float* Gg = G + G_off[g] + (long long)n * r * nkg + j;
        const float* Gi = G + G_off[g] + (long long)(nk + n) * r * nkg + j;
        const long long R0 = x.g_row_off[g];
        float gre = 0.f, gim = 0.f;
        for (int rr = 0; rr < r; ++rr) {
            float a = Gg[(long long)rr * nkg];
            float b = Gi[(long long)rr * nkg];
            if (m == 0) {
                a += Vf[(R0 + rr) * nkg + j];
                b = add_ff(b, kres[(long long)n * rows + R0 + rr]);
            } else if (m == 1) {
                a = add_ff(a, hq[(R0 + rr) * nkg + j]);
            }
            gre = fmaf(a, a, fmaf(-b, b, gre));
            gim = fmaf(a, b, gim);
        }
        re = fma(0.5 * sign, (double)gre, re);
        im = fma(0.5 * sign, 2.0 * (double)gim, im);
    }
    part[(long long)blockIdx.y * npt + e] = re;
    part[(long long)(nsplit + blockIdx.y) * npt + e] = im;
}

void launch_xi_square_mixed(const XiDevice& x, const long long* G_off, const float* G, int nk, int nkg, const float* Vf,
                            const float2* kres, const float2* hq, int rows, int nsplit, double* part, double* out_re,
                            double* out_im, cudaStream_t st) {
    const long long tot = (long long)nk * nkg;
    dim3 grid(ceil_div(tot, 128), nsplit);
    k_xi_square_mixed<<<grid, 128, 0, st>>>(x, G_off, G, nk, nkg, Vf, kres, hq, rows, nsplit, part);
    SGL_COUNT(1);
    k_xi_square_sum<<<ceil_div(tot, 256), 256, 0, st>>>(part, nsplit, tot, out_re, out_im);
    SGL_COUNT(1);
}

// stage C: thread per output (n, j) and group chunk (blockIdx.y); groups and rows in a fixed
// order; per-chunk partials then a fixed-order sum (deterministic).  Within a group the FP32 path
// accumulates in FP32 (rows of one group), across groups in FP64.
// V != nullptr: compensated m = 0 form (real part + V instead of - sum_rows).
template <typename TT>
__global__ void k_xi_square(XiDevice x, const long long* __restrict__ G_off, const TT* __restrict__ G,
                            const double* __restrict__ kk, int nk, const double* __restrict__ kg, int nkg,
                            const double* __restrict__ V, int nsplit, double* __restrict__ part) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long npt = (long long)nk * nkg;
    if (e >= npt) return;
    const int n = (int)(e / nkg), j = (int)(e % nkg);
    const double k = kk[n], q = kg[j];
    const int per = (x.n_groups + nsplit - 1) / nsplit;
    const int g0 = blockIdx.y * per, g1 = min(x.n_groups, g0 + per);
    double re = 0.0, im = 0.0;
    for (int g = g0; g < g1; ++g) {
        const int r = x.g_r[g], m = x.g_m[g];
        const double sign = (m == 0) ? 1.0 : ((m & 1) ? -2.0 : 2.0);
        const TT* Gg = G + G_off[g] + (long long)n * r * nkg + j;
        const TT* Gi = G + G_off[g] + (long long)(nk + n) * r * nkg + j;
        const double* res = x.res + x.g_row_off[g];
        const double* srow = x.sum_rows + x.g_row_off[g];
        const double* Vg = V ? V + x.g_row_off[g] * (long long)nkg + j : nullptr;
        TT gre = TT(0), gim = TT(0);
        for (int rr = 0; rr < r; ++rr) {
            TT a = Gg[(long long)rr * nkg];
            TT b = Gi[(long long)rr * nkg];
            if (m == 0) {
                if (Vg) a += (TT)Vg[(long long)rr * nkg];
                else a = (TT)((double)a - srow[rr]);
                b = (TT)fma(k, res[rr], (double)b);
            } else if (m == 1) {
                a = (TT)fma(0.5 * q, res[rr], (double)a);
            }
            gre = fma(a, a, fma(-b, b, gre));
            gim = fma(a, b, gim);
        }
        re = fma(0.5 * sign, (double)gre, re);
        im = fma(0.5 * sign, 2.0 * (double)gim, im);
    }
    part[(long long)blockIdx.y * npt + e] = re;
    part[(long long)(nsplit + blockIdx.y) * npt + e] = im;
}

__global__ void k_xi_square_sum(const double* __restrict__ part, int nsplit, long long npt, double* __restrict__ out_re,
                                double* __restrict__ out_im) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= npt) return;
    double re = 0.0, im = 0.0;
    for (int s = 0; s < nsplit; ++s) { re += part[(long long)s * npt + e]; im += part[(long long)(nsplit + s) * npt + e]; }
    out_re[e] = re;
    out_im[e] = im;
}

void launch_xi_square(int precision, const XiDevice& x, const long long* G_off, const void* G, const double* kk, int nk,
                      const double* kg, int nkg, const double* V, int nsplit, double* part, double* out_re,
                      double* out_im, cudaStream_t st) {
    const long long tot = (long long)nk * nkg;
    dim3 grid(ceil_div(tot, 128), nsplit);
    if (precision == SGL_FP64) { k_xi_square<double><<<grid, 128, 0, st>>>(x, G_off, (const double*)G, kk, nk, kg, nkg, V, nsplit, part); SGL_COUNT(1); }
    else { k_xi_square<float><<<grid, 128, 0, st>>>(x, G_off, (const float*)G, kk, nk, kg, nkg, V, nsplit, part); SGL_COUNT(1); }
    k_xi_square_sum<<<ceil_div(tot, 256), 256, 0, st>>>(part, nsplit, tot, out_re, out_im);
    SGL_COUNT(1);
}

// ---- 1-D path along k_kappa (k_gamma = 0): G_R = sum_p e^{i k kap_p} W0[R, p] - sum0_R + i k res0_R
// CTA (point, row chunk); partial sums part[chunk, point], then a fixed-order sum.
__global__ void __launch_bounds__(256)
k_xi_line_k(XiDevice x, const double* __restrict__ kk, int nk, double* __restrict__ part) {
    extern __shared__ double sm[];
    double* ec = sm;
    double* es = sm + x.n_kmc;
    double* red = sm + 2 * x.n_kmc;
    const int n = blockIdx.x;
    const double k = kk[n];
    for (int p = threadIdx.x; p < x.n_kmc; p += blockDim.x) sincos(k * x.kmc[p], &es[p], &ec[p]);
    __syncthreads();
    const int per = (x.R0 + kLineChunks - 1) / kLineChunks;
    const int r0 = blockIdx.y * per, r1 = min(x.R0, r0 + per);
    double re = 0.0, im = 0.0;
    for (int R = r0 + threadIdx.x; R < r1; R += blockDim.x) {
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
    if (threadIdx.x == 0) {
        part[(long long)blockIdx.y * nk + n] = 0.5 * re;
        part[(long long)(kLineChunks + blockIdx.y) * nk + n] = 0.5 * im;
    }
}

__global__ void k_line_reduce(const double* __restrict__ part, int nchunks, int npt, double* __restrict__ re,
                              double* __restrict__ im) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npt) return;
    double r = 0.0, m = 0.0;
    for (int c = 0; c < nchunks; ++c) { r += part[(long long)c * npt + i]; m += part[(long long)(nchunks + c) * npt + i]; }
    re[i] = r;
    im[i] = m;
}

void launch_xi_line_k(const XiDevice& x, const double* kk, int nk, double* out_re, double* out_im, double* part,
                      cudaStream_t st) {
    const size_t sm = (2 * (size_t)x.n_kmc + 32) * sizeof(double);
    dim3 grid(nk, kLineChunks);
    { k_xi_line_k<<<grid, 256, sm, st>>>(x, kk, nk, part); SGL_COUNT(1); }
    { k_line_reduce<<<ceil_div(nk, 256), 256, 0, st>>>(part, kLineChunks, nk, out_re, out_im); SGL_COUNT(1); }
}

// ---- 1-D path along k_gamma (k_kappa = 0): per m, G_R = sum_q U_m[R, q] J_m(gam_q kg) (+ residuals)
// CTA (point, chunk of the concatenated m = 0, 1, 2 rows); partials then a fixed-order sum.
__global__ void __launch_bounds__(256)
k_xi_line_g(XiDevice x, const double* __restrict__ kg, int nkg, double* __restrict__ part) {
    extern __shared__ double sm[];
    double* Jq = sm;                 // [3][n_gmc]
    double* red = sm + 3 * x.n_gmc;
    const int j = blockIdx.x;
    const double q = kg[j];
    for (int c = threadIdx.x; c < 3 * x.n_gmc; c += blockDim.x) {
        const int m = c / x.n_gmc, qi = c % x.n_gmc;
        Jq[c] = bessel_jm(m, x.gmc[qi] * q);
    }
    __syncthreads();
    const int Rtot = x.Rm[0] + x.Rm[1] + x.Rm[2];
    const int per = (Rtot + kLineChunks - 1) / kLineChunks;
    const int r0 = blockIdx.y * per, r1 = min(Rtot, r0 + per);
    double tot = 0.0;
    for (int Rg = r0 + threadIdx.x; Rg < r1; Rg += blockDim.x) {
        int m = 0, R = Rg;
        if (R >= x.Rm[0]) { R -= x.Rm[0]; m = 1; if (R >= x.Rm[1]) { R -= x.Rm[1]; m = 2; } }
        const double* u = x.U[m] + (long long)R * x.n_gmc;
        const double* J = Jq + m * x.n_gmc;
        double a = 0.0;
        for (int c = 0; c < x.n_gmc; ++c) a = fma(u[c], J[c], a);
        if (m == 0) a -= x.summ[m][R];
        else if (m == 1) a = fma(0.5 * q, x.resm[m][R], a);
        const double sign = (m == 0) ? 1.0 : ((m & 1) ? -2.0 : 2.0);
        tot += 0.5 * sign * (a * a);
    }
    tot = block_sum(tot, red);
    if (threadIdx.x == 0) {
        part[(long long)blockIdx.y * nkg + j] = tot;
        part[(long long)(kLineChunks + blockIdx.y) * nkg + j] = 0.0;
    }
}

void launch_xi_line_g(const XiDevice& x, const double* kg, int nkg, double* out_re, double* out_im, double* part,
                      cudaStream_t st) {
    const size_t sm = (3 * (size_t)x.n_gmc + 32) * sizeof(double);
    dim3 grid(nkg, kLineChunks);
    { k_xi_line_g<<<grid, 256, sm, st>>>(x, kg, nkg, part); SGL_COUNT(1); }
    { k_line_reduce<<<ceil_div(nkg, 256), 256, 0, st>>>(part, kLineChunks, nkg, out_re, out_im); SGL_COUNT(1); }
}

}  // namespace sgl
