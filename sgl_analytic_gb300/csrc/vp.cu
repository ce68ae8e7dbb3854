// Positive (vp) Cox closure: ln R(k, q) = ln E_U exp( sum_s z_s(U_s; k, q) ),
//   z_s(u_j) = sum_{g in shell s} D_g(u_j) Y_g,   Y_g = sum_{c in g} w_c F_c,
//   F_c(k, q) = e_c J_c + J_c - 1,  e = expm1(i k kap_c), J = J0(q gam_c)
// (reference: FusedVP.lnR_blocked pos_closure_fused.py:119-140 = _fused_groups :51-105 +
//  _chain_recursion pos_closure.py:184-240).
//
// D_g(u) = lam_g(u) - 1 is, per group, c + a (u - anchor) + b on an interval of states that reaches
// an end of the state grid (rate_intervals pos_closure_fused.py:18-48), and E_w[D_g] = 0 exactly
// (the rates keep the mean, pos_closure.py:15).  The host sorts each shell's groups into RUNS of
// one kind and one interval bound (linear; "left" = states lo..47; "right" = states 0..hi) and
// stores per-cell weights (w a, w b).  Then
//   z_s(u_j) = u_j A_lin + sum_{left runs, lo <= j} [(u_j - u_lo) A_r + B_r]
//            + sum_{right runs, j <= hi} [(u_j - u_hi) A_r + B_r] + const,
//   A_r = sum_{c in r} (w a)_c F_c,  B_r = sum_{c in r} (w b)_c F_c.
// The constant (c = -1 offsets, linear intercepts) is not formed: z_s has zero stationary mean, so
// z_s = z_partial - E_w[z_partial] exactly, and that projection also removes the common-mode part
// of the rounding error (what keeps the mixed path within 1e-8 of FP64).
//
// Phase 1 (k_vp_z): one CTA per (shell, 16 k x 32 q tile); each thread owns 2 x 2 points.  Cells of
// a run stream through shared memory in chunks of 32 (table rows e[u][k], (J, J - 1)[u][q] gathered
// by cell index, coalesced along k / q); per point 4 FMAs + 2 for F.  Mixed: FP32 chunk sums folded
// into float-float run totals (TwoSum); FP64: FP64 throughout.  Run totals go to FP64 running sums
// over the sorted bounds and each state's z is written once (FP64, [shell][state][point]).
// Phase 2 (k_vp_chain): one thread per point walks the shells: projection, alpha' = K^T alpha (or the
// stationary weights at s = 0) times exp(z - max Re z), renormalisation by max |alpha|, log scale;
// FP64 in both precisions.  Thread-private shared memory, no barriers.
#include "kernels.cuh"

namespace sgl {

constexpr int kVpNS = 48;                 // latent states (Gauss-Hermite nodes)
constexpr int kZK = 16, kZQ = 32;         // phase-1 point tile (k x q)
constexpr int kZThreads = 128;            // 2 x 2 points per thread
constexpr int kZCh = 32;                  // cells per staged chunk
constexpr int kChPts = 56;                // phase-2 points per CTA (2 CTAs per SM with K staged)

template <typename TT> struct V2;
template <> struct V2<float> { using T = float2; };
template <> struct V2<double> { using T = double2; };

// e[u][i] = (cos - 1, sin)(k_i kap_u) from the half angle (no cancellation); Jt[u][j] = (J0, J0 - 1)
template <typename TT>
__global__ void k_vp_tables(const double* __restrict__ ku, const double* __restrict__ gu, int U,
                            const double* __restrict__ kv, int nk, const double* __restrict__ qv, int nq,
                            typename V2<TT>::T* __restrict__ e, typename V2<TT>::T* __restrict__ Jt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long ne = (long long)U * nk;
    if (t < ne) {
        const int u = (int)(t / nk), i = (int)(t % nk);
        const double ph = kv[i] * ku[u];
        double s, c;
        sincos(0.5 * ph, &s, &c);
        e[t].x = (TT)(-2.0 * s * s);
        e[t].y = (TT)(2.0 * s * c);
    } else if (t < ne + (long long)U * nq) {
        const long long r = t - ne;
        const int u = (int)(r / nq), j = (int)(r % nq);
        const double jm = j0m1_d(qv[j] * gu[u]);
        Jt[r].x = (TT)(1.0 + jm);
        Jt[r].y = (TT)jm;
    }
}

// hi + lo += p  (Knuth TwoSum; no FMA contraction applies to additions)
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float p) {
    const float s = hi + p;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (p - bb);
    hi = s;
    lo += err;
}

// asynchronous global -> shared copies (zero-filled when !pred; the source address is then unused)
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem, bool pred) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    const int n = pred ? BYTES : 0;
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" :: "r"(sa), "l"(gmem), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" :: "r"(sa), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" :: "n"(N) : "memory"); }

template <typename TT>
__global__ void __launch_bounds__(kZThreads)
k_vp_z(VpDevice d, const typename V2<TT>::T* __restrict__ e, const typename V2<TT>::T* __restrict__ Jt, int nk,
       int nq, int kb, int nkc, double2* __restrict__ zp, double2* __restrict__ alin, long long NP, int npieces) {
    using T2 = typename V2<TT>::T;
    __shared__ __align__(16) T2 s_e[2][kZCh][kZK];
    __shared__ __align__(16) T2 s_J[2][kZCh][kZQ];
    __shared__ __align__(16) T2 s_w[2][kZCh];
    constexpr bool MIX = sizeof(TT) == 4;
    constexpr int EB = (int)sizeof(T2);
    // blockIdx.z = (shell, piece): a piece is a contiguous part of the shell's run list.  Each run's
    // contribution to the states is additive, so pieces write partial z and A_lin (their own
    // slices of zp / alin) that the chain kernel sums in piece order.  More than one piece only
    // when the point tile grid alone would leave the GPU idle (the k-reach probes).
    const int s = blockIdx.z / npieces, piece = blockIdx.z % npieces;
    zp += (long long)piece * d.nsh * kVpNS * NP;
    alin += (long long)piece * d.nsh * NP;
    const int q0 = blockIdx.x * kZQ, k0 = kb + blockIdx.y * kZK, kend = kb + nkc;
    const int t = threadIdx.x, tq = t % 16, tk = t / 16;
    // my points: (k0 + tk + 8 m, q0 + tq + 16 i), index P = 2 m + i
    double SAr[4], SAi[4], SBr[4], SBi[4], ALr[4], ALi[4];
#pragma unroll
    for (int P = 0; P < 4; ++P) { SAr[P] = SAi[P] = SBr[P] = SBi[P] = ALr[P] = ALi[P] = 0.0; }
    long long pidx[4];
    bool live[4];
#pragma unroll
    for (int P = 0; P < 4; ++P) {
        const int k = k0 + tk + 8 * (P >> 1), q = q0 + tq + 16 * (P & 1);
        live[P] = k < kend && q < nq;
        pidx[P] = (long long)(k - kb) * nq + q;
    }
    int jcur = 0;
    auto emit_to = [&](int jend) {
        for (; jcur < jend; ++jcur) {
            const double uj = d.u[jcur];
            double2* row = zp + ((long long)s * kVpNS + jcur) * NP;
#pragma unroll
            for (int P = 0; P < 4; ++P)
                if (live[P]) row[pidx[P]] = make_double2(fma(uj, SAr[P], SBr[P]), fma(uj, SAi[P], SBi[P]));
        }
    };
    // chunks of <= 32 cells never straddle a run; the next chunk is copied (cp.async) into the other
    // buffer while the current one is summed
    auto issue = [&](int buf, long long base, long long c1) {
        const int cnt = (int)((c1 - base) < kZCh ? (c1 - base) : kZCh);
        for (int idx = t; idx < kZCh * kZK; idx += kZThreads) {
            const int c = idx / kZK, rr = idx % kZK, k = k0 + rr;
            const bool ok = c < cnt && k < kend;
            cp_async<EB>(&s_e[buf][c][rr], ok ? (const void*)(e + (long long)d.cu[base + c] * nk + k) : (const void*)e, ok);
        }
        for (int idx = t; idx < kZCh * kZQ; idx += kZThreads) {
            const int c = idx / kZQ, rr = idx % kZQ, q = q0 + rr;
            const bool ok = c < cnt && q < nq;
            cp_async<EB>(&s_J[buf][c][rr], ok ? (const void*)(Jt + (long long)d.cu[base + c] * nq + q) : (const void*)Jt, ok);
        }
        if (t < kZCh) {
            const bool ok = t < cnt;
            if constexpr (MIX) cp_async<EB>(&s_w[buf][t], ok ? (const void*)(d.wabf + base + t) : (const void*)d.wabf, ok);
            else cp_async<EB>(&s_w[buf][t], ok ? (const void*)(d.wab + base + t) : (const void*)d.wab, ok);
        }
        cp_async_commit();
    };
    const int rs0 = d.sh_run[s], rs1 = d.sh_run[s + 1];
    const int r0 = rs0 + (int)((long long)(rs1 - rs0) * piece / npieces);
    const int r1 = rs0 + (int)((long long)(rs1 - rs0) * (piece + 1) / npieces);
    int buf = 0;
    if (r0 < r1) issue(0, d.run_cell[r0], d.run_cell[r0 + 1]);
    for (int r = r0; r < r1; ++r) {
        const long long c0 = d.run_cell[r], c1 = d.run_cell[r + 1];
        // run totals: mixed = float-float (hi, lo), FP64 = plain
        TT hi[4][4], lo[4][4];
#pragma unroll
        for (int P = 0; P < 4; ++P)
#pragma unroll
            for (int v = 0; v < 4; ++v) { hi[P][v] = TT(0); lo[P][v] = TT(0); }
        for (long long base = c0; base < c1; base += kZCh) {
            const int cnt = (int)((c1 - base) < kZCh ? (c1 - base) : kZCh);
            // prefetch the next chunk (this run's, or the next run's first)
            const long long nb = base + kZCh;
            const bool has_next = nb < c1 || r + 1 < r1;
            if (has_next) {
                if (nb < c1) issue(buf ^ 1, nb, c1);
                else issue(buf ^ 1, d.run_cell[r + 1], d.run_cell[r + 2]);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
            TT p[4][4];
#pragma unroll
            for (int P = 0; P < 4; ++P)
#pragma unroll
                for (int v = 0; v < 4; ++v) p[P][v] = TT(0);
            for (int c = 0; c < cnt; ++c) {
                const T2 wv = s_w[buf][c];
                const T2 ev[2] = {s_e[buf][c][tk], s_e[buf][c][tk + 8]};
                const T2 jv[2] = {s_J[buf][c][tq], s_J[buf][c][tq + 16]};
#pragma unroll
                for (int P = 0; P < 4; ++P) {
                    const T2 ee = ev[P >> 1], jj = jv[P & 1];
                    const TT Fr = ee.x * jj.x + jj.y;          // (cos - 1) J + (J - 1)
                    const TT Fi = ee.y * jj.x;                 // sin J
                    p[P][0] += wv.x * Fr; p[P][1] += wv.x * Fi;
                    p[P][2] += wv.y * Fr; p[P][3] += wv.y * Fi;
                }
            }
#pragma unroll
            for (int P = 0; P < 4; ++P)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    if constexpr (MIX) ff_acc(hi[P][v], lo[P][v], p[P][v]);
                    else hi[P][v] += p[P][v];
                }
            __syncthreads();                  // buffer `buf` is refilled by the next prefetch
            buf ^= 1;
        }
        const int kind = d.run_kind[r], bound = d.run_bound[r];
        if (kind == 0) {                                   // linear: u_j A (intercept dropped)
#pragma unroll
            for (int P = 0; P < 4; ++P) {
                ALr[P] += (double)hi[P][0] + (double)lo[P][0];
                ALi[P] += (double)hi[P][1] + (double)lo[P][1];
            }
        } else if (kind == 1) {                            // left: states >= lo, anchored at u_lo
            emit_to(bound);
            const double ub = d.u[bound];
#pragma unroll
            for (int P = 0; P < 4; ++P) {
                const double Ar = (double)hi[P][0] + (double)lo[P][0], Ai = (double)hi[P][1] + (double)lo[P][1];
                const double Br = (double)hi[P][2] + (double)lo[P][2], Bi = (double)hi[P][3] + (double)lo[P][3];
                SAr[P] += Ar; SAi[P] += Ai;
                SBr[P] += fma(-ub, Ar, Br); SBi[P] += fma(-ub, Ai, Bi);
            }
        } else {                                           // right: states <= hi, anchored at u_hi
            // = u_j A on every state (+ a dropped constant) minus [(u_j - u_hi) A + B] on states > hi
            emit_to(bound + 1);
            const double ub = d.u[bound];
#pragma unroll
            for (int P = 0; P < 4; ++P) {
                const double Ar = (double)hi[P][0] + (double)lo[P][0], Ai = (double)hi[P][1] + (double)lo[P][1];
                const double Br = (double)hi[P][2] + (double)lo[P][2], Bi = (double)hi[P][3] + (double)lo[P][3];
                ALr[P] += Ar; ALi[P] += Ai;
                SAr[P] -= Ar; SAi[P] -= Ai;
                SBr[P] += fma(ub, Ar, -Br); SBi[P] += fma(ub, Ai, -Bi);
            }
        }
    }
    emit_to(kVpNS);
#pragma unroll
    for (int P = 0; P < 4; ++P)
        if (live[P]) alin[(long long)s * NP + pidx[P]] = make_double2(ALr[P], ALi[P]);
}

__global__ void __launch_bounds__(kChPts)
k_vp_chain(VpDevice d, const double2* __restrict__ zp, const double2* __restrict__ alin, long long NP, int nq, int kb,
           double* __restrict__ out_re, double* __restrict__ out_im, int npieces) {
    extern __shared__ __align__(16) unsigned char vsm[];
    double (*ar)[kChPts] = (double (*)[kChPts])vsm;                       // alpha (normalised)
    double (*ai)[kChPts] = (double (*)[kChPts])(vsm + 1 * kVpNS * kChPts * 8);
    double (*br)[kChPts] = (double (*)[kChPts])(vsm + 2 * kVpNS * kChPts * 8);   // z, then alpha'
    double (*bi)[kChPts] = (double (*)[kChPts])(vsm + 3 * kVpNS * kChPts * 8);
    double* sK = (double*)(vsm + 4 * kVpNS * kChPts * 8);                    // K[s-1], 48 x 48
    const int t = threadIdx.x;
    const long long p = (long long)blockIdx.x * kChPts + t;
    const bool live = p < NP;                  // dead threads only help stage K
    double scale = 0.0;
    for (int s = 0; s < d.nsh; ++s) {
        if (s > 0) {
            __syncthreads();
            const double* Ks = d.K + (long long)(s - 1) * kVpNS * kVpNS;
            for (int e = t; e < kVpNS * kVpNS; e += kChPts) sK[e] = Ks[e];
            __syncthreads();
        }
        if (!live) continue;
        double2 al = alin[(long long)s * NP + p];
        for (int pc = 1; pc < npieces; ++pc) {
            const double2 a2 = alin[((long long)pc * d.nsh + s) * NP + p];
            al.x += a2.x; al.y += a2.y;
        }
        double mr = 0.0, mi = 0.0;
        for (int j = 0; j < kVpNS; ++j) {
            double2 zz = zp[((long long)s * kVpNS + j) * NP + p];
            for (int pc = 1; pc < npieces; ++pc) {
                const double2 z2 = zp[(((long long)pc * d.nsh + s) * kVpNS + j) * NP + p];
                zz.x += z2.x; zz.y += z2.y;
            }
            const double uj = d.u[j], wj = d.w[j];
            const double zr = fma(uj, al.x, zz.x), zi = fma(uj, al.y, zz.y);
            br[j][t] = zr; bi[j][t] = zi;
            mr = fma(wj, zr, mr); mi = fma(wj, zi, mi);
        }
        double mx = -1e300;
        for (int j = 0; j < kVpNS; ++j) {
            const double zr = br[j][t] - mr;
            br[j][t] = zr; bi[j][t] -= mi;
            mx = fmax(mx, zr);
        }
        double nrm = 0.0;
        for (int j0 = 0; j0 < kVpNS; j0 += 4) {
            double gr[4], gi[4];
            if (s == 0) {
#pragma unroll
                for (int q = 0; q < 4; ++q) { gr[q] = d.w[j0 + q]; gi[q] = 0.0; }
            } else {
#pragma unroll
                for (int q = 0; q < 4; ++q) { gr[q] = 0.0; gi[q] = 0.0; }
#pragma unroll 4
                for (int i = 0; i < kVpNS; ++i) {
                    const double xr = ar[i][t], xi = ai[i][t];
                    const double2 k01 = *(const double2*)(sK + i * kVpNS + j0);
                    const double2 k23 = *(const double2*)(sK + i * kVpNS + j0 + 2);
                    gr[0] = fma(k01.x, xr, gr[0]); gi[0] = fma(k01.x, xi, gi[0]);
                    gr[1] = fma(k01.y, xr, gr[1]); gi[1] = fma(k01.y, xi, gi[1]);
                    gr[2] = fma(k23.x, xr, gr[2]); gi[2] = fma(k23.x, xi, gi[2]);
                    gr[3] = fma(k23.y, xr, gr[3]); gi[3] = fma(k23.y, xi, gi[3]);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = j0 + q;
                const double m = exp(br[j][t] - mx);
                double sn, cs;
                sincos(bi[j][t], &sn, &cs);
                const double er = m * cs, ei = m * sn;
                const double nr = gr[q] * er - gi[q] * ei, ni = gr[q] * ei + gi[q] * er;
                br[j][t] = nr; bi[j][t] = ni;
                nrm = fmax(nrm, nr * nr + ni * ni);
            }
        }
        nrm = sqrt(nrm);
        const double inv = 1.0 / nrm;
        for (int j = 0; j < kVpNS; ++j) { ar[j][t] = br[j][t] * inv; ai[j][t] = bi[j][t] * inv; }
        scale += mx + log(nrm);
    }
    if (!live) return;
    double sr = 0.0, si = 0.0;
    for (int j = 0; j < kVpNS; ++j) { sr += ar[j][t]; si += ai[j][t]; }
    const long long o = (long long)kb * nq + p;
    out_re[o] = scale + 0.5 * log(sr * sr + si * si);
    out_im[o] = atan2(si, sr);
}

// The same chain for few points (the k-reach probe lines): one CTA per point, one thread per state.
// The per-state work (mat-vec over i in the same order, exp, sincos, normalisation) runs in
// parallel; the two ordered sums (the projection's weighted mean, the final state sum) stay on
// one thread in state order, and the maxima are order-free, so the results are those of
// k_vp_chain.
constexpr int kChSmallThreads = 64;

__global__ void __launch_bounds__(kChSmallThreads)
k_vp_chain_small(VpDevice d, const double2* __restrict__ zp, const double2* __restrict__ alin, long long NP, int nq,
                 int kb, double* __restrict__ out_re, double* __restrict__ out_im, int npieces) {
    __shared__ double sK[kVpNS * kVpNS];
    __shared__ double zr_s[kVpNS], zi_s[kVpNS], ar[kVpNS], ai[kVpNS];
    __shared__ double red[kChSmallThreads];
    __shared__ double s_mr, s_mi;
    const int j = threadIdx.x;
    const long long p = blockIdx.x;
    const bool st = j < kVpNS;
    double scale = 0.0;
    for (int s = 0; s < d.nsh; ++s) {
        __syncthreads();
        if (s > 0) {
            const double* Ks = d.K + (long long)(s - 1) * kVpNS * kVpNS;
            for (int e = j; e < kVpNS * kVpNS; e += kChSmallThreads) sK[e] = Ks[e];
        }
        double2 al = alin[(long long)s * NP + p];
        for (int pc = 1; pc < npieces; ++pc) {
            const double2 a2 = alin[((long long)pc * d.nsh + s) * NP + p];
            al.x += a2.x; al.y += a2.y;
        }
        if (st) {
            double2 zz = zp[((long long)s * kVpNS + j) * NP + p];
            for (int pc = 1; pc < npieces; ++pc) {
                const double2 z2 = zp[(((long long)pc * d.nsh + s) * kVpNS + j) * NP + p];
                zz.x += z2.x; zz.y += z2.y;
            }
            const double uj = d.u[j];
            zr_s[j] = fma(uj, al.x, zz.x);
            zi_s[j] = fma(uj, al.y, zz.y);
        }
        __syncthreads();
        if (j == 0) {
            double mr = 0.0, mi = 0.0;
            for (int i = 0; i < kVpNS; ++i) { mr = fma(d.w[i], zr_s[i], mr); mi = fma(d.w[i], zi_s[i], mi); }
            s_mr = mr; s_mi = mi;
        }
        __syncthreads();
        double zr = 0.0, zi = 0.0;
        if (st) { zr = zr_s[j] - s_mr; zi = zi_s[j] - s_mi; }
        red[j] = st ? zr : -1e300;
        __syncthreads();
        for (int o = kChSmallThreads / 2; o > 0; o >>= 1) {
            if (j < o) red[j] = fmax(red[j], red[j + o]);
            __syncthreads();
        }
        const double mx = red[0];
        __syncthreads();
        double nr = 0.0, ni = 0.0;
        if (st) {
            double gr, gi;
            if (s == 0) { gr = d.w[j]; gi = 0.0; }
            else {
                gr = 0.0; gi = 0.0;
                for (int i = 0; i < kVpNS; ++i) {
                    const double kij = sK[i * kVpNS + j];
                    gr = fma(kij, ar[i], gr); gi = fma(kij, ai[i], gi);
                }
            }
            const double m = exp(zr - mx);
            double sn, cs;
            sincos(zi, &sn, &cs);
            const double er = m * cs, ei = m * sn;
            nr = gr * er - gi * ei;
            ni = gr * ei + gi * er;
        }
        red[j] = st ? nr * nr + ni * ni : 0.0;
        __syncthreads();
        for (int o = kChSmallThreads / 2; o > 0; o >>= 1) {
            if (j < o) red[j] = fmax(red[j], red[j + o]);
            __syncthreads();
        }
        const double nrm = sqrt(red[0]);
        const double inv = 1.0 / nrm;
        if (st) { ar[j] = nr * inv; ai[j] = ni * inv; }
        scale += mx + log(nrm);
    }
    __syncthreads();
    if (j == 0) {
        double sr = 0.0, si = 0.0;
        for (int i = 0; i < kVpNS; ++i) { sr += ar[i]; si += ai[i]; }
        const long long o = (long long)kb * nq + p;
        out_re[o] = scale + 0.5 * log(sr * sr + si * si);
        out_im[o] = atan2(si, sr);
    }
}

size_t vp_table_bytes(int precision, int U, int nk, int nq) {
    const size_t es = precision == SGL_FP64 ? 8 : 4;
    return 2 * es * ((size_t)U * nk + (size_t)U * nq) + 256;
}

int vp_rows_per_pass(int nsh, int nk, int nq, size_t z_cap_bytes) {
    const size_t per_row = (size_t)nsh * (kVpNS + 1) * 16 * (size_t)nq;
    long long rows = (long long)(z_cap_bytes / (per_row > 0 ? per_row : 1));
    if (rows < 1) rows = 1;
    if (rows > nk) rows = nk;
    const long long passes = (nk + rows - 1) / rows;            // balanced passes (no thin last pass)
    return (int)((nk + passes - 1) / passes);
}

int vp_pieces(int nsh, int rows, int nq) {
    const long long base = (long long)ceil_div(nq, kZQ) * ceil_div(rows, kZK) * nsh;
    const long long want = 8LL * kNumSMs;                   // CTAs of 128 threads
    return (int)std::max(1LL, std::min(32LL, (want + base - 1) / base));
}

void launch_vp_lnR(int precision, const VpDevice& d, const double* kv, int nk, const double* qv, int nq, void* tables,
                   double2* zbuf, int rows_per_pass, double* out_re, double* out_im, cudaStream_t st, int npieces) {
    const long long tot = (long long)d.U * (nk + nq);
    const size_t es = precision == SGL_FP64 ? 8 : 4;
    void* e = tables;
    void* Jt = (char*)tables + 2 * es * (size_t)d.U * nk;
    if (precision == SGL_FP64) {
        k_vp_tables<double><<<ceil_div(tot, 256), 256, 0, st>>>(d.ku, d.gu, d.U, kv, nk, qv, nq, (double2*)e, (double2*)Jt);
        SGL_COUNT(1);
    } else {
        k_vp_tables<float><<<ceil_div(tot, 256), 256, 0, st>>>(d.ku, d.gu, d.U, kv, nk, qv, nq, (float2*)e, (float2*)Jt);
        SGL_COUNT(1);
    }
    const size_t chain_smem = (4 * (size_t)kVpNS * kChPts + (size_t)kVpNS * kVpNS) * sizeof(double);
    cudaFuncSetAttribute(k_vp_chain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chain_smem);
    for (int kb = 0; kb < nk; kb += rows_per_pass) {
        const int nkc = nk - kb < rows_per_pass ? nk - kb : rows_per_pass;
        const long long NP = (long long)nkc * nq;
        double2* zp = zbuf;
        double2* al = zbuf + (long long)npieces * d.nsh * kVpNS * NP;
        dim3 g1(ceil_div(nq, kZQ), ceil_div(nkc, kZK), d.nsh * npieces);
        if (precision == SGL_FP64) {
            k_vp_z<double><<<g1, kZThreads, 0, st>>>(d, (const double2*)e, (const double2*)Jt, nk, nq, kb, nkc, zp, al, NP,
                                                     npieces);
            SGL_COUNT(1);
        } else {
            k_vp_z<float><<<g1, kZThreads, 0, st>>>(d, (const float2*)e, (const float2*)Jt, nk, nq, kb, nkc, zp, al, NP,
                                                    npieces);
            SGL_COUNT(1);
        }
        if (NP <= 4LL * kNumSMs) {
            k_vp_chain_small<<<(unsigned)NP, kChSmallThreads, 0, st>>>(d, zp, al, NP, nq, kb, out_re, out_im, npieces);
            SGL_COUNT(1);
        } else {
            k_vp_chain<<<ceil_div(NP, kChPts), kChPts, chain_smem, st>>>(d, zp, al, NP, nq, kb, out_re, out_im, npieces);
            SGL_COUNT(1);
        }
    }
}

}  // namespace sgl
