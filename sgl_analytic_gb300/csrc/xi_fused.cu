// Fused gauss Psi_2 term of the mixed path (reference: Lam._Qxi_gauss, sgl_full.py:2869-2951).
//
// For xi_lin group g and a tile of jt <= 8 coarse k_gamma columns j0 .. j0 + jt - 1, one CTA forms
//   T[p, (jl, rr)] = sum_{entries e of p} rows[rr, e] J_m(gam_{q_e} kg_{j0 + jl})   CUDA cores, FP32
//   Gc[n, (jl, rr)] = sum_p Ec[n, p] T[p, (jl, rr)]                                  tcgen05, TMEM
//   Gs[n, (jl, rr)] = sum_p Es[n, p] T[p, (jl, rr)]
//   part[g, j, n]   = ( sum_rr (a^2 - b^2), sum_rr a b )                              epilogue
// with a = Gc + V (m = 0) or Gc + kg res / 2 (m = 1), b = Gs + kk res (m = 0) or Gs, and
// Ec = cos(kk_n kap_p) (cos - 1 for m = 0 groups), Es = sin(kk_n kap_p).  The k_kappa index n sits
// on the 128 TMEM lanes (nk <= 128), the (jl, rr) pairs on the accumulator columns, so each thread
// of the epilogue holds every row rr of its (n, j) and sums over them without communication.  T and
// G never reach global memory: the unfused form writes and re-reads about 2 GB of them per PDF.
//
// Pipeline (kXfStages shared-memory stages of 64 KB: E 4 x 8 KB [part][cos | sin], T 2 x 16 KB [part]):
//   12 producer warps build the T tile of a 16-p K block from the CSR entries: 3 warps per 4-p block,
//                     lanes over (column half, row) tasks; each block's entries (rows and gamma-cell
//                     indices) stream through its own two shared-memory chunk buffers by bulk copy,
//                     J_m of the CTA's columns is staged once; T is split into TF32 hi + lo and
//                     stored in the canonical K-major layout; fence.proxy.async, one arrival per warp;
//   1 copy thread     brings the packed E block (both parts, both halves) with one bulk copy;
//   1 MMA thread      issues A0 B0 + A0 B1 + A1 B0 (TF32 hi/lo, ~2^-21 per product) into the cos and
//                     sin accumulators (TMEM columns 0 and 256) and commits each stage to its "empty"
//                     barrier.
// The summation order of T over entries and of the squares over rr is that of the unfused kernels.
// The epilogue's correction terms are staged by the producers in the freed chunk buffers.
// Every wait is bounded; a wait that runs out sets *err and the CTA skips to its TMEM release.
#include "kernels.cuh"
#include "tcgen05.cuh"

namespace sgl {

constexpr int kXfStages = 2;
constexpr int kXfABytes = 4 * 8192;                  // E: [part][cos | sin] x 128 lanes x 16 p
constexpr int kXfBPart = 16384;                      // T: 256 columns x 16 p, per part
constexpr int kXfStageBytes = kXfABytes + 2 * kXfBPart;
constexpr int kXfRMax = 48;                          // rows per group (2 r tasks <= producer threads)
constexpr int kXfGroupWarps = 3;                     // producer warps per 4-p block
constexpr int kXfProdWarps = 4 * kXfGroupWarps;
constexpr int kXfProd = kXfProdWarps * 32;
constexpr int kXfThreads = kXfProd + 64;             // + copy warp + MMA warp
constexpr int kXfJt = 8;                             // k_gamma columns per CTA at most
constexpr int kXfChunk = 64;                         // entries per chunk of one warp group, at most
constexpr int kXfRowsCap = 64 * 36;                  // row values per chunk buffer: 64 entries of <= 36 rows,
                                                     // fewer entries per chunk for longer groups
constexpr int kXfSmemStages = kXfStages * kXfStageBytes;
constexpr int kXfRowsBuf = kXfRowsCap * 4 + 64;      // + room for the aligned superset
constexpr int kXfQBuf = kXfChunk * 4 + 64;
constexpr int kXfBlocks = 4;                          // producer warp groups, one per 4-p block of a K block
constexpr int kXfChunkBytes = kXfBlocks * 2 * (kXfRowsBuf + kXfQBuf);
constexpr int kXfSmemFixed = kXfSmemStages + kXfChunkBytes;
static_assert(2 * kXfRMax <= 32 * kXfGroupWarps, "one (row, column half) task per producer lane");
static_assert(kXfRMax * 128 * 8 + kXfRMax * kXfJt * 8 <= kXfChunkBytes, "epilogue tables fit the chunk buffers");
static_assert(kXfRowsCap / kXfRMax >= 4, "a chunk holds a few entries of the longest group");

// entries per chunk for a group of r rows: the chunk's rows fill at most kXfRowsCap values
__host__ __device__ constexpr int xf_chunk_entries(int r) { return r * kXfChunk <= kXfRowsCap ? kXfChunk : kXfRowsCap / r; }


__device__ __forceinline__ int xf_find(const long long* prefix, int ng, long long v) {
    int lo = 0, hi = ng - 1;                          // largest g with prefix[g] <= v
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ float xf_add_ff(float b, float2 hl) {   // round(b + (h + l)) in FP32
    const float s = b + hl.x, bp = s - b;
    const float err = (b - (s - bp)) + (hl.x - bp);
    return s + (err + hl.y);
}

int xi_fused_jt(int r) { return r <= 0 ? 0 : std::min(kXfJt, 256 / r); }

// stages, entry chunks, J_m columns, then the mbarriers, the TMEM address and the failure flag
size_t xi_fused_smem(int n_gmc) { return (size_t)kXfSmemFixed + (size_t)n_gmc * kXfJt * 4 + 8 * (2 * kXfStages + 1 + 2 * kXfBlocks) + 32; }

bool xi_fused_fits(int r_max, int nk, int n_gmc) {
    return nk >= 1 && nk <= 128 && r_max >= 1 && r_max <= kXfRMax && xi_fused_smem(n_gmc) <= 227 * 1024;
}

// Packed E: per group, per 16-p K block, 4 blocks of 128 lanes x 16 p in the canonical layout,
// [part 0 cos][part 0 sin][part 1 cos][part 1 sin].  One CTA per padded p, one thread per lane n;
// lanes n >= nk and p >= nP are zero.  The phase path is that of k_xi_E_ff (float-float k kap,
// exact reduction, half-angle sin / cos).
__global__ void __launch_bounds__(128)
k_xi_E_pack(XiDevice x, const double* __restrict__ kk, int nk, const long long* __restrict__ pp_prefix,
            const long long* __restrict__ p_prefix, const long long* __restrict__ e_off, float* __restrict__ Epk) {
    const long long P = blockIdx.x;
    const int g = xf_find(pp_prefix, x.n_groups, P);
    const int p = (int)(P - pp_prefix[g]);
    const int n = threadIdx.x;
    float ec = 0.f, es = 0.f;
    if (p < x.g_nP[g] && n < nk) {
        const ff kap = ff_from_double(x.kmc[x.idx_p[p_prefix[g] + p]]);
        float s, c, ph_hi, ph_lo;
        halfangle_sincos_ff(ff_from_double(kk[n]), kap, s, c, ph_hi, ph_lo);
        ec = x.g_m[g] == 0 ? -2.f * s * s : (c - s) * (c + s);
        es = 2.f * s * c;
    }
    const int k = p & 15;
    float* base = Epk + e_off[g] + (long long)(p >> 4) * (kXfABytes / 4);
    const int o = (n >> 3) * 128 + (k >> 2) * 32 + (n & 7) * 4 + (k & 3);
    const float ch = tf32_rna(ec), sh = tf32_rna(es);
    base[o] = ch;
    base[2048 + o] = sh;
    base[4096 + o] = tf32_rna(ec - ch);
    base[6144 + o] = tf32_rna(es - sh);
}

struct XiFusedArgs {
    XiDevice x;
    const long long* p_prefix;      // [n_groups + 1] global index of each group's first p
    const long long* rowel_off;     // [n_groups] float offset of each group's rows
    const int* jt;                  // [n_groups] k_gamma columns per CTA
    const long long* cta_prefix;    // [n_groups + 1]
    const long long* e_off;         // [n_groups] packed E offsets (floats)
    const float* Epk;
    const float* J;                 // FP32 Bessel tables [4][n_gmc][nkg]
    const float* Vf;                // [rows][nkg]  U (J0 - 1), m = 0 rows
    const float2* kresT;            // [rows][nk]   kk_n res_R as float-float
    const float2* hq;               // [rows][nkg]  kg_j res_R / 2 as float-float
    int nk, nkg;
    float2* part;                   // [n_groups][nkg][nk]
    int* err;
};

// one entry chunk of a warp group: entries [ea, eb) of its 4-p block in K block kb, at most
// xf_chunk_entries(r)
struct XfChunk { int kb, ea, eb; };

__global__ void __launch_bounds__(kXfThreads, 1)
k_xi_fused(XiFusedArgs a) {
    extern __shared__ __align__(1024) unsigned char xsm[];
    const XiDevice& x = a.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long cta = blockIdx.x;
    const int g = xf_find(a.cta_prefix, x.n_groups, cta);
    const int jt = a.jt[g];
    const int j0 = (int)(cta - a.cta_prefix[g]) * jt;
    const int r = x.g_r[g], m = x.g_m[g], nP = x.g_nP[g];
    const int N = ((jt * r + 15) / 16) * 16;            // MMA N (<= 256)
    const int nkb = (nP + 15) / 16;
    const int nk = a.nk, nkg = a.nkg, n_gmc = x.n_gmc;
    float* s_J = (float*)(xsm + kXfSmemFixed);                           // [n_gmc][8]
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(xsm);
    const uint32_t boff = kXfSmemFixed + n_gmc * kXfJt * 4;
    const uint32_t bar = sbase + boff;                   // full[S], empty[S], done, chunk[groups][2]
    constexpr int kNBar = 2 * kXfStages + 1 + 2 * kXfBlocks;
    const uint32_t tslot = bar + 8 * kNBar;
    volatile int* s_fail = (volatile int*)(xsm + boff + 8 * kNBar + 8);
    auto full = [&](int s) { return bar + 8 * s; };
    auto empty = [&](int s) { return bar + 8 * (kXfStages + s); };
    const uint32_t done = bar + 8 * (2 * kXfStages);
    auto cbar = [&](int pr, int b) { return bar + 8 * (2 * kXfStages + 1 + 2 * pr + b); };

    if (warp == kXfProdWarps + 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(tslot), "r"(512) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kXfStages; ++s) {
            mbar_init(full(s), kXfProdWarps + 1);
            mbar_init(empty(s), 1);
        }
        mbar_init(done, 1);
        for (int b = 0; b < 2 * kXfBlocks; ++b) mbar_init(cbar(b >> 1, b & 1), 1);
        *s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    {
        const float* Jm = a.J + (long long)m * n_gmc * nkg;
        for (int i = tid; i < n_gmc * kXfJt; i += kXfThreads) {
            const int q = i / kXfJt, jl = i % kXfJt, j = j0 + jl;
            s_J[i] = (jl < jt && j < nkg) ? Jm[(long long)q * nkg + j] : 0.f;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *(volatile uint32_t*)(xsm + boff + 8 * kNBar);

    if (warp < kXfProdWarps && nkb > 0) {
        // ---- T producers: warp group pb (kXfGroupWarps warps) owns p = 16 kb + 4 pb .. + 3 of every
        // K block; its lanes take the tasks (column half jh, row rr), t = jh r + rr < 2 r.  The group
        // streams its own entries (CSR by p: one contiguous run per K block) through its own two chunk
        // buffers: lane 0 of the group's first warp brings a chunk's rows and gamma-cell indices with
        // two bulk copies of their 16-byte-aligned supersets, one chunk ahead of the one being summed.
        // The groups run independently; the full barrier of a stage collects one arrival per warp.
        const long long gp0 = a.p_prefix[g], ent0 = x.g_ent_off[g];
        const float* rowsg = x.rows_f + a.rowel_off[g];
        const int* pptr = x.p_ptr + gp0;
        const int pb = warp / kXfGroupWarps, sub = warp % kXfGroupWarps;
        const int t = sub * 32 + lane;
        const bool active = t < 2 * r;
        const int jh = active ? t / r : 0, rr = active ? t - jh * r : 0;
        const bool issuer = sub == 0 && lane == 0;
        float* const rbuf0 = (float*)(xsm + kXfSmemStages + (pb * 2) * kXfRowsBuf);
        int* const qbuf0 = (int*)(xsm + kXfSmemStages + 2 * kXfBlocks * kXfRowsBuf + (pb * 2) * kXfQBuf);
        auto lo_of = [&](int kb) { return pptr[min(16 * kb + 4 * pb, nP)]; };
        auto hi_of = [&](int kb) { return pptr[min(16 * kb + 4 * pb + 4, nP)]; };
        auto rows_at = [&](int e) { return rowsg + (long long)(e - ent0) * r; };
        auto issue = [&](XfChunk c, int buf) {          // issuer lane only
            const uint32_t cb = cbar(pb, buf);
            if (c.eb == c.ea) { mbar_arrive(cb); return; }
            const uintptr_t r0 = (uintptr_t)rows_at(c.ea), r1 = (uintptr_t)rows_at(c.eb);
            const uintptr_t q0 = (uintptr_t)(x.ent_qg + c.ea), q1 = (uintptr_t)(x.ent_qg + c.eb);
            const uintptr_t r0a = r0 & ~(uintptr_t)15, q0a = q0 & ~(uintptr_t)15;
            const uint32_t rb = (uint32_t)(((r1 + 15) & ~(uintptr_t)15) - r0a);
            const uint32_t qb = (uint32_t)(((q1 + 15) & ~(uintptr_t)15) - q0a);
            mbar_expect_tx(cb, rb + qb);
            bulk_g2s((uint32_t)__cvta_generic_to_shared(rbuf0) + buf * kXfRowsBuf, (const void*)r0a, rb, cb);
            bulk_g2s((uint32_t)__cvta_generic_to_shared(qbuf0) + buf * kXfQBuf, (const void*)q0a, qb, cb);
        };
        const int chunk = xf_chunk_entries(r);
        XfChunk cur{0, lo_of(0), 0};
        int cur_hi = hi_of(0);
        cur.eb = min(cur.ea + chunk, cur_hi);
        if (issuer) issue(cur, 0);
        int ci = 0, issued = 0;                         // chunk counters: buffer ci & 1, parity (ci >> 1) & 1
        float acc[4][4];                                // [p of the block][column of the half]
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < 4; ++w) acc[u][w] = 0.f;
        int pbnd[5];
#pragma unroll
        for (int u = 0; u < 5; ++u) pbnd[u] = pptr[min(4 * pb + u, nP)];
        bool failed = false;
        while (cur.kb < nkb) {
            // group barrier (the buffer of the previous chunk is free) that also ORs the warps'
            // failure flags, so that they leave the loop together
            int any_fail;
            asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.b32 p, %1, 0;\n\t"
                         "bar.red.or.pred q, %2, %3, p;\n\tselp.b32 %0, 1, 0, q;\n\t}\n"
                         : "=r"(any_fail) : "r"((failed || *s_fail) ? 1 : 0), "r"(1 + pb), "r"(32 * kXfGroupWarps)
                         : "memory");
            if (any_fail) break;
            XfChunk nxt;
            int nxt_hi = cur_hi;
            if (cur.eb < cur_hi) {
                nxt.kb = cur.kb; nxt.ea = cur.eb;
            } else {
                nxt.kb = cur.kb + 1;
                nxt.ea = nxt.kb < nkb ? lo_of(nxt.kb) : 0;
                nxt_hi = nxt.kb < nkb ? hi_of(nxt.kb) : 0;
            }
            nxt.eb = nxt.kb < nkb ? min(nxt.ea + chunk, nxt_hi) : nxt.ea;
            if (nxt.kb < nkb) {
                if (issuer) issue(nxt, (ci + 1) & 1);
                issued = ci + 1;
            }
            const int b = ci & 1;
            if (!mbar_wait_sleep(cbar(pb, b), (uint32_t)((ci >> 1) & 1))) failed = true;
            if (!failed && cur.eb > cur.ea && active) {
                const int rlead = (int)(((uintptr_t)rows_at(cur.ea) & 15) >> 2);
                const int qlead = (int)(((uintptr_t)(x.ent_qg + cur.ea) & 15) >> 2);
                const float* sr = rbuf0 + b * (kXfRowsBuf / 4) + rlead + rr;
                const int* sq = qbuf0 + b * (kXfQBuf / 4) + qlead;
                const float* sj = s_J + 4 * jh;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e_lo = max(pbnd[u], cur.ea) - cur.ea, e_hi = min(pbnd[u + 1], cur.eb) - cur.ea;
                    int e = e_lo;
                    // four entries per step, their loads issued ahead of the FMAs (entry order kept)
                    for (; e + 3 < e_hi; e += 4) {
                        float4 jv[4];
                        float v[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            jv[k] = *(const float4*)(sj + sq[e + k] * kXfJt);
                            v[k] = sr[(e + k) * r];
                        }
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            acc[u][0] = fmaf(v[k], jv[k].x, acc[u][0]);
                            acc[u][1] = fmaf(v[k], jv[k].y, acc[u][1]);
                            acc[u][2] = fmaf(v[k], jv[k].z, acc[u][2]);
                            acc[u][3] = fmaf(v[k], jv[k].w, acc[u][3]);
                        }
                    }
                    for (; e < e_hi; ++e) {
                        const float4 j0 = *(const float4*)(sj + sq[e] * kXfJt);
                        const float v0 = sr[e * r];
                        acc[u][0] = fmaf(v0, j0.x, acc[u][0]);
                        acc[u][1] = fmaf(v0, j0.y, acc[u][1]);
                        acc[u][2] = fmaf(v0, j0.z, acc[u][2]);
                        acc[u][3] = fmaf(v0, j0.w, acc[u][3]);
                    }
                }
            }
            if (nxt.kb != cur.kb) {
                // the group's share of K block kb is complete: its stage must have been consumed by the
                // MMAs of kb - S
                const int kb = cur.kb, s = kb % kXfStages;
                if (kb >= kXfStages && !mbar_wait_sleep(empty(s), (uint32_t)(((kb / kXfStages) - 1) & 1)))
                    failed = true;                      // acted on at the next barrier
                float* Bst = (float*)(xsm + s * kXfStageBytes + kXfABytes);
                // column c = jl r + rr, K index 4 pb + u: one float4 (hi) + one (lo) per (row, column)
                auto put = [&](const float (&av)[4][4], int rr) {
#pragma unroll
                    for (int w = 0; w < 4; ++w) {
                        const int jl = 4 * jh + w;
                        if (jl < jt) {
                            const int c = jl * r + rr;
                            float hv[4], lv[4];
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                hv[u] = tf32_rna(av[u][w]);
                                lv[u] = tf32_rna(av[u][w] - hv[u]);
                            }
                            const int o = (c >> 3) * 128 + pb * 32 + (c & 7) * 4;
                            *(float4*)(Bst + o) = make_float4(hv[0], hv[1], hv[2], hv[3]);
                            *(float4*)(Bst + kXfBPart / 4 + o) = make_float4(lv[0], lv[1], lv[2], lv[3]);
                        }
                    }
                };
                if (active) put(acc, rr);
                fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(full(s));
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int w = 0; w < 4; ++w) acc[u][w] = 0.f;
                if (nxt.kb < nkb) {
#pragma unroll
                    for (int u = 0; u < 5; ++u) pbnd[u] = pptr[min(16 * nxt.kb + 4 * pb + u, nP)];
                }
            }
            cur = nxt;
            cur_hi = nxt_hi;
            ++ci;
        }
        // no bulk copy outlives the loop: the issuer waits (bounded) for any chunk it issued that was
        // not consumed (only after a failure)
        if (issuer)
            for (int c = ci; c <= issued; ++c) mbar_wait_sleep(cbar(pb, c & 1), (uint32_t)((c >> 1) & 1));
        if (failed) *s_fail = 1;
    } else if (warp == kXfProdWarps && lane == 0) {
        // ---- E: one bulk copy per K block (both parts, cos and sin halves)
        const float* Eg = a.Epk + a.e_off[g];
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kXfStages;
            if (kb >= kXfStages && (*s_fail || !mbar_wait_sleep(empty(s), (uint32_t)(((kb / kXfStages) - 1) & 1)))) {
                *s_fail = 1;
                break;
            }
            mbar_expect_tx(full(s), kXfABytes);
            bulk_g2s(sbase + s * kXfStageBytes, Eg + (long long)kb * (kXfABytes / 4), kXfABytes, full(s));
        }
    } else if (warp == kXfProdWarps + 1 && lane == 0 && nkb > 0) {
        // ---- MMA issuer: cos accumulator at TMEM column 0, sin at column 256
        constexpr int PA[3] = {0, 0, 1};
        constexpr int PB[3] = {0, 1, 0};
        const uint32_t idesc = tc_idesc_tf32(kTcBM, N);
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kXfStages;
            if (*s_fail || !mbar_wait_sleep(full(s), (uint32_t)((kb / kXfStages) & 1))) { *s_fail = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = sbase + s * kXfStageBytes, b0 = a0 + kXfABytes;
#pragma unroll
            for (int ks = 0; ks < 2; ++ks) {
                const uint32_t o = ks * 2 * kTcLBO;
#pragma unroll
                for (int trig = 0; trig < 2; ++trig)
#pragma unroll
                    for (int t = 0; t < 3; ++t)
                        tc_mma(tmem + 256u * trig, tc_desc(a0 + (PA[t] * 2 + trig) * 8192 + o),
                               tc_desc(b0 + PB[t] * kXfBPart + o), idesc, (kb | ks | t) ? 1u : 0u);
            }
            tc_commit(empty(s));
        }
        tc_commit(done);
    }

    // ---- epilogue.  Once every producer warp is done the chunk buffers are free: the producers
    // stage there the square's correction terms for this CTA's rows and columns while the last
    // MMAs run.
    const long long R0 = x.g_row_off[g];
    float2* s_kres = (float2*)(xsm + kXfSmemStages);                       // [r][128]  kk_n res (m = 0)
    float2* s_cor = (float2*)(xsm + kXfSmemStages + kXfRMax * 128 * 8);   // [r][8]    (V, 0) m = 0 / hq m = 1
    if (warp < kXfProdWarps) {
        asm volatile("bar.sync 5, %0;" :: "r"(kXfProd) : "memory");
        for (int i = tid; i < r * 128; i += kXfProd) {
            const int rq = i >> 7, n = i & 127;
            s_kres[i] = (m == 0 && n < nk) ? a.kresT[(R0 + rq) * nk + n] : make_float2(0.f, 0.f);
        }
        for (int i = tid; i < r * kXfJt; i += kXfProd) {
            const int rq = i / kXfJt, jl = i % kXfJt, j = j0 + jl;
            float2 v = make_float2(0.f, 0.f);
            if (jl < jt && j < nkg) {
                if (m == 0) v.x = a.Vf[(R0 + rq) * nkg + j];
                else if (m == 1) v = a.hq[(R0 + rq) * nkg + j];
            }
            s_cor[i] = v;
        }
    }
    bool ok = true;
    if (nkb > 0) ok = mbar_wait_sleep(done, 0u);
    const int all_ok = __syncthreads_and((ok && !*s_fail) ? 1 : 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (all_ok) {
        if (warp < kXfProdWarps) {
            // warp w reads TMEM lanes 32 (w % 4) .. + 31 (k_kappa index n) and the column part w / 4
            // (of kXfGroupWarps) of the (jl, rr) pairs; the rows rr of one (n, j) are summed in registers
            const int quad = warp & 3, part_ = warp >> 2;
            const int n = quad * 32 + lane;
            const int jl_lo = (jt * part_) / kXfGroupWarps, jl_hi = (jt * (part_ + 1)) / kXfGroupWarps;
            const int c_lo = jl_lo * r, c_hi = jl_hi * r;
            int jl = jl_lo, rr = 0;
            float gre = 0.f, gim = 0.f;
            const uint32_t lane_base = tmem + ((uint32_t)(quad * 32) << 16);
            for (int c0 = c_lo & ~15; c0 < c_hi; c0 += 16) {
                float vc[16], vs[16];
                if (nkb > 0) {
                    tmem_ld16x2(lane_base + (uint32_t)c0, lane_base + 256u + (uint32_t)c0, vc, vs);
                } else {
#pragma unroll
                    for (int q = 0; q < 16; ++q) { vc[q] = 0.f; vs[q] = 0.f; }
                }
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int c = c0 + q;
                    if (c < c_lo || c >= c_hi) continue;
                    float av = vc[q], bv = vs[q];
                    const float2 cor = s_cor[rr * kXfJt + jl];
                    if (m == 0) {
                        av += cor.x;
                        bv = xf_add_ff(bv, s_kres[rr * 128 + n]);
                    } else if (m == 1) {
                        av = xf_add_ff(av, cor);
                    }
                    gre = fmaf(av, av, fmaf(-bv, bv, gre));
                    gim = fmaf(av, bv, gim);
                    if (++rr == r) {
                        const int j = j0 + jl;
                        if (n < nk && j < nkg) a.part[((long long)g * nkg + j) * nk + n] = make_float2(gre, gim);
                        rr = 0;
                        ++jl;
                        gre = 0.f;
                        gim = 0.f;
                    }
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(a.err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == kXfProdWarps + 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(512) : "memory");
    }
}

// out(n, j) = sum_g sign_g / 2 (sum_rr (a^2 - b^2)) + i sign_g sum_rr a b, groups in order, FP64
__global__ void k_xi_fused_sum(const float2* __restrict__ part, const int* __restrict__ g_m, int n_groups, int nk,
                               int nkg, double* __restrict__ out_re, double* __restrict__ out_im) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nk * nkg) return;
    const int j = (int)(e / nk), n = (int)(e % nk);
    const long long stride = (long long)nkg * nk;
    const float2* pp = part + (long long)j * nk + n;
    double re = 0.0, im = 0.0;
    auto add = [&](int m, float2 v) {
        const double sign = (m == 0) ? 1.0 : ((m & 1) ? -2.0 : 2.0);
        re = fma(0.5 * sign, (double)v.x, re);
        im = fma(0.5 * sign, 2.0 * (double)v.y, im);
    };
    int g = 0;
    for (; g + 8 <= n_groups; g += 8) {            // eight loads in flight, summed in group order
        float2 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = pp[(long long)(g + k) * stride];
#pragma unroll
        for (int k = 0; k < 8; ++k) add(g_m[g + k], v[k]);
    }
    for (; g < n_groups; ++g) add(g_m[g], pp[(long long)g * stride]);
    out_re[(long long)n * nkg + j] = re;
    out_im[(long long)n * nkg + j] = im;
}

void launch_xi_E_pack(const XiDevice& x, const double* kk, int nk, const long long* pp_prefix, long long total_pp,
                      const long long* p_prefix, const long long* e_off, float* Epk, cudaStream_t st) {
    if (total_pp <= 0) return;
    k_xi_E_pack<<<(unsigned)total_pp, 128, 0, st>>>(x, kk, nk, pp_prefix, p_prefix, e_off, Epk);
    SGL_COUNT(1);
}

void launch_xi_fused(const XiDevice& x, const long long* p_prefix, const long long* rowel_off, const int* jt,
                     const long long* cta_prefix, long long ctas, const long long* e_off, const float* Epk,
                     const float* J, const float* Vf, const float2* kresT, const float2* hq, int nk, int nkg,
                     float2* part, int* err, double* out_re, double* out_im, cudaStream_t st) {
    if (ctas > 0) {
        XiFusedArgs a{x, p_prefix, rowel_off, jt, cta_prefix, e_off, Epk, J, Vf, kresT, hq, nk, nkg, part, err};
        const size_t sm = xi_fused_smem(x.n_gmc);
        cudaFuncSetAttribute(k_xi_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_xi_fused<<<(unsigned)ctas, kXfThreads, sm, st>>>(a);
        SGL_COUNT(1);
    }
    const long long tot = (long long)nk * nkg;
    k_xi_fused_sum<<<ceil_div(tot, 256), 256, 0, st>>>(part, x.g_m, x.n_groups, nk, nkg, out_re, out_im);
    SGL_COUNT(1);
}

}  // namespace sgl
