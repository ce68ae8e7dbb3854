// Grouped FP32 GEMM on the 5th-generation tensor cores (tcgen05), at FP32-level accuracy:
//   C(i, j) = sum_k A(i, k) B(k, j)
//
// Operands are first PACKED (k_tc_pack): every element is split into NP TF32 parts
// t0 = rna(x), t1 = rna(x - t0) (, t2 = rna(x - t0 - t1)) and written in the tensor core's
// canonical K-major no-swizzle layout, K in blocks of 16:
//   packed[kb][part][row][16 k]  with  row-group stride 512 B (8 rows) and K-chunk stride 128 B
//   (core matrices of 8 rows x 16 bytes),
// so the 16 K-columns of any 8-row-aligned run of rows are one contiguous span in global memory.
// The GEMM (k_tc_gemm) then moves each operand tile with one bulk copy per part
// (cp.async.bulk ... mbarrier::complete_tx::bytes: the TMA engine, no register staging) through a
// shared-memory ring (4 stages for NP = 2, 3 for NP = 3); one thread produces (copies), one thread
// issues the part products into an FP32 accumulator in tensor memory (128 lanes x bn columns):
//   NP = 2:  A0 B0 + A0 B1 + A1 B0                         (3 tcgen05.mma.kind::tf32 per K-step)
//            operands carried to ~22 bits: product error ~2^-21
//   NP = 3:  A0 B0 + A0 B1 + A1 B0 + A0 B2 + A2 B0 + A1 B1  (6 per K-step)
//            FP32 operands carried exactly (3 x 11 bits): product error ~2^-32
// and commits each stage's MMAs to that stage's "empty" mbarrier; the epilogue (4 warps, warp w owns
// TMEM lanes 32w..32w+31) reads TMEM with tcgen05.ld and stores alpha * C with arbitrary strides.
// Accumulation is FP32 in TMEM; callers bound its length by splitting K.
//
// BF16 mode (NP = 1, BF = true; the surrogate MLP): operands rounded to BF16 and packed in the same
// byte layout (a 16-byte core-matrix row holds 8 BF16 values, a 64-byte K block 32 of them), one
// tcgen05.mma.kind::f16 (BF16 inputs, FP32 accumulation) per K-step of 16.
//
// Every mbarrier wait is bounded (~2 s); a wait that runs out raises *err, the CTA skips the rest
// of its work, waits (bounded) for its own MMAs and frees its TMEM before returning.
#include <cuda_bf16.h>

#include "kernels.cuh"
#include "tcgen05.cuh"

namespace sgl {

template <int NP> struct TcCfg {
    static constexpr int kStages = NP == 3 ? 3 : 4;
    static constexpr int kStageBytes = NP * (kTcAbytes + kTcBbytes);      // 48 / 72 KB
    static constexpr int kBarOff = kStages * kStageBytes;                  // mbarriers after the ring
    static constexpr int kSmem = kBarOff + 128;
};

// ------------------------------------------------------------------ packing
// One thread per (row, 4 consecutive k): reads X(r, k..k+3), writes the NP float4 rows of its core
// matrix.  Rows >= R and k >= K are zero.
template <int NP>
__global__ void __launch_bounds__(256)
k_tc_pack(const TcPackDesc* __restrict__ descs, int nprob, float* __restrict__ base) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (descs[mid].quad_begin <= t) lo = mid; else hi = mid - 1;
    }
    const TcPackDesc d = descs[lo];
    const long long q = t - d.quad_begin;
    const long long nq = (long long)d.Rpad * d.nkb * 4;
    if (q < 0 || q >= nq) return;
    // quads ordered (kb, chunk, row): consecutive threads take consecutive rows
    const int r = (int)(q % d.Rpad);
    const long long rest = q / d.Rpad;
    const int c = (int)(rest % 4), kb = (int)(rest / 4);
    float part[NP][4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int k = kb * kTcBK + c * 4 + e;
        float v = (r < d.R && k < d.K) ? __ldg(d.X + (long long)r * d.x_rs + (long long)k * d.x_cs) : 0.f;
#pragma unroll
        for (int pp = 0; pp < NP; ++pp) {
            const float tv = tf32_rna(v);
            part[pp][e] = tv;
            v -= tv;
        }
    }
    float* out = base + d.out_off;
    const long long o = (long long)(r >> 3) * 128 + c * 32 + (r & 7) * 4;     // floats
    const long long pstride = (long long)d.Rpad * kTcBK;                       // floats per (kb, part)
#pragma unroll
    for (int pp = 0; pp < NP; ++pp)
        *(float4*)(out + ((long long)NP * kb + pp) * pstride + o) = make_float4(part[pp][0], part[pp][1], part[pp][2], part[pp][3]);
}

// BF16 packing: one thread per (row, 8 consecutive k) -> one 16-byte core-matrix row (K block = 32)
__global__ void __launch_bounds__(256)
k_tc_pack_bf16(const TcPackDesc* __restrict__ descs, int nprob, float* __restrict__ base) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (descs[mid].quad_begin <= t) lo = mid; else hi = mid - 1;
    }
    const TcPackDesc d = descs[lo];
    const long long q = t - d.quad_begin;
    const long long nq = (long long)d.Rpad * d.nkb * 4;
    if (q < 0 || q >= nq) return;
    const int r = (int)(q % d.Rpad);
    const long long rest = q / d.Rpad;
    const int c = (int)(rest % 4), kb = (int)(rest / 4);
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int k = kb * 32 + c * 8 + 2 * e;
        const float v0 = (r < d.R && k < d.K) ? __ldg(d.X + (long long)r * d.x_rs + (long long)k * d.x_cs) : 0.f;
        const float v1 = (r < d.R && k + 1 < d.K) ? __ldg(d.X + (long long)r * d.x_rs + (long long)(k + 1) * d.x_cs) : 0.f;
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(v0, v1);
        w[e] = *(const uint32_t*)&b2;
    }
    unsigned char* out = (unsigned char*)(base + d.out_off);
    const long long o = (long long)(r >> 3) * 512 + c * 128 + (r & 7) * 16;        // bytes
    *(uint4*)(out + (long long)kb * d.Rpad * 64 + o) = make_uint4(w[0], w[1], w[2], w[3]);
}

// ------------------------------------------------------------------ GEMM
template <int NP>
__global__ void __launch_bounds__(kTcThreads, 1)
k_tc_gemm(const TcGemmDesc* __restrict__ descs, int nprob, const float* __restrict__ packed, int* __restrict__ err) {
    using Cfg = TcCfg<NP>;
    constexpr int S = Cfg::kStages;
    extern __shared__ __align__(1024) unsigned char tsm[];
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(tsm);
    const uint32_t bar = sbase + Cfg::kBarOff;          // full[S], empty[S], done
    const uint32_t tslot = bar + 72;
    volatile int* s_fail = (volatile int*)(tsm + Cfg::kBarOff + 80);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    const int tile = blockIdx.x;
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (descs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
    }
    const TcGemmDesc d = descs[lo];
    const int local = tile - d.tile_begin;
    const int i0 = (local / d.tiles_n) * kTcBM, bn = d.bn, j0 = (local % d.tiles_n) * bn;
    constexpr int KB = NP == 1 ? 2 * kTcBK : kTcBK;      // elements per 64-byte K block
    const int nkb = (d.K + KB - 1) / KB;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(tslot), "r"(kTcBNmax) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < 2 * S + 1; ++s) mbar_init(bar + 8 * s, 1);
        *s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *(volatile uint32_t*)(tsm + Cfg::kBarOff + 72);

    const float* Ap = packed + d.a_off;       // [nkb][NP][Mpad][16]
    const float* Bp = packed + d.b_off;       // [nkb][NP][Npad][16]
    const long long a_part = (long long)d.Mpad * kTcBK, b_part = (long long)d.Npad * kTcBK;
    const uint32_t a_bytes = kTcAbytes, b_bytes = (uint32_t)bn * kTcBK * 4;

    if (tid == 0 && nkb > 0) {
        // producer: one bulk copy per operand part and K block
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % S;
            if (kb >= S && !mbar_wait_bounded(bar + 8 * (S + s), (uint32_t)(((kb / S) - 1) & 1))) {
                *s_fail = 1;
                break;
            }
            const uint32_t st = sbase + s * Cfg::kStageBytes;
            mbar_expect_tx(bar + 8 * s, NP * (a_bytes + b_bytes));
            const float* a = Ap + ((long long)NP * kb) * a_part + (long long)(i0 >> 3) * 128;
            const float* b = Bp + ((long long)NP * kb) * b_part + (long long)(j0 >> 3) * 128;
#pragma unroll
            for (int pp = 0; pp < NP; ++pp) {
                bulk_g2s(st + pp * kTcAbytes, a + pp * a_part, a_bytes, bar + 8 * s);
                bulk_g2s(st + NP * kTcAbytes + pp * kTcBbytes, b + pp * b_part, b_bytes, bar + 8 * s);
            }
        }
    } else if (tid == 32 && nkb > 0) {
        // MMA issuer: part products, larger terms first (NP = 1: BF16, one product)
        constexpr int NPROD = NP == 1 ? 1 : (NP == 2 ? 3 : 6);
        constexpr int PA[6] = {0, 0, 1, 0, 2, 1};
        constexpr int PB[6] = {0, 1, 0, 2, 0, 1};
        const uint32_t idesc = NP == 1 ? tc_idesc_bf16(kTcBM, bn) : tc_idesc_tf32(kTcBM, bn);
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % S;
            if (*s_fail || !mbar_wait_bounded(bar + 8 * s, (uint32_t)((kb / S) & 1))) { *s_fail = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = sbase + s * Cfg::kStageBytes, b0 = a0 + NP * kTcAbytes;
#pragma unroll
            for (int ks = 0; ks < kTcBK / 8; ++ks) {
                const uint32_t o = ks * 2 * kTcLBO;
#pragma unroll
                for (int t = 0; t < NPROD; ++t) {
                    if constexpr (NP == 1)
                        tc_mma_bf16(tmem, tc_desc(a0 + o), tc_desc(b0 + o), idesc, (kb | ks) ? 1u : 0u);
                    else
                        tc_mma(tmem, tc_desc(a0 + PA[t] * kTcAbytes + o), tc_desc(b0 + PB[t] * kTcBbytes + o), idesc,
                               (kb | ks | t) ? 1u : 0u);
                }
            }
            tc_commit(bar + 8 * (S + s));
        }
        tc_commit(bar + 8 * (2 * S));    // "done": every MMA issued above has completed
    }
    // epilogue: all threads wait for the done barrier (bounded), then read TMEM
    bool ok = true;
    if (nkb > 0) ok = mbar_wait_bounded(bar + 8 * (2 * S), 0u);
    const int all_ok = __syncthreads_and((ok && !*s_fail) ? 1 : 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = warp * 32 + lane, gi = i0 + row;
    if (all_ok) {
        for (int c0 = 0; c0 < bn; c0 += 16) {
            float v[16];
            if (nkb > 0) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            else {
#pragma unroll
                for (int q = 0; q < 16; ++q) v[q] = 0.f;
            }
            if (gi < d.M) {
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int gj = j0 + c0 + q;
                    if (gj < d.N) d.C[(long long)gi * d.c_rs + (long long)gj * d.c_cs] = d.alpha * v[q];
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kTcBNmax) : "memory");
    }
}

// ------------------------------------------------------------------ drained accumulation
// The same packed operands and ring, N tiles of at most kTcDrainBN columns, and the accumulation
// drained out of TMEM every kTcDrainKB K blocks: the MMAs of drain block b accumulate into one of
// two TMEM accumulators (b & 1), the first MMA of the block starting it from zero, while the four
// epilogue warps read the other accumulator (the previous block) with tcgen05.ld and add it to
// FP32 running sums in registers by Knuth's TwoSum (hi + lo per output).  The tensor core's FP32
// accumulation then runs over kTcDrainKB x 16 products only, from zero each time; its rounding
// (which, unlike an FMA chain's, is not round-to-nearest) does not build up over the whole K, and
// the running sums carry the block totals with their exact rounding errors.
// Warps 0-3: epilogue (TMEM lanes 32w .. 32w + 31 = tile rows); warp 4 lane 0: bulk copies;
// warp 5 lane 0: MMAs.  Every wait is bounded; a wait that runs out raises *err and the CTA frees
// its TMEM and returns.
constexpr int kTcDrainBN = 64;
constexpr int kTcDrainKB = 4;                  // K blocks of 16 per drain
constexpr int kTcDrainThreads = 192;

template <int NP> struct TcDrainCfg {
    static constexpr int kStages = NP == 3 ? 4 : 6;
    static constexpr int kABytes = kTcAbytes;                          // 128 x 16 TF32 per part
    static constexpr int kBBytes = kTcDrainBN * kTcBK * 4;              // 64 x 16 TF32 per part
    static constexpr int kStageBytes = NP * (kABytes + kBBytes);       // 36 / 24 KB
    static constexpr int kBarOff = kStages * kStageBytes;
    static constexpr int kNBar = 2 * kStages + 5;                      // full, empty, acc full[2], acc empty[2], done
    static constexpr int kSmem = kBarOff + 8 * kNBar + 32;
};

template <int NP>
__global__ void __launch_bounds__(kTcDrainThreads, 1)
k_tc_gemm_drain(const TcGemmDesc* __restrict__ descs, int nprob, const float* __restrict__ packed, int* __restrict__ err) {
    using Cfg = TcDrainCfg<NP>;
    constexpr int S = Cfg::kStages;
    extern __shared__ __align__(1024) unsigned char tsm[];
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(tsm);
    const uint32_t bar = sbase + Cfg::kBarOff;
    auto full = [&](int s) { return bar + 8 * s; };
    auto empty = [&](int s) { return bar + 8 * (S + s); };
    auto accf = [&](int a) { return bar + 8 * (2 * S + a); };
    auto acce = [&](int a) { return bar + 8 * (2 * S + 2 + a); };
    const uint32_t done = bar + 8 * (2 * S + 4);
    const uint32_t tslot = bar + 8 * Cfg::kNBar;
    volatile int* s_fail = (volatile int*)(tsm + Cfg::kBarOff + 8 * Cfg::kNBar + 8);
    volatile int* s_used = (volatile int*)(tsm + Cfg::kBarOff + 8 * Cfg::kNBar + 12);   // K blocks the MMAs took
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    const int tile = blockIdx.x;
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (descs[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
    }
    const TcGemmDesc d = descs[lo];
    const int local = tile - d.tile_begin;
    const int i0 = (local / d.tiles_n) * kTcBM, bn = d.bn, j0 = (local % d.tiles_n) * bn;
    const int nkb = (d.K + kTcBK - 1) / kTcBK;
    const int nblk = (nkb + kTcDrainKB - 1) / kTcDrainKB;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(tslot), "r"(2 * kTcDrainBN) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < S; ++s) { mbar_init(full(s), 1); mbar_init(empty(s), 1); }
        for (int a = 0; a < 2; ++a) { mbar_init(accf(a), 1); mbar_init(acce(a), 4); }
        mbar_init(done, 1);
        *s_fail = 0;
        *s_used = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *(volatile uint32_t*)(tsm + Cfg::kBarOff + 8 * Cfg::kNBar);

    const float* Ap = packed + d.a_off;       // [nkb][NP][Mpad][16]
    const float* Bp = packed + d.b_off;       // [nkb][NP][Npad][16]
    const long long a_part = (long long)d.Mpad * kTcBK, b_part = (long long)d.Npad * kTcBK;
    const uint32_t a_bytes = Cfg::kABytes, b_bytes = (uint32_t)bn * kTcBK * 4;

    int issued = 0;                            // K blocks whose copies the producer issued
    if (warp == 4) {
        if (lane == 0) {
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = kb % S;
                if (*s_fail || (kb >= S && !mbar_wait_bounded(empty(s), (uint32_t)(((kb / S) - 1) & 1)))) {
                    *s_fail = 1;
                    break;
                }
                issued = kb + 1;
                const uint32_t st = sbase + s * Cfg::kStageBytes;
                mbar_expect_tx(full(s), NP * (a_bytes + b_bytes));
                const float* a = Ap + ((long long)NP * kb) * a_part + (long long)(i0 >> 3) * 128;
                const float* b = Bp + ((long long)NP * kb) * b_part + (long long)(j0 >> 3) * 128;
#pragma unroll
                for (int pp = 0; pp < NP; ++pp) {
                    bulk_g2s(st + pp * Cfg::kABytes, a + pp * a_part, a_bytes, full(s));
                    bulk_g2s(st + NP * Cfg::kABytes + pp * Cfg::kBBytes, b + pp * b_part, b_bytes, full(s));
                }
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            constexpr int NPROD = NP == 2 ? 3 : 6;
            constexpr int PA[6] = {0, 0, 1, 0, 2, 1};
            constexpr int PB[6] = {0, 1, 0, 2, 0, 1};
            const uint32_t idesc = tc_idesc_tf32(kTcBM, bn);
            for (int kb = 0; kb < nkb; ++kb) {
                const int blk = kb / kTcDrainKB, a = blk & 1;
                const bool first = kb % kTcDrainKB == 0;
                // the accumulator of block blk was drained (block blk - 2) before its first MMA
                if (first && blk >= 2 && (*s_fail || !mbar_wait_bounded(acce(a), (uint32_t)(((blk >> 1) - 1) & 1)))) {
                    *s_fail = 1;
                    break;
                }
                const int s = kb % S;
                if (*s_fail || !mbar_wait_bounded(full(s), (uint32_t)((kb / S) & 1))) { *s_fail = 1; break; }
                *s_used = kb + 1;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = sbase + s * Cfg::kStageBytes, b0 = a0 + NP * Cfg::kABytes;
                const uint32_t acc = tmem + (uint32_t)(a * kTcDrainBN);
#pragma unroll
                for (int ks = 0; ks < kTcBK / 8; ++ks) {
                    const uint32_t o = ks * 2 * kTcLBO;
#pragma unroll
                    for (int t = 0; t < NPROD; ++t)
                        tc_mma(acc, tc_desc(a0 + PA[t] * Cfg::kABytes + o), tc_desc(b0 + PB[t] * Cfg::kBBytes + o), idesc,
                               (first && ks == 0 && t == 0) ? 0u : 1u);
                }
                tc_commit(empty(s));
                if (kb % kTcDrainKB == kTcDrainKB - 1 || kb == nkb - 1) tc_commit(accf(a));
            }
            // every MMA issued above has completed before TMEM can be freed
            tc_commit(done);
            if (!mbar_wait_bounded(done, 0u)) *s_fail = 1;
        }
    } else {
        // epilogue warps: drain each block's accumulator into the running sums (row = TMEM lane)
        float sh[kTcDrainBN], sl[kTcDrainBN];
#pragma unroll
        for (int c = 0; c < kTcDrainBN; ++c) { sh[c] = 0.f; sl[c] = 0.f; }
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        bool ok = true;
        for (int blk = 0; blk < nblk && ok; ++blk) {
            const int a = blk & 1;
            if (*s_fail || !mbar_wait_bounded(accf(a), (uint32_t)((blk >> 1) & 1))) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int c0 = 0; c0 < kTcDrainBN; c0 += 16) {
                float v[16];
                if (c0 < bn) tmem_ld16(lane_base + (uint32_t)(a * kTcDrainBN + c0), v);
                else {
#pragma unroll
                    for (int q = 0; q < 16; ++q) v[q] = 0.f;
                }
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const float h = sh[c0 + q], x = v[q];
                    const float sum = h + x, bb = sum - h;
                    sl[c0 + q] += (h - (sum - bb)) + (x - bb);
                    sh[c0 + q] = sum;
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(acce(a));
        }
        if (!ok) *s_fail = 1;
        const int row = warp * 32 + lane, gi = i0 + row;
        if (ok && gi < d.M) {
#pragma unroll
            for (int c = 0; c < kTcDrainBN; ++c) {
                const int gj = j0 + c;
                if (c < bn && gj < d.N) d.C[(long long)gi * d.c_rs + (long long)gj * d.c_cs] = d.alpha * (sh[c] + sl[c]);
            }
        }
    }
    // the MMAs have completed (the issuer waited on its final commit); after a failure no bulk copy
    // may outlive the CTA: the producer waits (bounded) for the copies the MMAs never took
    __syncthreads();
    if (*s_fail && warp == 4 && lane == 0)
        for (int kb = *s_used; kb < issued; ++kb) mbar_wait_bounded(full(kb % S), (uint32_t)((kb / S) & 1));
    if (*s_fail && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(2 * kTcDrainBN) : "memory");
    }
}

// ------------------------------------------------------------------ host planning / launch
long long tc_gemm_plan(TcGemmDesc* d, int n, int parts, TcPackDesc* pk, int* tiles_out, long long* quads_out,
                       bool pack_a, int bn_max) {
    long long off = 0, quads = 0;
    int tiles = 0;
    for (int i = 0; i < n; ++i) {
        TcGemmDesc& g = d[i];
        const int bn = g.N <= bn_max ? ((g.N + 15) / 16) * 16 : bn_max;
        g.bn = bn < 16 ? 16 : bn;
        g.tiles_n = (g.N + g.bn - 1) / g.bn;
        g.tile_begin = tiles;
        tiles += g.tiles_n * ((g.M + kTcBM - 1) / kTcBM);
        const int kbe = parts == 1 ? 2 * kTcBK : kTcBK;            // elements per 64-byte K block
        const int nkb = (g.K + kbe - 1) / kbe;
        g.Mpad = ((g.M + kTcBM - 1) / kTcBM) * kTcBM;
        g.Npad = g.tiles_n * g.bn;
        const int np = parts == 1 ? 1 : parts;                       // 64-byte rows per K block and part
        g.a_off = off;
        off += (long long)np * nkb * g.Mpad * kTcBK;
        g.b_off = off;
        off += (long long)np * nkb * g.Npad * kTcBK;
        // A(i, k) rows = i; B(k, j) is packed as rows j
        TcPackDesc& pa = pk[2 * i];
        pa.X = g.A; pa.x_rs = g.a_rs; pa.x_cs = g.a_cs; pa.R = g.M; pa.K = g.K; pa.Rpad = g.Mpad; pa.nkb = nkb;
        pa.out_off = g.a_off; pa.quad_begin = quads;
        if (pack_a) quads += 4LL * g.Mpad * nkb;
        else pa.nkb = 0;                               // A written packed by its producer
        TcPackDesc& pb = pk[2 * i + 1];
        pb.X = g.B; pb.x_rs = g.b_cs; pb.x_cs = g.b_rs; pb.R = g.N; pb.K = g.K; pb.Rpad = g.Npad; pb.nkb = nkb;
        pb.out_off = g.b_off; pb.quad_begin = quads;
        quads += 4LL * g.Npad * nkb;
    }
    *tiles_out = tiles;
    *quads_out = quads;
    return off;
}

void launch_tc_gemm(int parts, const TcGemmDesc* d_descs, int nprob, int tiles, const TcPackDesc* d_pack,
                    long long quads, float* packed, int* err, cudaStream_t st) {
    if (parts == 1) {
        if (quads > 0) { k_tc_pack_bf16<<<ceil_div(quads, 256), 256, 0, st>>>(d_pack, 2 * nprob, packed); SGL_COUNT(1); }
        cudaFuncSetAttribute(k_tc_gemm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<1>::kSmem);
        k_tc_gemm<1><<<tiles, kTcThreads, TcCfg<1>::kSmem, st>>>(d_descs, nprob, packed, err);
        SGL_COUNT(1);
    } else if (parts == 3) {
        if (quads > 0) { k_tc_pack<3><<<ceil_div(quads, 256), 256, 0, st>>>(d_pack, 2 * nprob, packed); SGL_COUNT(1); }
        cudaFuncSetAttribute(k_tc_gemm<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<3>::kSmem);
        k_tc_gemm<3><<<tiles, kTcThreads, TcCfg<3>::kSmem, st>>>(d_descs, nprob, packed, err);
        SGL_COUNT(1);
    } else {
        if (quads > 0) { k_tc_pack<2><<<ceil_div(quads, 256), 256, 0, st>>>(d_pack, 2 * nprob, packed); SGL_COUNT(1); }
        cudaFuncSetAttribute(k_tc_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<2>::kSmem);
        k_tc_gemm<2><<<tiles, kTcThreads, TcCfg<2>::kSmem, st>>>(d_descs, nprob, packed, err);
        SGL_COUNT(1);
    }
}

void launch_tc_gemm_drain(int parts, const TcGemmDesc* d_descs, int nprob, int tiles, const TcPackDesc* d_pack,
                          long long quads, float* packed, int* err, cudaStream_t st) {
    if (parts == 3) {
        if (quads > 0) { k_tc_pack<3><<<ceil_div(quads, 256), 256, 0, st>>>(d_pack, 2 * nprob, packed); SGL_COUNT(1); }
        cudaFuncSetAttribute(k_tc_gemm_drain<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcDrainCfg<3>::kSmem);
        k_tc_gemm_drain<3><<<tiles, kTcDrainThreads, TcDrainCfg<3>::kSmem, st>>>(d_descs, nprob, packed, err);
    } else {
        if (quads > 0) { k_tc_pack<2><<<ceil_div(quads, 256), 256, 0, st>>>(d_pack, 2 * nprob, packed); SGL_COUNT(1); }
        cudaFuncSetAttribute(k_tc_gemm_drain<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcDrainCfg<2>::kSmem);
        k_tc_gemm_drain<2><<<tiles, kTcDrainThreads, TcDrainCfg<2>::kSmem, st>>>(d_descs, nprob, packed, err);
    }
    SGL_COUNT(1);
}

int tc_drain_bn() { return kTcDrainBN; }

}  // namespace sgl
