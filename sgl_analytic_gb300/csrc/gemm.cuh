// Grouped, register-tiled SIMT GEMM used by the separable Psi_1 products, the gauss Psi_2
// coarse-grid contraction and the Hankel / kappa transforms.
//
// C(i, j) = alpha * sum_k A(i, k) B(k, j) + beta * C(i, j)
// with arbitrary element strides for A and B (row- or column-major views) and a row-major C.
// Several independent problems (e.g. the xi_lin groups) run in ONE launch: each CTA finds its
// problem from a prefix sum of tile counts.  FP64 instances are FMA-pipe bound (GB300's FP64
// rate is a small fraction of FP32); FP32 instances use 128x128 tiles with 8x8 per thread.
#pragma once
#include "common.cuh"

namespace sgl {

template <typename T>
struct GemmDesc {
    int M, N, K;
    const T* A; long long a_rs, a_cs;   // A(i,k) = A[i*a_rs + k*a_cs]
    const T* B; long long b_rs, b_cs;   // B(k,j) = B[k*b_rs + j*b_cs]
    T* C; long long ldc;                // C(i,j) = C[i*ldc + j]
    T alpha, beta;
    int tile_begin;                     // first global tile of this problem
    int tiles_n;                        // tiles along N
};

template <typename T> struct GemmCfg;
template <> struct GemmCfg<double> { static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4; };
template <> struct GemmCfg<float>  { static constexpr int BM = 128, BN = 128, BK = 8, TM = 8, TN = 8; };

template <typename T>
__global__ void __launch_bounds__(256)
grouped_gemm_kernel(const GemmDesc<T>* __restrict__ descs, int nprob) {
    constexpr int BM = GemmCfg<T>::BM, BN = GemmCfg<T>::BN, BK = GemmCfg<T>::BK;
    constexpr int TM = GemmCfg<T>::TM, TN = GemmCfg<T>::TN;
    constexpr int NT = (BM / TM) * (BN / TN);
    static_assert(NT == 256, "256 threads per CTA");
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];

    // locate the problem (binary search over the tile prefix)
    const int tile = blockIdx.x;
    int p = 0, ph = nprob - 1;                       // last problem with tile_begin <= tile
    while (p < ph) {
        const int mid = (p + ph + 1) >> 1;
        if (descs[mid].tile_begin <= tile) p = mid; else ph = mid - 1;
    }
    const GemmDesc<T> d = descs[p];
    const int local = tile - d.tile_begin;
    const int tm = local / d.tiles_n, tn = local % d.tiles_n;
    const int i0 = tm * BM, j0 = tn * BN;
    if (i0 >= d.M) return;

    const int tid = threadIdx.x;
    const int tx = tid % (BN / TN), ty = tid / (BN / TN);
    T acc[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) acc[a][b] = T(0);

    const bool a_kcontig = (d.a_cs == 1);
    const bool b_jcontig = (d.b_cs == 1);
    for (int k0 = 0; k0 < d.K; k0 += BK) {
        // A tile: BM x BK
        for (int e = tid; e < BM * BK; e += NT) {
            int i, k;
            if (a_kcontig) { i = e / BK; k = e % BK; } else { k = e / BM; i = e % BM; }
            const int gi = i0 + i, gk = k0 + k;
            As[k][i] = (gi < d.M && gk < d.K) ? d.A[(long long)gi * d.a_rs + (long long)gk * d.a_cs] : T(0);
        }
        // B tile: BK x BN
        for (int e = tid; e < BK * BN; e += NT) {
            int k, j;
            if (b_jcontig) { k = e / BN; j = e % BN; } else { j = e / BK; k = e % BK; }
            const int gk = k0 + k, gj = j0 + j;
            Bs[k][j] = (gk < d.K && gj < d.N) ? d.B[(long long)gk * d.b_rs + (long long)gj * d.b_cs] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            T a[TM], b[TN];
#pragma unroll
            for (int r = 0; r < TM; ++r) a[r] = As[k][ty * TM + r];
#pragma unroll
            for (int c = 0; c < TN; ++c) b[c] = Bs[k][tx * TN + c];
#pragma unroll
            for (int r = 0; r < TM; ++r)
#pragma unroll
                for (int c = 0; c < TN; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < TM; ++r) {
        const int gi = i0 + ty * TM + r;
        if (gi >= d.M) continue;
#pragma unroll
        for (int c = 0; c < TN; ++c) {
            const int gj = j0 + tx * TN + c;
            if (gj >= d.N) continue;
            T* cp = d.C + (long long)gi * d.ldc + gj;
            T v = d.alpha * acc[r][c];
            if (d.beta != T(0)) v += d.beta * *cp;
            *cp = v;
        }
    }
}

// FP32 specialisation: 128 x 128 x 16 tiles, double-buffered shared memory with register
// prefetch, each thread an 8 x 8 micro-tile as 2 x 2 blocks of 4 x 4 read with float4 from
// padded shared memory (conflict-free), FMA accumulation in FP32.
template <>
__global__ void __launch_bounds__(256)
grouped_gemm_kernel<float>(const GemmDesc<float>* __restrict__ descs, int nprob) {
    constexpr int BM = 128, BN = 128, BK = 16, PAD = 4;
    __shared__ __align__(16) float As[2][BK][BM + PAD];
    __shared__ __align__(16) float Bs[2][BK][BN + PAD];
    const int tile = blockIdx.x;
    int p = 0, ph = nprob - 1;                       // last problem with tile_begin <= tile
    while (p < ph) {
        const int mid = (p + ph + 1) >> 1;
        if (descs[mid].tile_begin <= tile) p = mid; else ph = mid - 1;
    }
    const GemmDesc<float> d = descs[p];
    const int local = tile - d.tile_begin;
    const int i0 = (local / d.tiles_n) * BM, j0 = (local % d.tiles_n) * BN;
    if (i0 >= d.M) return;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const bool a_kc = (d.a_cs == 1), b_jc = (d.b_cs == 1);
    float ra[8], rb[8];
    auto load_tiles = [&](int k0) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int e = tid + u * 256;
            int i, k;
            if (a_kc) { i = e >> 4; k = e & 15; } else { k = e >> 7; i = e & 127; }
            const int gi = i0 + i, gk = k0 + k;
            ra[u] = (gi < d.M && gk < d.K) ? d.A[(long long)gi * d.a_rs + (long long)gk * d.a_cs] : 0.f;
            int kb, j;
            if (b_jc) { kb = e >> 7; j = e & 127; } else { j = e >> 4; kb = e & 15; }
            const int gk2 = k0 + kb, gj = j0 + j;
            rb[u] = (gk2 < d.K && gj < d.N) ? d.B[(long long)gk2 * d.b_rs + (long long)gj * d.b_cs] : 0.f;
        }
    };
    auto store_tiles = [&](int buf) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int e = tid + u * 256;
            int i, k;
            if (a_kc) { i = e >> 4; k = e & 15; } else { k = e >> 7; i = e & 127; }
            As[buf][k][i] = ra[u];
            int kb, j;
            if (b_jc) { kb = e >> 7; j = e & 127; } else { j = e >> 4; kb = e & 15; }
            Bs[buf][kb][j] = rb[u];
        }
    };
    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    const int ntiles = (d.K + BK - 1) / BK;
    load_tiles(0);
    store_tiles(0);
    __syncthreads();
    for (int t = 0; t < ntiles; ++t) {
        const int cur = t & 1;
        if (t + 1 < ntiles) load_tiles((t + 1) * BK);
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[cur][k][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[cur][k][ty * 4 + 64]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[cur][k][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[cur][k][tx * 4 + 64]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int r = 0; r < 8; ++r)
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[r][c] = fmaf(av[r], bv[c], acc[r][c]);
        }
        if (t + 1 < ntiles) store_tiles(cur ^ 1);
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int gi = i0 + ty * 4 + (r & 3) + (r >> 2) * 64;
        if (gi >= d.M) continue;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int gj = j0 + tx * 4 + (c & 3) + (c >> 2) * 64;
            if (gj >= d.N) continue;
            float* cp = d.C + (long long)gi * d.ldc + gj;
            float v = d.alpha * acc[r][c];
            if (d.beta != 0.f) v += d.beta * *cp;
            *cp = v;
        }
    }
}

// FP32 with the operand layouts fixed at compile time (AK: A is k-contiguous, BJ: B is
// j-contiguous).  Same tiling as the generic FP32 kernel above, but the per-thread load addresses
// are one base pointer plus constant strides and the edge predicates are hoisted out of the K
// loop, which keeps the kernel within 128 registers: two CTAs (16 warps) per SM instead of one.
//
// Compensated blocked accumulation.  The register accumulators run over kF32FoldTiles K-tiles
// (64 products); then each is folded into a per-output running sum kept in shared memory with
// Knuth's TwoSum, and the fold's exact rounding error is left in the register accumulator as the
// start of the next block.  The FP32 rounding of a long chain (error ~ eps sqrt(K) |sum|, which
// the PDF tail is sensitive to) is thereby confined to the 64-product blocks, each of which is
// small next to the total: no extra registers, 64 KB of shared memory for the running sums
// (thread t owns words t, t + 256, ... so the folds are bank-conflict free).
constexpr int kF32FoldTiles = 4;

constexpr int kF32LayoutSmem = (2 * 16 * (128 + 4) * 2 + 64 * 256) * 4;   // operands + running sums
template <bool AK, bool BJ>
__global__ void __launch_bounds__(256, 2)
gemm_f32_layout_kernel(const GemmDesc<float>* __restrict__ descs, int nprob) {
    constexpr int BM = 128, BN = 128, BK = 16, PAD = 4;
    extern __shared__ __align__(16) float gemm_f32_smem[];
    auto As = reinterpret_cast<float (*)[BK][BM + PAD]>(gemm_f32_smem);
    auto Bs = reinterpret_cast<float (*)[BK][BN + PAD]>(gemm_f32_smem + 2 * BK * (BM + PAD));
    float* const Hs = gemm_f32_smem + 2 * BK * (BM + PAD) + 2 * BK * (BN + PAD);
    const int tile = blockIdx.x;
    int p = 0, ph = nprob - 1;
    while (p < ph) {
        const int mid = (p + ph + 1) >> 1;
        if (descs[mid].tile_begin <= tile) p = mid; else ph = mid - 1;
    }
    const GemmDesc<float> d = descs[p];
    const int local = tile - d.tile_begin;
    const int i0 = (local / d.tiles_n) * BM, j0 = (local % d.tiles_n) * BN;
    if (i0 >= d.M) return;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    // element u of this thread's share of a tile:
    //   A: AK ? (row ai + 16u, k ak) : (row ai, k ak + 2u)
    //   B: BJ ? (k bk + 2u, col bj) : (k bk, col bj + 16u)
    const int ai = AK ? (tid >> 4) : (tid & 127), ak = AK ? (tid & 15) : (tid >> 7);
    const int bj = BJ ? (tid & 127) : (tid >> 4), bk = BJ ? (tid >> 7) : (tid & 15);
    const float* pa = d.A + (long long)(i0 + ai) * d.a_rs + (long long)ak * d.a_cs;
    const float* pb = d.B + (long long)bk * d.b_rs + (long long)(j0 + bj) * d.b_cs;
    const long long a_u = AK ? 16 * d.a_rs : 2 * d.a_cs, a_t = (long long)BK * d.a_cs;
    const long long b_u = BJ ? 2 * d.b_rs : 16 * d.b_cs, b_t = (long long)BK * d.b_rs;
    unsigned a_ok = 0, b_ok = 0;            // bit u: row / column of element u inside the problem
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        if (i0 + ai + (AK ? 16 * u : 0) < d.M) a_ok |= 1u << u;
        if (j0 + bj + (BJ ? 0 : 16 * u) < d.N) b_ok |= 1u << u;
    }
    float ra[8], rb[8];
    auto load_tiles = [&](int t) {
        const int k0 = t * BK;
        const float* qa = pa + t * a_t;
        const float* qb = pb + t * b_t;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int gka = k0 + ak + (AK ? 0 : 2 * u);
            ra[u] = ((a_ok >> u) & 1u) && gka < d.K ? qa[u * a_u] : 0.f;
            const int gkb = k0 + bk + (BJ ? 2 * u : 0);
            rb[u] = ((b_ok >> u) & 1u) && gkb < d.K ? qb[u * b_u] : 0.f;
        }
    };
    auto store_tiles = [&](int buf) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (AK) As[buf][ak][ai + 16 * u] = ra[u]; else As[buf][ak + 2 * u][ai] = ra[u];
            if (BJ) Bs[buf][bk + 2 * u][bj] = rb[u]; else Bs[buf][bk][bj + 16 * u] = rb[u];
        }
    };
    // accumulators in column pairs: acc2[r][q] holds (acc[r][2q], acc[r][2q + 1]) for the packed FMA
    unsigned long long acc2[8][4];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
#pragma unroll
        for (int q = 0; q < 4; ++q) acc2[a][q] = 0ull;
#pragma unroll
        for (int b = 0; b < 8; ++b) Hs[(a * 8 + b) * 256 + tid] = 0.f;
    }
    // running sum += acc by TwoSum; acc keeps the exact rounding error of that addition
    auto fold = [&]() {
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float2 a2 = f32x2_unpack(acc2[r][q]);
                float av2[2] = {a2.x, a2.y};
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2) {
                    float* hp = Hs + (r * 8 + 2 * q + h2) * 256 + tid;
                    const float h = *hp, a = av2[h2];
                    const float sum = h + a;
                    const float bb = sum - h;
                    av2[h2] = (h - (sum - bb)) + (a - bb);
                    *hp = sum;
                }
                acc2[r][q] = f32x2_pack(av2[0], av2[1]);
            }
    };
    const int ntiles = (d.K + BK - 1) / BK;
    load_tiles(0);
    store_tiles(0);
    __syncthreads();
    for (int t = 0; t < ntiles; ++t) {
        const int cur = t & 1;
        if (t + 1 < ntiles) load_tiles(t + 1);
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[cur][k][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[cur][k][ty * 4 + 64]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[cur][k][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[cur][k][tx * 4 + 64]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const unsigned long long bp[4] = {f32x2_pack(b0.x, b0.y), f32x2_pack(b0.z, b0.w), f32x2_pack(b1.x, b1.y),
                                              f32x2_pack(b1.z, b1.w)};
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const unsigned long long ap = f32x2_pack(av[r], av[r]);
#pragma unroll
                for (int q = 0; q < 4; ++q) f32x2_fma(acc2[r][q], ap, bp[q]);
            }
        }
        if (t + 1 < ntiles) store_tiles(cur ^ 1);
        __syncthreads();
        if ((t + 1) % kF32FoldTiles == 0 && t + 1 < ntiles) fold();
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int gi = i0 + ty * 4 + (r & 3) + (r >> 2) * 64;
        if (gi >= d.M) continue;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int gj = j0 + tx * 4 + (c & 3) + (c >> 2) * 64;
            if (gj >= d.N) continue;
            float* cp = d.C + (long long)gi * d.ldc + gj;
            const float2 a2 = f32x2_unpack(acc2[r][c >> 1]);
            float v = d.alpha * (Hs[(r * 8 + c) * 256 + tid] + ((c & 1) ? a2.y : a2.x));
            if (d.beta != 0.f) v += d.beta * *cp;
            *cp = v;
        }
    }
}

// FP64, 16 x 16 output tiles, one output per thread: for problems too small to fill the GPU with
// 64 x 64 tiles (the 101 x 101 spline-coefficient products).  Each output accumulates over k in
// the same order as the tiled kernel, so the results are identical.
template <int B>
__global__ void __launch_bounds__(B * B)
gemm_f64_small_kernel(const GemmDesc<double>* __restrict__ descs, int nprob) {
    __shared__ double As[B][B + 1];
    __shared__ double Bs[B][B + 1];
    const int tile = blockIdx.x;
    int p = 0, ph = nprob - 1;
    while (p < ph) {
        const int mid = (p + ph + 1) >> 1;
        if (descs[mid].tile_begin <= tile) p = mid; else ph = mid - 1;
    }
    const GemmDesc<double> d = descs[p];
    const int local = tile - d.tile_begin;
    const int i0 = (local / d.tiles_n) * B, j0 = (local % d.tiles_n) * B;
    if (i0 >= d.M) return;
    const int tx = threadIdx.x % B, ty = threadIdx.x / B;
    double acc = 0.0;
    for (int k0 = 0; k0 < d.K; k0 += B) {
        {
            const int gi = i0 + ty, gk = k0 + tx;        // A(i0 + ty, k0 + tx) -> As[tx][ty]
            As[tx][ty] = (gi < d.M && gk < d.K) ? d.A[(long long)gi * d.a_rs + (long long)gk * d.a_cs] : 0.0;
            const int gk2 = k0 + ty, gj = j0 + tx;       // B(k0 + ty, j0 + tx) -> Bs[ty][tx]
            Bs[ty][tx] = (gk2 < d.K && gj < d.N) ? d.B[(long long)gk2 * d.b_rs + (long long)gj * d.b_cs] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < B; ++k) acc = fma(As[k][ty], Bs[k][tx], acc);
        __syncthreads();
    }
    const int gi = i0 + ty, gj = j0 + tx;
    if (gi < d.M && gj < d.N) {
        double* cp = d.C + (long long)gi * d.ldc + gj;
        double v = d.alpha * acc;
        if (d.beta != 0.0) v += d.beta * *cp;
        *cp = v;
    }
}

// Host helper: fills tile_begin / tiles_n and returns the total tile count.
template <typename T>
inline int gemm_plan(GemmDesc<T>* d, int nprob, int bm = GemmCfg<T>::BM, int bn = GemmCfg<T>::BN) {
    int t = 0;
    for (int p = 0; p < nprob; ++p) {
        d[p].tiles_n = ceil_div(d[p].N, bn);
        d[p].tile_begin = t;
        t += ceil_div(d[p].M, bm) * d[p].tiles_n;
    }
    return t;
}

}  // namespace sgl
