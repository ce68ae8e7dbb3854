// Fused inference of the surrogate MLP (8 -> 256 -> 5 x (256 -> 256) -> 2, SiLU): one persistent
// kernel, one CTA per SM, 128-row tiles; the activations never leave the SM.
//
// Per tile, the input layer (K = 8) runs on the CUDA cores in FP32.  Each hidden layer is one
// accumulation in TMEM (128 lanes x 256 columns FP32) of tcgen05.mma.kind::f16 products of the
// layer's input, held in shared memory as two BF16 parts (hi = bf16(a), lo = bf16(a - hi): the FP32
// activation to 2^-17), with the layer's BF16 weights streamed through a 4-stage ring of 16 KB bulk
// copies (the same for every tile: L2-resident).  The epilogue warps read the accumulator with
// tcgen05.ld, add the bias, apply SiLU and write the next layer's hi / lo parts in the canonical
// K-major layout; after the last hidden layer they form the two outputs as FP32 dot products.  The
// arithmetic is that of the training forward (BF16 weights, split BF16 inputs, FP32 accumulation).
//
// Warps 0-3: epilogue (row = thread), warp 4 lane 0: weight copies, warp 5 lane 0: MMAs.  Every wait
// is bounded; a wait that runs out raises *err, and the CTA waits for its copies in flight and
// frees its TMEM before it returns.
#include <cuda_bf16.h>

#include <algorithm>

#include "kernels.cuh"
#include "tcgen05.cuh"

namespace sgl {
namespace {

constexpr int kMfRows = 128;
constexpr int kMfW = 256;                          // hidden width
constexpr int kMfIn = 8;
constexpr int kMfHidden = 5;                       // 256 -> 256 layers on the tensor cores
constexpr int kMfKB = kMfW / 32;                   // 32-element K blocks per layer
constexpr int kMfABlock = kMfRows * 64;            // bytes of one K block of one activation part
constexpr int kMfWBlock = kMfW * 64;               // bytes of one K block of a weight matrix
constexpr int kMfStages = 4;
constexpr int kMfThreads = 192;
constexpr int kMfOffAhi = 0;
constexpr int kMfOffAlo = kMfKB * kMfABlock;                         // 64 KB
constexpr int kMfOffRing = 2 * kMfKB * kMfABlock;                    // 128 KB
constexpr int kMfOffSmall = kMfOffRing + kMfStages * kMfWBlock;      // 192 KB
// small tables (floats): W0 [8][256], biases [6][256], W6 [256][2], b6 [2]
constexpr int kMfSmallFloats = kMfIn * kMfW + 6 * kMfW + 2 * kMfW + 2;
constexpr int kMfOffBar = kMfOffSmall + ((kMfSmallFloats * 4 + 127) / 128) * 128;
constexpr int kMfSmem = kMfOffBar + 128;

// byte offset of (row r, k) of a K-major activation part: K blocks of 32, core matrices 8 x 16 B
__device__ __forceinline__ uint32_t mf_a_off(int r, int k) {
    return (uint32_t)((k >> 5) * kMfABlock + (r >> 3) * 512 + ((k & 31) >> 3) * 128 + (r & 7) * 16);
}

__device__ __forceinline__ float mf_silu(float z) { return z / (1.f + expf(-z)); }

// 8 consecutive activations of one row (k0 multiple of 8) into the hi / lo parts
__device__ __forceinline__ void mf_store8(unsigned char* sm, int r, int k0, const float* a) {
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a[2 * e], a[2 * e + 1]);
        const float2 hf = __bfloat1622float2(h);
        const __nv_bfloat162 l = __floats2bfloat162_rn(a[2 * e] - hf.x, a[2 * e + 1] - hf.y);
        hi[e] = *(const uint32_t*)&h;
        lo[e] = *(const uint32_t*)&l;
    }
    const uint32_t o = mf_a_off(r, k0);
    *(uint4*)(sm + kMfOffAhi + o) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *(uint4*)(sm + kMfOffAlo + o) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
}

__global__ void __launch_bounds__(kMfThreads, 1)
k_mlp_fused(int n, const float* __restrict__ X, const unsigned char* __restrict__ Wp, const float* __restrict__ small,
            float* __restrict__ Y, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t sb = (uint32_t)__cvta_generic_to_shared(sm);
    const uint32_t bar = sb + kMfOffBar;               // full[4], empty[4], layer_done, a_ready
    const uint32_t b_full = bar, b_empty = bar + 8 * kMfStages, b_done = bar + 16 * kMfStages,
                   b_ready = b_done + 8;
    volatile int* s_fail = (volatile int*)(sm + kMfOffBar + 96);
    const uint32_t tslot = sb + kMfOffBar + 104;
    float* s_small = (float*)(sm + kMfOffSmall);
    const float* s_W0 = s_small;                       // [k][n]
    const float* s_b = s_small + kMfIn * kMfW;          // [layer][n], layer 0 .. 5
    const float* s_W6 = s_b + 6 * kMfW;                 // [k][2]
    const float* s_b6 = s_W6 + 2 * kMfW;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_tiles = (n + kMfRows - 1) / kMfRows;

    for (int e = tid; e < kMfSmallFloats; e += kMfThreads) s_small[e] = small[e];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(tslot), "r"(kMfW) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < 2 * kMfStages + 1; ++s) mbar_init(bar + 8 * s, 1);
        mbar_init(b_ready, kMfRows);
        *s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *(volatile uint32_t*)(sm + kMfOffBar + 104);

    if (warp == 4) {
        if (lane == 0) {
            // weight copies: per tile, every hidden layer's 8 K blocks, through the ring
            long long it = 0;
            for (int t = blockIdx.x; t < n_tiles && !*s_fail; t += gridDim.x) {
                for (int q = 0; q < kMfHidden * kMfKB; ++q, ++it) {
                    const int s = (int)(it % kMfStages);
                    if (it >= kMfStages && !mbar_wait_bounded(b_empty + 8 * s, (uint32_t)(((it / kMfStages) - 1) & 1))) {
                        *s_fail = 1;
                        break;
                    }
                    mbar_expect_tx(b_full + 8 * s, kMfWBlock);
                    bulk_g2s(sb + kMfOffRing + s * kMfWBlock, Wp + (long long)q * kMfWBlock, kMfWBlock, b_full + 8 * s);
                }
                if (*s_fail) break;
            }
            // the copies issued last have landed before the CTA moves on (normally already consumed)
            for (long long j = it - 1; j >= 0 && j >= it - kMfStages; --j)
                if (!mbar_wait_bounded(b_full + 8 * (int)(j % kMfStages), (uint32_t)((j / kMfStages) & 1))) *s_fail = 1;
        }
    } else if (warp == 5) {
        if (lane == 0) {
            const uint32_t idesc = tc_idesc_bf16(kMfRows, kMfW);
            long long it = 0, use = 0;
            for (int t = blockIdx.x; t < n_tiles && !*s_fail; t += gridDim.x) {
                for (int l = 0; l < kMfHidden; ++l, ++use) {
                    if (!mbar_wait_bounded(b_ready, (uint32_t)(use & 1))) { *s_fail = 1; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    for (int kb = 0; kb < kMfKB; ++kb, ++it) {
                        const int s = (int)(it % kMfStages);
                        if (*s_fail || !mbar_wait_bounded(b_full + 8 * s, (uint32_t)((it / kMfStages) & 1))) {
                            *s_fail = 1;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t w0 = sb + kMfOffRing + s * kMfWBlock;
                        const uint32_t ah = sb + kMfOffAhi + kb * kMfABlock, al = sb + kMfOffAlo + kb * kMfABlock;
#pragma unroll
                        for (int ks = 0; ks < 2; ++ks) {
                            const uint32_t o = ks * 2 * kTcLBO;
                            tc_mma_bf16(tmem, tc_desc(ah + o), tc_desc(w0 + o), idesc, (kb | ks) ? 1u : 0u);
                            tc_mma_bf16(tmem, tc_desc(al + o), tc_desc(w0 + o), idesc, 1u);
                        }
                        tc_commit(b_empty + 8 * s);
                    }
                    if (*s_fail) break;
                    tc_commit(b_done);
                }
            }
        }
    } else {
        // epilogue: row tid of the tile
        const int r = tid;
        long long use = 0;
        for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) {
            const long long gr = (long long)t * kMfRows + r;
            float x[kMfIn];
#pragma unroll
            for (int k = 0; k < kMfIn; ++k) x[k] = gr < n ? X[gr * kMfIn + k] : 0.f;
            // input layer on the CUDA cores
            for (int n0 = 0; n0 < kMfW; n0 += 8) {
                float a[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    float z = s_b[n0 + j];
#pragma unroll
                    for (int k = 0; k < kMfIn; ++k) z = fmaf(x[k], s_W0[k * kMfW + n0 + j], z);
                    a[j] = mf_silu(z);
                }
                mf_store8(sm, r, n0, a);
            }
            fence_proxy_async_smem();
            mbar_arrive(b_ready);
            float y0 = 0.f, y1 = 0.f;
            bool bad = false;
            for (int l = 0; l < kMfHidden; ++l, ++use) {
                // the decision to stop is the whole warp's: tcgen05.ld below is warp-collective
                bad = *s_fail != 0 || !mbar_wait_bounded(b_done, (uint32_t)(use & 1));
                if (__any_sync(0xffffffffu, bad)) { bad = true; *s_fail = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const float* bl = s_b + (l + 1) * kMfW;
                for (int c0 = 0; c0 < kMfW; c0 += 16) {
                    float v[16];
                    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
                    for (int q = 0; q < 16; ++q) v[q] = mf_silu(v[q] + bl[c0 + q]);
                    if (l < kMfHidden - 1) {
                        mf_store8(sm, r, c0, v);
                        mf_store8(sm, r, c0 + 8, v + 8);
                    } else {
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            y0 = fmaf(v[q], s_W6[2 * (c0 + q)], y0);
                            y1 = fmaf(v[q], s_W6[2 * (c0 + q) + 1], y1);
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                if (l < kMfHidden - 1) {
                    fence_proxy_async_smem();
                    mbar_arrive(b_ready);
                }
            }
            if (bad) break;
            if (gr < n) {
                Y[2 * gr] = y0 + s_b6[0];
                Y[2 * gr + 1] = y1 + s_b6[1];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && *s_fail) atomicExch(err, 1);
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kMfW) : "memory");
    }
}

// hidden weights W_l (FP32 [k][n], l = 1 .. 5) -> BF16 canonical K-major B blocks [l][kb][n rows][64 B]
__global__ void k_mlp_pack_hidden(const float* const* __restrict__ W, unsigned char* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;           // (layer, kb, n, chunk of 8 k)
    const int total = kMfHidden * kMfKB * kMfW * 4;
    if (e >= total) return;
    const int c = e & 3, nrow = (e >> 2) % kMfW, kb = ((e >> 2) / kMfW) % kMfKB, l = (e >> 2) / kMfW / kMfKB;
    const float* Wl = W[l];
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int k = kb * 32 + c * 8 + 2 * q;
        const __nv_bfloat162 b2 = __floats2bfloat162_rn(Wl[k * kMfW + nrow], Wl[(k + 1) * kMfW + nrow]);
        w[q] = *(const uint32_t*)&b2;
    }
    const long long o = (long long)(l * kMfKB + kb) * kMfWBlock + (nrow >> 3) * 512 + c * 128 + (nrow & 7) * 16;
    *(uint4*)(out + o) = make_uint4(w[0], w[1], w[2], w[3]);
}

// the small tables: input weights and last weights rounded to BF16 (as the training forward's GEMMs
// use them), biases FP32
__global__ void k_mlp_pack_small(const float* __restrict__ W0, const float* const* __restrict__ b,
                                 const float* __restrict__ W6, const float* __restrict__ b6, float* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < kMfIn * kMfW) { out[e] = __bfloat162float(__float2bfloat16_rn(W0[e])); return; }
    int f = e - kMfIn * kMfW;
    if (f < 6 * kMfW) { out[e] = b[f / kMfW][f % kMfW]; return; }
    f -= 6 * kMfW;
    if (f < 2 * kMfW) { out[e] = __bfloat162float(__float2bfloat16_rn(W6[f])); return; }
    f -= 2 * kMfW;
    if (f < 2) out[e] = b6[f];
}

}  // namespace

int mlp_fused_smem() { return kMfSmem; }
int mlp_fused_small_floats() { return kMfSmallFloats; }
long long mlp_fused_wp_bytes() { return (long long)kMfHidden * kMfKB * kMfWBlock; }

void launch_mlp_fused(int n, const float* X, const float* const* W_dev, const float* const* b_dev, unsigned char* Wp,
                      float* small, const float** ptrs, float* Y, int* err, int ctas, cudaStream_t st) {
    // ptrs (device): W_1 .. W_5, then b_0 .. b_5
    k_mlp_pack_hidden<<<ceil_div(kMfHidden * kMfKB * kMfW * 4, 256), 256, 0, st>>>(ptrs, Wp);
    k_mlp_pack_small<<<ceil_div(kMfSmallFloats, 256), 256, 0, st>>>(W_dev[0], ptrs + kMfHidden, W_dev[6], b_dev[6], small);
    const int n_tiles = (n + kMfRows - 1) / kMfRows;
    k_mlp_fused<<<std::max(1, std::min(ctas, n_tiles)), kMfThreads, kMfSmem, st>>>(n, X, Wp, small, Y, err);
    SGL_COUNT(3);
}

sgl_status mlp_fused_attr() {
    return cudaFuncSetAttribute(k_mlp_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, kMfSmem) == cudaSuccess
               ? SGL_OK : SGL_ERR_CUDA;
}

}  // namespace sgl
