// Element-wise kernels of the per-plane log-CF surrogate MLP (BF16 tensor-core GEMMs are in
// tc_gemm.cu): bias + SiLU forward, SiLU backward, column sums for the bias gradients, MSE loss
// gradient and AdamW.  FP32 storage, FP64 for the reductions.
#include "kernels.cuh"

namespace sgl {

// Zb = Z + bias[col]; A = silu(Zb) (or Zb when silu = 0)
__global__ void k_bias_act(int M, int N, const float* __restrict__ Z, const float* __restrict__ bias,
                           float* __restrict__ Zb, float* __restrict__ A, int silu) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)M * N) return;
    const float z = Z[e] + bias[e % N];
    Zb[e] = z;
    A[e] = silu ? z / (1.f + expf(-z)) : z;
}

// dZ = dA * silu'(Zb),  silu'(z) = s (1 + z (1 - s)),  s = 1 / (1 + e^-z)
__global__ void k_act_grad(int M, int N, const float* __restrict__ dA, const float* __restrict__ Zb,
                           float* __restrict__ dZ) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)M * N) return;
    const float z = Zb[e];
    const float sg = 1.f / (1.f + expf(-z));
    dZ[e] = dA[e] * sg * (1.f + z * (1.f - sg));
}

// out[j] = sum_i X[i, j]: one CTA per column, FP64 tree
__global__ void __launch_bounds__(256) k_col_sum(int M, int N, const float* __restrict__ X, float* __restrict__ out) {
    __shared__ double sh[32];
    const int j = blockIdx.x;
    double a = 0.0;
    for (int i = threadIdx.x; i < M; i += blockDim.x) a += (double)X[(long long)i * N + j];
    a = block_sum(a, sh);
    if (threadIdx.x == 0) out[j] = (float)a;
}

// dpred = 2 (pred - target) / n; partial sums of (pred - target)^2 per CTA
__global__ void __launch_bounds__(256) k_mse(long long n, const float* __restrict__ pred, const float* __restrict__ tgt,
                                             float* __restrict__ dpred, double* __restrict__ part) {
    __shared__ double sh[32];
    double a = 0.0;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float d = pred[e] - tgt[e];
        dpred[e] = 2.f * d / (float)n;
        a += (double)d * d;
    }
    a = block_sum(a, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

// AdamW (decoupled weight decay), bias-corrected moments
__global__ void k_adamw(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                        float* __restrict__ v, float lr, float b1, float b2, float eps, float wd, float c1, float c2) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float gr = g[e];
    const float mm = b1 * m[e] + (1.f - b1) * gr;
    const float vv = b2 * v[e] + (1.f - b2) * gr * gr;
    m[e] = mm;
    v[e] = vv;
    w[e] = w[e] - lr * (mm / c1 / (sqrtf(vv / c2) + eps) + wd * w[e]);
}

void launch_bias_act(int M, int N, const float* Z, const float* bias, float* Zb, float* A, int silu, cudaStream_t st) {
    const long long t = (long long)M * N;
    if (t > 0) { k_bias_act<<<ceil_div(t, 256), 256, 0, st>>>(M, N, Z, bias, Zb, A, silu); SGL_COUNT(1); }
}
void launch_act_grad(int M, int N, const float* dA, const float* Zb, float* dZ, cudaStream_t st) {
    const long long t = (long long)M * N;
    if (t > 0) { k_act_grad<<<ceil_div(t, 256), 256, 0, st>>>(M, N, dA, Zb, dZ); SGL_COUNT(1); }
}
void launch_col_sum(int M, int N, const float* X, float* out, cudaStream_t st) {
    if (N > 0) { k_col_sum<<<N, 256, 0, st>>>(M, N, X, out); SGL_COUNT(1); }
}
int mse_blocks(long long n) { return (int)std::min<long long>(1024, std::max<long long>(1, ceil_div(n, 256))); }
void launch_mse(long long n, const float* pred, const float* tgt, float* dpred, double* part, cudaStream_t st) {
    k_mse<<<mse_blocks(n), 256, 0, st>>>(n, pred, tgt, dpred, part);
    SGL_COUNT(1);
}
void launch_adamw(long long n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                  float wd, float c1, float c2, cudaStream_t st) {
    if (n > 0) { k_adamw<<<ceil_div(n, 256), 256, 0, st>>>(n, w, g, m, v, lr, b1, b2, eps, wd, c1, c2); SGL_COUNT(1); }
}

}  // namespace sgl
