// Allocation-free variant of the kappa-axis sweep:
//   out[n] = sum_c w_c (e^{i kk_n kap_c} - 1 - i kk_n kap_c)      (Psi_1 at k_gamma = 0, FP64)
// The regular path (sgl_lnphi) keeps the per-chunk partial sums in device scratch that the
// context allocates.  This entry point keeps them in a fixed file-scope device array instead, so
// it calls no cudaMalloc / cudaFree and no allocating library routine.  It is for callers that
// may not allocate device memory themselves: e.g. a host that hands its whole device budget to
// a caching allocator or memory pool at start-up (a second allocator would fragment it or fail
// under the cap), or a runtime whose policy forbids allocations from third-party libraries on its
// streams.  The caller passes device-accessible inputs and outputs and the stream to run on.
#include <string>

#include "kernels.cuh"

namespace sgl {

// 16 chunks x 32768 k-points of double2 partial sums = 8 MiB.  Every GPU that loads this library
// holds this array until the process exits.
constexpr int kNoAllocChunks = 16;
constexpr int kNoAllocMaxK = 32768;
static __device__ __align__(256) double2 g_noalloc_partials[kNoAllocChunks * kNoAllocMaxK];

constexpr int kNoAllocRows = 128;
constexpr int kNoAllocStage = 128;

// CTA (row tile, chunk): each thread owns one kk row; the chunk's cells are staged in shared
// memory and broadcast.  Writes every part[chunk * nk + n] with n < nk (nothing is read before
// it is written in the same call, so the array needs no clearing between calls).
__global__ void __launch_bounds__(kNoAllocRows)
k_cf_kappa_partials(const double* __restrict__ kk, int nk, const double* __restrict__ k0,
                    const double* __restrict__ w0, long long nc, double2* __restrict__ part) {
    __shared__ double s_k[kNoAllocStage];
    __shared__ double s_w[kNoAllocStage];
    const int n = blockIdx.x * kNoAllocRows + threadIdx.x;
    const double k = (n < nk) ? kk[n] : 0.0;
    const long long per = (nc + kNoAllocChunks - 1) / kNoAllocChunks;
    const long long c0 = (long long)blockIdx.y * per;
    const long long c1 = c0 + per < nc ? c0 + per : nc;
    double ar = 0.0, ai = 0.0;
    for (long long base = c0; base < c1; base += kNoAllocStage) {
        const int cnt = (int)((c1 - base) < kNoAllocStage ? (c1 - base) : kNoAllocStage);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += kNoAllocRows) { s_k[e] = k0[base + e]; s_w[e] = w0[base + e]; }
        __syncthreads();
        for (int e = 0; e < cnt; ++e) {
            const double ph = k * s_k[e];
            double s, c;
            sincos(0.5 * ph, &s, &c);
            const double cm1 = -2.0 * s * s;               // cos(ph) - 1 without cancellation
            double smp;                                     // sin(ph) - ph
            if (fabs(ph) < 1e-2) {
                const double p2 = ph * ph;
                smp = -ph * p2 / 6.0 * (1.0 - p2 / 20.0 * (1.0 - p2 / 42.0));
            } else {
                smp = 2.0 * s * c - ph;
            }
            ar = fma(s_w[e], cm1, ar);
            ai = fma(s_w[e], smp, ai);
        }
    }
    if (n < nk) part[(long long)blockIdx.y * nk + n] = make_double2(ar, ai);
}

__global__ void k_cf_kappa_reduce(const double2* __restrict__ part, int nk, double* __restrict__ re,
                                  double* __restrict__ im) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nk) return;
    double r = 0.0, i = 0.0;
    for (int c = 0; c < kNoAllocChunks; ++c) { const double2 v = part[(long long)c * nk + n]; r += v.x; i += v.y; }
    re[n] = r;
    im[n] = i;
}

}  // namespace sgl

std::string& sgl_noctx_error();   // message slot read by sgl_last_error(NULL, ...)

extern "C" sgl_status sgl_cf_kappa_noalloc(const double* kk, int nk, const double* k0, const double* w0,
                                           int64_t n_cells, double* out_re, double* out_im, void* stream) {
    using namespace sgl;
    if (nk < 1 || nk > kNoAllocMaxK) {
        sgl_noctx_error() = "sgl_cf_kappa_noalloc: nk must be in [1, " + std::to_string(kNoAllocMaxK) +
                        "] (fixed 8 MiB scratch), got " + std::to_string(nk);
        return SGL_ERR_VALUE;
    }
    if (n_cells < 0 || (n_cells > 0 && (!k0 || !w0)) || !kk || !out_re || !out_im) {
        sgl_noctx_error() = "sgl_cf_kappa_noalloc: null pointer or negative n_cells";
        return SGL_ERR_VALUE;
    }
    // The device address of the scratch array, looked up on every call with the caller's device
    // current.  The lookup is a host-side query, not stream work; it is repeated rather than cached
    // so that a context torn down and recreated (cudaDeviceReset), which may reload the module at
    // another address, is followed.  The first call on a device may load the module: make it
    // before any stream capture.
    void* scratch = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_partials);
    if (e != cudaSuccess || !scratch) {
        int dev = -1;
        const cudaError_t ed = cudaGetDevice(&dev);
        sgl_noctx_error() = std::string("sgl_cf_kappa_noalloc: cudaGetSymbolAddress of the scratch array failed on device ") +
                            (ed == cudaSuccess ? std::to_string(dev) : std::string("(none current)")) + ": " +
                            cudaGetErrorString(e);
        return SGL_ERR_CUDA;
    }
    cudaStream_t st = (cudaStream_t)stream;
    dim3 grid(ceil_div(nk, kNoAllocRows), kNoAllocChunks);
    k_cf_kappa_partials<<<grid, kNoAllocRows, 0, st>>>(kk, nk, k0, w0, (long long)n_cells, (double2*)scratch);
    SGL_COUNT(1);
    k_cf_kappa_reduce<<<ceil_div(nk, 256), 256, 0, st>>>((const double2*)scratch, nk, out_re, out_im);
    SGL_COUNT(1);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        sgl_noctx_error() = std::string("sgl_cf_kappa_noalloc: launch failed: ") + cudaGetErrorString(e);
        return SGL_ERR_CUDA;
    }
    return SGL_OK;
}
