// Device-side preparation of the xi_lin groups when the GPU reads host memory coherently
// (pageable-memory access through the host page tables: Grace + NVLink-C2C).  The caller's rows
// are read once, coalesced, straight into device memory; nothing is staged through the host.
//   k_xi_stage_rows flat copy of the caller's rows into device memory
//   k_xi_row_norms  Euclidean norm of every raw row (the prune threshold)
//   k_xi_transpose  rows_t[i][rr] = row_rr[order[i]] (FP64 and FP32 copies), coalesced tiles
//   k_xi_rowprep    one CTA per kept row, the row held in shared memory:
//                   the row sum and residual, the per-gamma-cell sums U[row][q] and, for m = 0 rows,
//                   the per-kappa-cell sums W0[row][p], the compacted U0 and the sigma term
//                   (row . kc + res).  Every sum runs over a fixed entry order (deterministic).
#include "kernels.cuh"

namespace sgl {

// flat copy of the caller's rows into device memory: 16-byte loads, four independent ones in flight
// per thread so that enough bytes are outstanding to cover the link's latency.  `lead` doubles
// (0 or 1) are copied singly so that the vector part starts on a 16-byte boundary of src.
__global__ void __launch_bounds__(256)
k_xi_stage_rows(const double* __restrict__ src, long long n, double* __restrict__ dst, int lead) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < lead && t < n) dst[t] = src[t];
    const long long nv = (n - lead) / 2;
    const double2* s2 = (const double2*)(src + lead);
    double* d = dst + lead;
    long long i = t;
    for (; i + 3 * stride < nv; i += 4 * stride) {
        const double2 a = s2[i], b = s2[i + stride], c = s2[i + 2 * stride], e = s2[i + 3 * stride];
        d[2 * i] = a.x; d[2 * i + 1] = a.y;
        d[2 * (i + stride)] = b.x; d[2 * (i + stride) + 1] = b.y;
        d[2 * (i + 2 * stride)] = c.x; d[2 * (i + 2 * stride) + 1] = c.y;
        d[2 * (i + 3 * stride)] = e.x; d[2 * (i + 3 * stride) + 1] = e.y;
    }
    for (; i < nv; i += stride) { const double2 a = s2[i]; d[2 * i] = a.x; d[2 * i + 1] = a.y; }
    if (t == 0 && lead + 2 * nv < n) dst[n - 1] = src[n - 1];
}

__global__ void __launch_bounds__(256)
k_xi_row_norms(const double* __restrict__ rows, const long long* __restrict__ row_start,
               const int* __restrict__ row_len, int nrows, double* __restrict__ norms) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nrows) return;
    const double* r = rows + row_start[warp];
    const int n = row_len[warp];
    double a = 0.0;
    for (int e = lane; e < n; e += 32) a = fma(r[e], r[e], a);
    a = warp_sum(a);
    if (lane == 0) norms[warp] = sqrt(a);
}

__global__ void __launch_bounds__(256)
k_xi_rowprep(const double* __restrict__ rows, const XiPrepRow* __restrict__ kr, const XiPrepIdx ix,
             const double* __restrict__ kmc, XiPrepOut o) {
    extern __shared__ __align__(16) double xr[];
    __shared__ double sh[32];
    const XiPrepRow d = kr[blockIdx.x];
    const double* r = rows + d.src;
    for (int e = threadIdx.x; e <= d.ne; e += blockDim.x) xr[e] = r[e];
    __syncthreads();
    // the row sum (the transposed copies come from k_xi_transpose)
    double a = 0.0;
    for (int e = threadIdx.x; e < d.ne; e += blockDim.x) a += xr[e];
    a = block_sum(a, sh);
    if (threadIdx.x == 0) { o.sums[d.row] = a; o.res[d.row] = xr[d.ne]; }
    // U[row][q]: one thread per gamma cell of the group, entries in q-order
    const int* qord = ix.qord + d.ent0;
    const int* qseg = ix.qseg + d.qseg0;
    for (int j = threadIdx.x; j < d.nQ; j += blockDim.x) {
        double s = 0.0;
        for (int i = qseg[j]; i < qseg[j + 1]; ++i) s += xr[qord[i]];
        o.U[d.u_off + ix.idx_q[d.q0 + j]] = s;
        if (d.m == 0) o.U0[d.u0_off + j] = s;
    }
    if (d.m != 0) return;
    // W0[row][p] (entries in p-order, segments from the group's CSR) and the sigma term
    const int* pord = ix.pord + d.ent0;
    double dot = 0.0;
    for (int j = threadIdx.x; j < d.nP; j += blockDim.x) {
        double s = 0.0;
        for (int i = ix.p_ptr[d.p0 + j] - (int)d.ent0; i < ix.p_ptr[d.p0 + j + 1] - (int)d.ent0; ++i) s += xr[pord[i]];
        const int pcell = ix.idx_p[d.p0 + j];
        o.W0[d.w0_off + pcell] = s;
        dot = fma(s, kmc[pcell], dot);
    }
    dot = block_sum(dot, sh);
    if (threadIdx.x == 0) o.sig[d.row] = dot + xr[d.ne];
}

// word copy of a host array the device reads coherently (the source must stay alive until the
// stream reaches this copy)
__global__ void k_copy_words(const uint32_t* __restrict__ src, long long n, uint32_t* __restrict__ dst) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}

void launch_copy_from_host(const void* src, size_t bytes, void* dst, cudaStream_t st) {
    const long long n = (long long)(bytes / 4);
    if (n <= 0) return;
    k_copy_words<<<(unsigned)std::min<long long>(152 * 8, (n + 255) / 256), 256, 0, st>>>((const uint32_t*)src, n,
                                                                                          (uint32_t*)dst);
    SGL_COUNT(1);
}

void launch_xi_stage_rows(const double* rows, long long n, double* dst, cudaStream_t st) {
    if (n <= 0) return;
    const int lead = ((uintptr_t)rows & 15) ? 1 : 0;      // rows is 8-byte aligned (doubles)
    k_xi_stage_rows<<<152 * 8, 256, 0, st>>>(rows, n, dst, lead);
    SGL_COUNT(1);
}

// rows_t[i][rr] = row_rr[order[i]] (FP64 and FP32), one CTA per tile of kXiTransTile entries of a
// group: the tile's rows_t region is contiguous, so the writes are coalesced; the gathers from the
// group's rows hit L2.
constexpr int kXiTransTile = 64;

__global__ void __launch_bounds__(256)
k_xi_transpose(const double* __restrict__ rows, const XiPrepRow* __restrict__ kr, const int2* __restrict__ tiles,
               const int* __restrict__ pord, double* __restrict__ rt, float* __restrict__ rtf) {
    __shared__ long long s_src[256];
    __shared__ int s_po[kXiTransTile];
    const int2 tl = tiles[blockIdx.x];
    const XiPrepRow d0 = kr[tl.x];
    const int R = d0.R, i0 = tl.y, ni = min(kXiTransTile, d0.ne - i0);
    for (int rr = threadIdx.x; rr < R; rr += blockDim.x) s_src[rr] = kr[tl.x + rr].src;
    for (int il = threadIdx.x; il < ni; il += blockDim.x) s_po[il] = pord[d0.ent0 + i0 + il];
    __syncthreads();
    const long long base = d0.dst + (long long)i0 * R;
    for (int t = threadIdx.x; t < ni * R; t += blockDim.x) {
        const int il = t / R, rr = t - il * R;
        const double v = rows[s_src[rr] + s_po[il]];
        rt[base + t] = v;
        rtf[base + t] = (float)v;
    }
}

void launch_xi_transpose(const double* rows, const XiPrepRow* kr, const int2* tiles, int ntiles, const int* pord,
                         double* rt, float* rtf, cudaStream_t st) {
    if (ntiles > 0) { k_xi_transpose<<<ntiles, 256, 0, st>>>(rows, kr, tiles, pord, rt, rtf); SGL_COUNT(1); }
}

void launch_xi_row_norms(const double* rows, const long long* row_start, const int* row_len, int nrows,
                         double* norms, cudaStream_t st) {
    if (nrows > 0) { k_xi_row_norms<<<ceil_div((long long)nrows * 32, 256), 256, 0, st>>>(rows, row_start, row_len, nrows, norms); SGL_COUNT(1); }
}

void launch_xi_rowprep(const double* rows, const XiPrepRow* kr, int nkept, int ne_max, const XiPrepIdx& ix,
                       const double* kmc, const XiPrepOut& o, cudaStream_t st) {
    if (nkept <= 0) return;
    const size_t sm = ((size_t)ne_max + 1) * sizeof(double);
    cudaFuncSetAttribute(k_xi_rowprep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_xi_rowprep<<<nkept, 256, sm, st>>>(rows, kr, ix, kmc, o);
    SGL_COUNT(1);
}

}  // namespace sgl
