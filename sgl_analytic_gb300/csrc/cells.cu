// Binned-cell deposit of the population build (the reference's Cells accumulator, sgl_full.py:1282-1533):
// every emitter's points (kappa, gamma, weight, and for the xi_lin term the lens distance R) binned on
// the fine and coarse (kappa, gamma) lattices held in HBM (a few MB: L2-resident while a batch runs).
//
//   k_cells_hist   one thread per point: the exact searchsorted(side='right') bins (log-guessed, then
//                  corrected against the edges in shared memory), FP64 atomics into the fine sums of
//                  w, w kappa, w gamma and the coarse sums of w beta^n per shell, and per object the
//                  totals (w, w inside the fine lattice, w kappa over |kappa| < the fine grid's top)
//                  by a segmented warp scan (points of one object are contiguous).
//   k_cells_xi     one warp per point inside the coarse box: lanes over the k_perp nodes evaluate
//                  J0, J2, J4 of k_j R (reused while consecutive points share R and shear type) and add
//                  beta w J_{2m} into the point's coarse-bin row; the exact first moments accumulate in
//                  registers and leave once per warp.
//   k_cells_xi_*   the node's compression (xi_end): occupied rows per m, the residual first-moment row,
//                  the rows scaled by sqrt(c / dchi), their 42 x 42 Gram matrix (two-stage reduction in
//                  a fixed order) and the projection onto the kept eigenvectors.
#include <algorithm>

#include <math_constants.h>

#include "kernels.cuh"

namespace sgl {

namespace {

__device__ __forceinline__ int bracket(const double* e, int n, double v, int g) {
    g = g < 0 ? 0 : (g > n ? n : g);
    while (g > 0 && e[g - 1] > v) --g;
    while (g < n && e[g] <= v) ++g;
    return g;
}

// searchsorted(e, v, side='right') with the last edge moved into the last bin; e signed-log (-pos[::-1],
// pos) with pos = lo e^{i dl}: the log of |v| only guesses, bracket() makes the index exact
__device__ __forceinline__ int bin_signed_log(const double* e, int n, double v, double lo, double dl) {
    if (!(v == v)) return n;
    if (v < e[0]) return 0;
    int i;
    if (v >= e[n - 1]) {
        i = n;
    } else {
        const double a = fabs(v);
        int g = n / 2;
        if (a >= lo) {
            const int gl = (int)(log(a / lo) / dl) + 1;
            g = v > 0 ? n / 2 + gl : n / 2 - gl;
        }
        i = bracket(e, n, v, g);
    }
    if (v == e[n - 1]) --i;
    return i;
}

// the same on a geometric edge list lo e^{i dl}
__device__ __forceinline__ int bin_geom(const double* e, int n, double v, double lo, double dl) {
    if (!(v == v)) return n;
    if (v < e[0]) return 0;
    int i;
    if (v >= e[n - 1]) i = n;
    else i = bracket(e, n, v, (int)(log(v / lo) / dl) + 1);
    if (v == e[n - 1]) --i;
    return i;
}

__device__ __forceinline__ int object_of(const long long* off, int n_obj, long long i) {
    int lo = 0, hi = n_obj;            // the last o with off[o] <= i (empty objects are skipped)
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void load_edges(double* s, const double* e, int n) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) s[t] = e[t];
    __syncthreads();
}

// inclusive segmented scan over lanes whose segment starts at lane `lead`
__device__ __forceinline__ double seg_scan(double x, int lane, int lead) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const double v = __shfl_up_sync(0xffffffffu, x, d);
        if (lane - d >= lead) x += v;
    }
    return x;
}

// J0, J2, J4 of x as the deposit evaluates them: the power series below x = 2 (3 / 6 / 14 terms below
// 0.02 / 0.3 / 2), above it J0(x), J1(x) and the upward recurrence J_{n+1} = 2n J_n / x - J_{n-1}
__device__ __forceinline__ void bessel_even(double x, bool tang, double& J0, double& J2, double& J4) {
    if (x < 2.0) {
        const double h = 0.5 * x, h2 = h * h;
        double t0 = 1.0, s0 = 1.0, t2 = 0.5, s2 = 0.5, t4 = 1.0 / 24.0, s4 = 1.0 / 24.0;
        const int nt = x < 0.02 ? 3 : (x < 0.3 ? 6 : 14);
        for (int k = 1; k < nt; ++k) {
            const double f = (-h2) / k;
            t0 *= f / k;
            s0 += t0;
            t2 *= f / (k + 2);
            s2 += t2;
            t4 *= f / (k + 4);
            s4 += t4;
        }
        J0 = s0;
        J2 = tang ? s2 * (h * h) : 0.0;
        J4 = tang ? s4 * (h * h * h * h) : 0.0;
    } else {
        J0 = j0(x);
        if (tang) {
            const double inv = 1.0 / x, j1v = j1(x);
            J2 = 2.0 * inv * j1v - J0;
            const double j3 = 4.0 * inv * J2 - j1v;
            J4 = 6.0 * inv * j3 - J2;
        } else {
            J2 = J4 = 0.0;
        }
    }
}

__global__ void __launch_bounds__(256) k_cells_hist(CellsGeom G, const double* __restrict__ edges, long long n,
                                                    const double* __restrict__ K, const double* __restrict__ Gm,
                                                    const double* __restrict__ W, const long long* __restrict__ off,
                                                    int n_obj, const int* __restrict__ obj_shell,
                                                    const double* __restrict__ obj_betas, double* __restrict__ H0,
                                                    double* __restrict__ H0k, double* __restrict__ H0g,
                                                    double* __restrict__ Hc, double* __restrict__ sums) {
    extern __shared__ double s_e[];
    const int ne = G.nekf + G.negf + G.nekc + G.negc;
    load_edges(s_e, edges, ne);
    const double* ekf = s_e;
    const double* egf = ekf + G.nekf;
    const double* ekc = egf + G.negf;
    const double* egc = ekc + G.nekc;
    const int nkf = G.nekf - 1, ngf = G.negf - 1, nkc = G.nekc - 1, ngc = G.negc - 1, no = G.nord + 1;
    const int lane = threadIdx.x & 31;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
        const long long i = base + threadIdx.x;
        int o = 0x7fffffff;
        double w = 0.0, hin = 0.0, lin = 0.0;
        if (i < n) {
            o = object_of(off, n_obj, i);
            const double k = K[i];
            double g = Gm[i];
            w = W[i];
            g = g < G.g_clip ? G.g_clip : g;            // NaN stays NaN, as np.clip leaves it
            const int a = bin_signed_log(ekf, G.nekf, k, G.kf_lo, G.kf_dl);
            const int b = bin_geom(egf, G.negf, g, G.gf_lo, G.gf_dl);
            if (a >= 1 && a <= nkf && b >= 1 && b <= ngf) {
                const long long f = (long long)(a - 1) * ngf + (b - 1);
                atomicAdd(H0 + f, w);
                atomicAdd(H0k + f, __dmul_rn(w, k));
                atomicAdd(H0g + f, __dmul_rn(w, g));
                hin = w;
            }
            const int ac = bin_signed_log(ekc, G.nekc, k, G.kc_lo, G.kc_dl);
            const int bc = bin_geom(egc, G.negc, g, G.gc_lo, G.gc_dl);
            if (ac >= 1 && ac <= nkc && bc >= 1 && bc <= ngc) {
                double* h = Hc + (long long)obj_shell[o] * no * nkc * ngc + (long long)(ac - 1) * ngc + (bc - 1);
                for (int q = 0; q < no; ++q) atomicAdd(h + (long long)q * nkc * ngc, __dmul_rn(w, obj_betas[(long long)o * no + q]));
            }
            if (fabs(k) < G.k_max_fine) lin = __dmul_rn(w, k);
        }
        const unsigned same = __match_any_sync(0xffffffffu, o);
        const int lead = __ffs(same) - 1, last = 31 - __clz(same);
        w = seg_scan(w, lane, lead);
        hin = seg_scan(hin, lane, lead);
        lin = seg_scan(lin, lane, lead);
        if (lane == last && o != 0x7fffffff) {
            atomicAdd(sums + 3LL * o, w);
            atomicAdd(sums + 3LL * o + 1, hin);
            atomicAdd(sums + 3LL * o + 2, lin);
        }
    }
}

// One CTA per work item (a chunk of at most kXiChunk points of one object).  The chunk's points inside
// the coarse box are sorted in shared memory by (R, coarse bin); each warp takes runs of one radius,
// evaluates J0, J2, J4 at the 42 k_perp nodes once for it, merges the radius's points per bin (sum of
// beta w) and adds v J_{2m} into the bin's row; the radius's sums of beta w kappa and beta w gamma feed
// the exact first moments.  The same grouping as the reference's default deposit (sgl_full.py:1081-1130).
__global__ void __launch_bounds__(256) k_cells_xi(CellsGeom G, const double* __restrict__ edges,
                                                  const CellsXiItem* __restrict__ items,
                                                  const double* __restrict__ K, const double* __restrict__ Gm,
                                                  const double* __restrict__ W, const double* __restrict__ R,
                                                  const double* __restrict__ obj_beta,
                                                  const unsigned char* __restrict__ obj_tang,
                                                  const double* __restrict__ kp, int nkp, int mm,
                                                  double* __restrict__ Hx, double* __restrict__ lx,
                                                  double* __restrict__ Wb) {
    __shared__ double s_ek[kCellsXiMaxEdges];
    __shared__ double s_R[kXiChunk];
    __shared__ int s_c[kXiChunk], s_i[kXiChunk], s_seg[kXiChunk + 1];
    __shared__ double s_lx[8][2][64];
    __shared__ int s_nin, s_nseg;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;     // 256 threads
    const CellsXiItem it = items[blockIdx.x];
    const int nekc = G.nekc, negc = G.negc, nkc = nekc - 1, ngc = negc - 1;
    const double* ekc_g = edges + G.nekf + G.negf;
    for (int t = tid; t < nekc + negc; t += blockDim.x) s_ek[t] = ekc_g[t];
    if (tid == 0) { s_nin = 0; s_nseg = 0; }
    __syncthreads();
    const double* ekc = s_ek;
    const double* egc = s_ek + nekc;
    int n2 = 32;
    while (n2 < it.count) n2 <<= 1;
    for (int t = tid; t < n2; t += blockDim.x) {
        double r = CUDART_INF;
        int c = 0x7fffffff;
        if (t < it.count) {
            const long long i = it.first + t;
            const double k = K[i];
            double g = Gm[i];
            g = g < G.g_clip ? G.g_clip : g;
            const int ac = bin_signed_log(ekc, nekc, k, G.kc_lo, G.kc_dl);
            const int bc = bin_geom(egc, negc, g, G.gc_lo, G.gc_dl);
            if (ac >= 1 && ac <= nkc && bc >= 1 && bc <= ngc) {
                r = R[i];
                c = (ac - 1) * ngc + (bc - 1);
                atomicAdd(&s_nin, 1);
            }
        }
        s_R[t] = r;
        s_c[t] = c;
        s_i[t] = t;
    }
    __syncthreads();
    // bitonic sort of (R, bin) ascending; points outside the box (R = inf) go last
    for (int k = 2; k <= n2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int t = tid; t < n2; t += blockDim.x) {
                const int u = t ^ j;
                if (u > t) {
                    const bool gt = s_R[t] > s_R[u] || (s_R[t] == s_R[u] && s_c[t] > s_c[u]);
                    if (gt == ((t & k) == 0)) {
                        const double r = s_R[t]; s_R[t] = s_R[u]; s_R[u] = r;
                        const int c = s_c[t]; s_c[t] = s_c[u]; s_c[u] = c;
                        const int q = s_i[t]; s_i[t] = s_i[u]; s_i[u] = q;
                    }
                }
            }
            __syncthreads();
        }
    const int nin = s_nin;
    // starts of the runs of one radius (an emitter's cell centres repeat exactly across orientations),
    // in order: each thread flags 4 consecutive points, a block-wide exclusive scan places the starts
    {
        constexpr int kPer = kXiChunk / 256;
        int f[kPer], cnt = 0;
        for (int q = 0; q < kPer; ++q) {
            const int t = tid * kPer + q;
            f[q] = t < nin && (t == 0 || s_R[t] != s_R[t - 1]);
            cnt += f[q];
        }
        int inc = cnt;
        for (int d = 1; d < 32; d <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += v;
        }
        __shared__ int s_wsum[8];
        if (lane == 31) s_wsum[warp] = inc;
        __syncthreads();
        int base = inc - cnt;
        for (int w = 0; w < warp; ++w) base += s_wsum[w];
        for (int q = 0; q < kPer; ++q)
            if (f[q]) s_seg[base++] = tid * kPer + q;
        if (tid == 255) s_nseg = base;
        __syncthreads();
        if (tid == 0) s_seg[s_nseg] = nin;
        __syncthreads();
    }
    const int nseg = s_nseg;
    const double beta = obj_beta[it.obj];
    const bool tang = obj_tang[it.obj] != 0;
    const bool on0 = lane < nkp, on1 = lane + 32 < nkp;
    const double kp0 = on0 ? kp[lane] : 0.0, kp1 = on1 ? kp[lane + 32] : 0.0;
    const int mrow = (mm + 1) * nkp;
    double a00 = 0.0, a01 = 0.0, a10 = 0.0, a11 = 0.0;
    for (int sg = warp; sg < nseg; sg += blockDim.x >> 5) {
        const int p0 = s_seg[sg], p1 = s_seg[sg + 1];
        const double r = s_R[p0];
        double J0a = 0.0, J2a = 0.0, J4a = 0.0, J0b = 0.0, J2b = 0.0, J4b = 0.0;
        if (on0) bessel_even(kp0 * r, tang, J0a, J2a, J4a);
        if (on1) bessel_even(kp1 * r, tang, J0b, J2b, J4b);
        double sk = 0.0, sgm = 0.0;
        int p = p0;
        while (p < p1) {                   // runs of one bin within the radius: merged, then one row update
            const int c = s_c[p];
            double v = 0.0, ws = 0.0;
            for (; p < p1 && s_c[p] == c; ++p) {
                const long long i = it.first + s_i[p];
                const double w = W[i], k = K[i];
                double g = Gm[i];
                g = g < G.g_clip ? G.g_clip : g;
                const double bw = beta * w;
                v += bw;
                ws += w;
                sk += bw * k;
                sgm += bw * g;
            }
            double* row = Hx + (long long)c * mrow;
            if (on0) atomicAdd(row + lane, v * J0a);
            if (on1) atomicAdd(row + lane + 32, v * J0b);
            if (tang && mm >= 1) {
                if (on0) atomicAdd(row + nkp + lane, v * J2a);
                if (on1) atomicAdd(row + nkp + lane + 32, v * J2b);
                if (mm >= 2) {
                    if (on0) atomicAdd(row + 2 * nkp + lane, v * J4a);
                    if (on1) atomicAdd(row + 2 * nkp + lane + 32, v * J4b);
                }
            }
            if (Wb && lane == 0) atomicAdd(Wb + c, ws);
        }
        a00 += sk * J0a;
        a01 += sk * J0b;
        if (tang && mm >= 1) {
            a10 += sgm * J2a;
            a11 += sgm * J2b;
        }
    }
    s_lx[warp][0][lane] = a00;
    s_lx[warp][0][lane + 32] = a01;
    s_lx[warp][1][lane] = a10;
    s_lx[warp][1][lane + 32] = a11;
    __syncthreads();
    if (tid < 2 * nkp) {
        const int m = tid / nkp, j = tid % nkp;
        if (m == 0 || mm >= 1) {
            double s = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += s_lx[w][m][j];
            if (s != 0.0) atomicAdd(lx + m * nkp + j, s);
        }
    }
}

// lx[1][j] += beta n_area 2 pi Gam J1(k_j Rm) / (k_j Rm): the shear beyond the emitted radius
__global__ void k_cells_xi_tail(const double* __restrict__ kp, int nkp, double coef, double Rm, double* __restrict__ lx) {
    const int j = threadIdx.x;
    if (j < nkp) {
        const double a = kp[j] * Rm;
        lx[nkp + j] += coef * j1(a) / a;
    }
}

// flags[m * nbins + b] = 1 where the node's row (b, m) has a nonzero entry
__global__ void k_cells_xi_flags(const double* __restrict__ Hx, int nbins, int mm, int nkp, unsigned char* __restrict__ flags) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nbins * (mm + 1)) return;
    const int b = (int)(t / (mm + 1)), m = (int)(t % (mm + 1));
    const double* row = Hx + ((long long)b * (mm + 1) + m) * nkp;
    unsigned char any = 0;
    for (int j = 0; j < nkp; ++j) any |= row[j] != 0.0;
    flags[(long long)m * nbins + b] = any;
}

// A = [H[idx] ; lres] diag(sw): the residual row lres_j = lx_j - sum_r cen[idx_r] H[idx_r, j] (rows added
// in order, one thread per j), then the scaled rows
__global__ void k_cells_xi_rows(const double* __restrict__ Hx, int mm, int nkp, int m, const int* __restrict__ idx,
                                int nidx, const double* __restrict__ cen, int ngc, int cen_axis,
                                const double* __restrict__ lxm, const double* __restrict__ sw, double* __restrict__ A) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < (long long)nidx * nkp) {
        const long long r = t / nkp;
        const int j = (int)(t % nkp);
        A[t] = Hx[((long long)idx[r] * (mm + 1) + m) * nkp + j] * sw[j];
    }
    if (blockIdx.x == 0 && threadIdx.x < nkp) {
        const int j = threadIdx.x;
        double s = 0.0;
        if (cen_axis >= 0) {
            for (int r = 0; r < nidx; ++r) {
                const int b = idx[r];
                const double cb = cen[cen_axis == 0 ? b / ngc : b % ngc];
                s += cb * Hx[((long long)b * (mm + 1) + m) * nkp + j];
            }
        }
        const double lres = cen_axis >= 0 ? lxm[j] - s : 0.0;
        A[(long long)nidx * nkp + j] = lres * sw[j];
    }
}

// Gram partials: CTA c sums rows [c * chunk, (c + 1) * chunk) of A into part[c][p * nkp + q], p <= q
__global__ void __launch_bounds__(256) k_cells_gram(const double* __restrict__ A, long long nrows, int nkp, int chunk,
                                                    double* __restrict__ part) {
    extern __shared__ double s_a[];            // chunk x nkp
    const long long r0 = (long long)blockIdx.x * chunk;
    const int nr = (int)min((long long)chunk, nrows - r0);
    for (int t = threadIdx.x; t < nr * nkp; t += blockDim.x) s_a[t] = A[r0 * nkp + t];
    __syncthreads();
    for (int pq = threadIdx.x; pq < nkp * nkp; pq += blockDim.x) {
        const int p = pq / nkp, q = pq % nkp;
        if (q < p) continue;
        double s = 0.0;
        for (int r = 0; r < nr; ++r) s += s_a[r * nkp + p] * s_a[r * nkp + q];
        part[(long long)blockIdx.x * nkp * nkp + pq] = s;
    }
}

__global__ void k_cells_gram_sum(const double* __restrict__ part, int nparts, int nkp, double* __restrict__ Gram) {
    const int pq = blockIdx.x * blockDim.x + threadIdx.x;
    if (pq >= nkp * nkp) return;
    const int p = pq / nkp, q = pq % nkp;
    if (q < p) return;
    double s = 0.0;
    for (int c = 0; c < nparts; ++c) s += part[(long long)c * nkp * nkp + pq];
    Gram[p * nkp + q] = s;
    Gram[q * nkp + p] = s;
}

// rows[q][r] = sum_j A[r][j] V[j][q]: the kept modes, one thread per row of A
__global__ void k_cells_project(const double* __restrict__ A, long long nrows, int nkp, const double* __restrict__ V,
                                int nkeep, double* __restrict__ rows) {
    extern __shared__ double s_v[];            // nkp x nkeep
    for (int t = threadIdx.x; t < nkp * nkeep; t += blockDim.x) s_v[t] = V[t];
    __syncthreads();
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const double* a = A + r * nkp;
    for (int q = 0; q < nkeep; ++q) {
        double s = 0.0;
        for (int j = 0; j < nkp; ++j) s += a[j] * s_v[j * nkeep + q];
        rows[(long long)q * nrows + r] = s;
    }
}

}  // namespace

int cells_edge_smem_bytes(const CellsGeom& g) { return 8 * (g.nekf + g.negf + g.nekc + g.negc); }

void launch_cells_hist(const CellsGeom& g, const double* edges, long long n, const double* K, const double* Gm,
                       const double* W, const long long* off, int n_obj, const int* shell, const double* betas,
                       double* H0, double* H0k, double* H0g, double* Hc, double* sums, int n_sm, cudaStream_t st) {
    if (n <= 0) return;
    const long long blocks = std::min<long long>((n + 255) / 256, (long long)n_sm * 8);
    SGL_COUNT(1);
    k_cells_hist<<<(int)blocks, 256, cells_edge_smem_bytes(g), st>>>(g, edges, n, K, Gm, W, off, n_obj, shell, betas,
                                                                     H0, H0k, H0g, Hc, sums);
}

void launch_cells_xi(const CellsGeom& g, const double* edges, const CellsXiItem* items, int n_items,
                     const double* K, const double* Gm, const double* W, const double* R, const double* beta,
                     const unsigned char* tang, const double* kp, int nkp, int mm, double* Hx, double* lx, double* Wb,
                     cudaStream_t st) {
    if (n_items <= 0) return;
    SGL_COUNT(1);
    k_cells_xi<<<n_items, 256, 0, st>>>(g, edges, items, K, Gm, W, R, beta, tang, kp, nkp, mm, Hx, lx, Wb);
}

void launch_cells_xi_tail(const double* kp, int nkp, double coef, double Rm, double* lx, cudaStream_t st) {
    SGL_COUNT(1);
    k_cells_xi_tail<<<1, 64, 0, st>>>(kp, nkp, coef, Rm, lx);
}

void launch_cells_xi_flags(const double* Hx, int nbins, int mm, int nkp, unsigned char* flags, cudaStream_t st) {
    const long long n = (long long)nbins * (mm + 1);
    SGL_COUNT(1);
    k_cells_xi_flags<<<(int)((n + 255) / 256), 256, 0, st>>>(Hx, nbins, mm, nkp, flags);
}

void launch_cells_xi_rows(const double* Hx, int mm, int nkp, int m, const int* idx, int nidx, const double* cen,
                          int ngc, int cen_axis, const double* lxm, const double* sw, double* A, cudaStream_t st) {
    const long long n = std::max<long long>((long long)nidx * nkp, 64);
    SGL_COUNT(1);
    k_cells_xi_rows<<<(int)((n + 255) / 256), 256, 0, st>>>(Hx, mm, nkp, m, idx, nidx, cen, ngc, cen_axis, lxm, sw, A);
}

int cells_gram_parts(long long nrows, int chunk) { return (int)((nrows + chunk - 1) / chunk); }

void launch_cells_gram(const double* A, long long nrows, int nkp, int chunk, double* part, double* Gram, cudaStream_t st) {
    const int np = cells_gram_parts(nrows, chunk);
    SGL_COUNT(2);
    k_cells_gram<<<np, 256, 8 * chunk * nkp, st>>>(A, nrows, nkp, chunk, part);
    k_cells_gram_sum<<<(nkp * nkp + 255) / 256, 256, 0, st>>>(part, np, nkp, Gram);
}

void launch_cells_project(const double* A, long long nrows, int nkp, const double* V, int nkeep, double* rows,
                          cudaStream_t st) {
    SGL_COUNT(1);
    k_cells_project<<<(int)((nrows + 127) / 128), 128, 8 * nkp * nkeep, st>>>(A, nrows, nkp, V, nkeep, rows);
}

}  // namespace sgl
