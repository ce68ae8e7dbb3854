// Surrogate + judge assembly of instance log-CFs (the production sweep of the learned per-plane
// log-CF).  Per instance and k-point, the sum over the instance's planes of dz H(s k), H from the
// ensemble members' outputs at the plane's ln q nodes.  The judge pass also reduces, per plane, the
// members' largest disagreement (as is, and weighted by |Phi| of the surrogate sum) and the band of k
// points from the first to the last whose weighted disagreement exceeds the threshold; the finishing
// pass takes the exact solver's values on each plane's band.  Planes can also be sent back for exact
// values at their nodes (k_sur_nodes_exact), which then replace the members' outputs there.
//
// The members learn the residual of ln H over the two-moment form
//     H0(q) = -(mu2 / 2) q^2 / (1 - i q Sbar),   Sbar = mu2 / (2 mu1),
// which has the exact small-q (-mu2 q^2 / 2) and large-q (-i mu1 q) behaviour of H:
//     ln |H| = r0 + ln(mu2 / 2) + 2 ln q - ln(1 + (q Sbar)^2) / 2,   arg(-H) = r1 + atan(q Sbar).
//
// No counterpart in the reference.
#include <climits>

#include "common.cuh"
#include "kernels.cuh"

namespace sgl {
namespace {

constexpr int kSurThreads = 256;

struct SurArgs {
    const CfbInst* inst;
    const SurPlane* planes;
    const float* Y;                      // [member][plane][node] (y0, y1): r0 = y0 scale + shift, r1 = y1 scale
    long long y_member_stride;           // floats per member
    int members, nq;
    float shift, scale;
    float tau;                           // judge: threshold of the weighted disagreement
    const double2* exact;                // the exact solver's ln Phi per plane (finishing pass)
    double2* lnphi;                      // out: per instance and k
    unsigned int* dis;                   // judge: per plane (max dz spread, max |Phi| dz spread) as float bits
    int* first;                          // judge: per plane, the first k index above tau (stays large: none)
    int* last;                           // judge: per plane, 1 + the last k index above tau (stays 0: none)
};

// (r0, r1) of one member at node coordinate x = (ln q - lnq0) / hq: 4-point Lagrange interpolation
// between nodes (one-sided at the ends); below the first node r (q / q0) (r -> 0 as q -> 0: H0 holds
// the exact small-q limit)
__device__ __forceinline__ float2 sur_r(const float* __restrict__ Yp, int nq, float x, float dl, float scale,
                                        float shift) {
    if (x < 0.f) {
        const float2 v = *reinterpret_cast<const float2*>(Yp);
        const float f = expf(dl);
        return make_float2(fmaf(v.x, scale, shift) * f, v.y * scale * f);
    }
    int j = (int)floorf(x);
    j = max(1, min(j, nq - 3));
    const float u = x - (float)j;
    const float um = u + 1.f, u1 = u - 1.f, u2 = u - 2.f;
    const float w0 = -u * u1 * u2 * (1.f / 6.f);
    const float w1 = um * u1 * u2 * 0.5f;
    const float w2 = -um * u * u2 * 0.5f;
    const float w3 = um * u * u1 * (1.f / 6.f);
    const float2* n = reinterpret_cast<const float2*>(Yp) + (j - 1);
    const float2 a = n[0], b = n[1], c = n[2], d = n[3];
    const float y0 = fmaf(w0, a.x, fmaf(w1, b.x, fmaf(w2, c.x, w3 * d.x)));
    const float y1 = fmaf(w0, a.y, fmaf(w1, b.y, fmaf(w2, c.y, w3 * d.y)));
    return make_float2(fmaf(y0, scale, shift), y1 * scale);
}

// H of plane P (index p) at k: members' mean and spread 2 max_m |H_m - mean|
__device__ __forceinline__ void sur_plane(const SurArgs& a, const SurPlane& P, long long p, double k, float2& mean,
                                          float& spread) {
    const double lq = log(P.s * k);
    const float x = (float)((lq - P.lnq0) / P.hq);
    const float dl = (float)(lq - P.lnq0);
    const float qs = (float)(exp(lq) * P.sbar);
    const float b0 = (float)(P.lnmu2h + 2.0 * lq) - 0.5f * log1pf(qs * qs);
    const float b1 = atanf(qs);
    float hr[4], hi[4];
    const int M = min(a.members, 4);
    float mr = 0.f, mi = 0.f;
    for (int m = 0; m < M; ++m) {
        const float2 r = sur_r(a.Y + (long long)m * a.y_member_stride + p * 2LL * a.nq, a.nq, x, dl, a.scale, a.shift);
        const float e = expf(r.x + b0);
        float s, c;
        sincosf(r.y + b1, &s, &c);
        hr[m] = -e * c;
        hi[m] = -e * s;
        mr += hr[m];
        mi += hi[m];
    }
    mr /= (float)M;
    mi /= (float)M;
    float sp = 0.f;
    for (int m = 0; m < M; ++m) sp = fmaxf(sp, hypotf(hr[m] - mr, hi[m] - mi));
    mean = make_float2(mr, mi);
    spread = 2.f * sp;
}

template <bool JUDGE>
__global__ void __launch_bounds__(kSurThreads) k_sur_sum(SurArgs a) {
    const CfbInst I = a.inst[blockIdx.y];
    const int n = blockIdx.x * kSurThreads + threadIdx.x;
    const bool live = n < I.nk;
    const double k = (double)n * I.dk;
    double sr = 0.0, si = 0.0;
    for (int p = I.p0; p < I.p1; ++p) {
        const SurPlane P = a.planes[p];
        if (!JUDGE && P.exact_off >= 0 && n >= P.exact_lo && n < P.exact_lo + P.exact_nk) {
            const double2 e = a.exact[P.exact_off + (n - P.exact_lo)];
            sr += e.x;
            si += e.y;
            continue;
        }
        if (live && n > 0) {
            float2 h;
            float sp;
            sur_plane(a, P, p, k, h, sp);
            sr = fma(P.dz, (double)h.x, sr);
            si = fma(P.dz, (double)h.y, si);
        }
    }
    if (live) a.lnphi[I.k_off + n] = make_double2(sr, si);
    if (JUDGE) {
        const float phim = live ? (float)exp(sr) : 0.f;
        const int lane = threadIdx.x & 31;
        for (int p = I.p0; p < I.p1; ++p) {
            const SurPlane P = a.planes[p];
            float du = 0.f;
            if (live && n > 0) {
                float2 h;
                sur_plane(a, P, p, k, h, du);
                du *= (float)P.dz;
            }
            float dw = du * phim;
            const bool above = dw > a.tau;
            int first = above ? n : INT_MAX, last = above ? n + 1 : 0;
            for (int o = 16; o > 0; o >>= 1) {
                du = fmaxf(du, __shfl_xor_sync(0xffffffffu, du, o));
                dw = fmaxf(dw, __shfl_xor_sync(0xffffffffu, dw, o));
                first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
                last = max(last, __shfl_xor_sync(0xffffffffu, last, o));
            }
            if (lane == 0) {
                atomicMax(a.dis + 2LL * p, __float_as_uint(du));            // non-negative: bits order as values
                atomicMax(a.dis + 2LL * p + 1, __float_as_uint(dw));
                if (last > 0) {
                    atomicMin(a.first + p, first);
                    atomicMax(a.last + p, last);
                }
            }
        }
    }
}

// Planes sent back for exact node values: instance j of the batched solver holds plane planes[j]'s
// cells on the k points of its nodes node_lo[j] .. node_lo[j] + nk_j - 1 (q_node / s), so its ln Phi is
// dz H(q_node); the node's residual over the two-moment form, normalised, replaces every member's output
__global__ void k_sur_nodes_exact(long long total, const int* __restrict__ planes, const int* __restrict__ node_lo,
                                  const CfbInst* __restrict__ ci, const double2* __restrict__ lnphi,
                                  const SurPlane* __restrict__ sp, int nq, float* __restrict__ Y, long long stride,
                                  int members, float shift, float scale) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int j = (int)(e / nq), t = (int)(e - (long long)j * nq);
    const CfbInst I = ci[j];
    if (t >= I.nk) return;
    const int p = planes[j];
    const int node = node_lo[j] + t;
    const SurPlane P = sp[p];
    const double2 L = lnphi[I.k_off + t];
    const double hr = L.x / P.dz, hi = L.y / P.dz;
    const double lq = P.lnq0 + node * P.hq;
    const double qs = exp(lq) * P.sbar;
    const double r0 = 0.5 * log(hr * hr + hi * hi) - (P.lnmu2h + 2.0 * lq - 0.5 * log1p(qs * qs));
    const double r1 = atan2(-hi, -hr) - atan(qs);
    const float y0 = (float)((r0 - shift) / scale), y1 = (float)(r1 / scale);
    for (int m = 0; m < members; ++m) {
        float* o = Y + m * stride + ((long long)p * nq + node) * 2;
        o[0] = y0;
        o[1] = y1;
    }
}

}  // namespace

void launch_sur_sum(bool judge, const CfbInst* inst, int n_inst, int max_nk, const SurPlane* planes, const float* Y,
                    long long y_member_stride, int members, int nq, float shift, float scale, float tau,
                    const double2* exact, double2* lnphi, unsigned int* dis, int* first, int* last, cudaStream_t st) {
    SurArgs a{inst, planes, Y, y_member_stride, members, nq, shift, scale, tau, exact, lnphi, dis, first, last};
    const dim3 grid((unsigned)ceil_div(max_nk, kSurThreads), (unsigned)n_inst);
    if (judge) k_sur_sum<true><<<grid, kSurThreads, 0, st>>>(a);
    else k_sur_sum<false><<<grid, kSurThreads, 0, st>>>(a);
    SGL_COUNT(1);
}

void launch_sur_nodes_exact(int n, const int* planes, const int* node_lo, const CfbInst* cfb_inst,
                            const double2* cfb_lnphi, const SurPlane* sp, int nq, float* Y, long long y_member_stride,
                            int members, float shift, float scale, cudaStream_t st) {
    const long long total = (long long)n * nq;
    k_sur_nodes_exact<<<(unsigned)ceil_div(total, 256), 256, 0, st>>>(total, planes, node_lo, cfb_inst, cfb_lnphi, sp,
                                                                     nq, Y, y_member_stride, members, shift, scale);
    SGL_COUNT(1);
}

}  // namespace sgl
