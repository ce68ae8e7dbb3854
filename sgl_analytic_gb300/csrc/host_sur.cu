// Surrogate + judge production sweep: the instance table and its planes (sgl_sur_set), the judge
// pass over the ensemble's node outputs (sgl_sur_judge), the finishing pass that takes the batched
// solver's exact values for the planes sent back (sgl_sur_finish) and the inversion to dP/dln mu
// (sgl_sur_pdf).  Kernels: sursweep.cu (assembly), cfbatch.cu (Phi and the inversion).
//
// No counterpart in the reference.
#include "host.cuh"

struct SurState {
    int n_inst = 0, n_planes = 0, nq = 0, max_nk = 0;
    long long total_k = 0;
    std::vector<CfbInst> inst;
    std::vector<SurPlane> planes;
};

void sur_state_free(SurState* s) { delete s; }

namespace sglh {
namespace {

sgl_status sur_launch(sgl_ctx* ctx, bool judge, const float* Y, int members, double shift, double scale, double tau) {
    SurState& S = *ctx->sur;
    DBUF(lnphi, double2, "sur_lnphi", std::max<long long>(1, S.total_k));
    DBUF(dis, unsigned int, "sur_dis", 2LL * S.n_planes);
    DBUF(range, int, "sur_range", 2LL * S.n_planes);          // first indices, then ends
    if (judge) {
        CK(cudaMemsetAsync(dis, 0, sizeof(unsigned int) * 2 * (size_t)S.n_planes, ctx->stream));
        CK(cudaMemsetAsync(range, 0x7f, sizeof(int) * (size_t)S.n_planes, ctx->stream));   // 0x7f7f7f7f: none
        CK(cudaMemsetAsync(range + S.n_planes, 0, sizeof(int) * (size_t)S.n_planes, ctx->stream));
    }
    launch_sur_sum(judge, (const CfbInst*)ctx->arena.find("sur_inst"), S.n_inst, S.max_nk,
                   (const SurPlane*)ctx->arena.find("sur_planes"), Y, 2LL * S.nq * S.n_planes, members, S.nq, (float)shift,
                   (float)scale, (float)tau, (const double2*)ctx->arena.find("cfb_lnphi"), lnphi, dis, range, range + S.n_planes, ctx->stream);
    CKLAUNCH();
    return SGL_OK;
}

sgl_status check_Y(sgl_ctx* ctx, const float* Y, int members, double shift, double scale) {
    if (!ctx->sur) return fail(ctx, SGL_ERR_STATE, "no surrogate sweep set (sgl_sur_set)");
    if (!Y || members < 1 || members > 4) return fail(ctx, SGL_ERR_VALUE, "surrogate outputs: NULL or members not in 1..4");
    if (!std::isfinite(shift) || !(scale > 0) || !std::isfinite(scale)) return fail(ctx, SGL_ERR_VALUE, "invalid output scaling");
    return SGL_OK;
}

}  // namespace
}  // namespace sglh

extern "C" {

sgl_status sgl_sur_set(sgl_ctx* ctx, int n_inst, const int32_t* inst_plane0, const int32_t* nk, const double* dk,
                       const double* s, const double* dz, const double* mu1, const double* mu2, const double* lnq0,
                       const double* hq, int nq) {
    if (!ctx) return SGL_ERR_VALUE;
    if (n_inst < 1 || !inst_plane0 || !nk || !dk || !s || !dz || !mu1 || !mu2 || !lnq0 || !hq || nq < 4)
        return fail(ctx, SGL_ERR_VALUE, "sgl_sur_set: invalid sizes or NULL arrays (nq >= 4)");
    if (inst_plane0[0] != 0) return fail(ctx, SGL_ERR_VALUE, "sgl_sur_set: inst_plane0[0] must be 0");
    const int n_planes = inst_plane0[n_inst];
    for (int i = 0; i < n_inst; ++i) {
        if (inst_plane0[i + 1] <= inst_plane0[i]) return fail(ctx, SGL_ERR_VALUE, "sgl_sur_set: an instance has no plane");
        if (nk[i] < 2 || !(dk[i] > 0) || !std::isfinite(dk[i]))
            return fail(ctx, SGL_ERR_VALUE, "sgl_sur_set: invalid k grid of instance " + std::to_string(i));
    }
    for (int p = 0; p < n_planes; ++p)
        if (!(s[p] >= 0) || !std::isfinite(s[p]) || !(dz[p] >= 0) || !std::isfinite(dz[p]) || !std::isfinite(lnq0[p]) ||
            !(hq[p] > 0) || !std::isfinite(hq[p]) || !(mu1[p] > 0) || !std::isfinite(mu1[p]) || !(mu2[p] > 0) ||
            !std::isfinite(mu2[p]))
            return fail(ctx, SGL_ERR_VALUE, "sgl_sur_set: invalid plane " + std::to_string(p));
    CK(cudaSetDevice(ctx->device));
    CKS(sync_stream(ctx));
    if (ctx->sur) sur_state_free(ctx->sur);
    ctx->sur = new SurState();
    SurState& S = *ctx->sur;
    S.n_inst = n_inst; S.n_planes = n_planes; S.nq = nq;
    S.inst.resize((size_t)n_inst);
    long long koff = 0;
    for (int i = 0; i < n_inst; ++i) {
        CfbInst& I = S.inst[(size_t)i];
        I = CfbInst{};
        I.p0 = inst_plane0[i]; I.p1 = inst_plane0[i + 1];
        I.k_off = koff; I.nk = nk[i]; I.dk = dk[i]; I.vp_slot = -1;
        koff += nk[i];
        S.max_nk = std::max(S.max_nk, nk[i]);
    }
    S.total_k = koff;
    S.planes.resize((size_t)n_planes);
    for (int p = 0; p < n_planes; ++p)
        S.planes[(size_t)p] = SurPlane{s[p], dz[p], lnq0[p], hq[p], std::log(0.5 * mu2[p]), mu2[p] / (2.0 * mu1[p]), -1, 0, 0};
    std::vector<long long> k_offs((size_t)n_inst + 1);
    for (int i = 0; i < n_inst; ++i) k_offs[(size_t)i] = S.inst[(size_t)i].k_off;
    k_offs[(size_t)n_inst] = koff;
    DBUF(d_inst, CfbInst, "sur_inst", n_inst);
    DBUF(d_koffs, long long, "sur_koffs", n_inst + 1);
    DBUF(d_planes, SurPlane, "sur_planes", n_planes);
    CKS(upload(ctx, d_inst, S.inst.data(), S.inst.size()));
    CKS(upload(ctx, d_koffs, k_offs.data(), k_offs.size()));
    CKS(upload(ctx, d_planes, S.planes.data(), S.planes.size()));
    return sync_stream(ctx);
}

sgl_status sgl_sur_judge(sgl_ctx* ctx, const float* Y, int members, double shift, double scale, double tau,
                         float* dis_out, int32_t* band_out) {
    if (!ctx) return SGL_ERR_VALUE;
    CKS(check_Y(ctx, Y, members, shift, scale));
    if (!dis_out || !band_out || !(tau >= 0)) return fail(ctx, SGL_ERR_VALUE, "sgl_sur_judge: NULL output or invalid threshold");
    CK(cudaSetDevice(ctx->device));
    SurState& S = *ctx->sur;
    for (auto& P : S.planes) { P.exact_off = -1; P.exact_lo = 0; P.exact_nk = 0; }
    DBUF(d_planes, SurPlane, "sur_planes", S.n_planes);
    CKS(upload(ctx, d_planes, S.planes.data(), S.planes.size()));
    CKS(sur_launch(ctx, true, Y, members, shift, scale, tau));
    CK(cudaMemcpyAsync(dis_out, ctx->arena.find("sur_dis"), sizeof(float) * 2 * (size_t)S.n_planes, cudaMemcpyDeviceToHost,
                       ctx->stream));
    std::vector<int32_t> r(2 * (size_t)S.n_planes);
    CK(cudaMemcpyAsync(r.data(), ctx->arena.find("sur_range"), sizeof(int) * r.size(), cudaMemcpyDeviceToHost, ctx->stream));
    CKS(sync_stream(ctx));
    for (int p = 0; p < S.n_planes; ++p) {
        const int e = r[(size_t)S.n_planes + p];
        band_out[2 * (size_t)p] = e > 0 ? r[(size_t)p] : 0;
        band_out[2 * (size_t)p + 1] = e;
    }
    return SGL_OK;
}

sgl_status sgl_sur_finish(sgl_ctx* ctx, const float* Y, int members, double shift, double scale,
                          const int32_t* exact_inst, const int32_t* exact_lo) {
    if (!ctx) return SGL_ERR_VALUE;
    CKS(check_Y(ctx, Y, members, shift, scale));
    if (!exact_inst) return fail(ctx, SGL_ERR_VALUE, "sgl_sur_finish: NULL exact_inst");
    CK(cudaSetDevice(ctx->device));
    SurState& S = *ctx->sur;
    bool any = false;
    for (int i = 0; i < S.n_inst; ++i) {
        const CfbInst& I = S.inst[(size_t)i];
        for (int p = I.p0; p < I.p1; ++p) {
            const int e = exact_inst[p];
            SurPlane& P = S.planes[(size_t)p];
            P.exact_off = -1;
            P.exact_lo = 0;
            P.exact_nk = 0;
            if (e < 0) continue;
            if (!ctx->cfb || e >= cfb_n_inst(ctx->cfb))
                return fail(ctx, SGL_ERR_VALUE, "sgl_sur_finish: plane " + std::to_string(p) + " names no solved instance");
            long long off;
            int enk;
            double edk, ek0;
            cfb_inst_grid(ctx->cfb, e, &off, &enk, &edk, &ek0);
            const int lo = exact_lo ? exact_lo[p] : 0;
            if (lo < 0 || (long long)lo + enk > I.nk || edk != I.dk || ek0 != (double)lo * I.dk)
                return fail(ctx, SGL_ERR_VALUE, "sgl_sur_finish: plane " + std::to_string(p) + "'s exact k points differ");
            P.exact_off = off;
            P.exact_lo = lo;
            P.exact_nk = enk;
            any = true;
        }
    }
    if (any && !ctx->arena.find("cfb_lnphi")) return fail(ctx, SGL_ERR_STATE, "sgl_sur_finish: exact planes not solved");
    DBUF(d_planes, SurPlane, "sur_planes", S.n_planes);
    CKS(upload(ctx, d_planes, S.planes.data(), S.planes.size()));
    CKS(sur_launch(ctx, false, Y, members, shift, scale, 0.0));
    return SGL_OK;
}

sgl_status sgl_sur_nodes_exact(sgl_ctx* ctx, int n, const int32_t* planes, const int32_t* node_lo, float* Y,
                               int members, double shift, double scale) {
    if (!ctx) return SGL_ERR_VALUE;
    CKS(check_Y(ctx, Y, members, shift, scale));
    if (n < 1 || !planes) return fail(ctx, SGL_ERR_VALUE, "sgl_sur_nodes_exact: no planes");
    CK(cudaSetDevice(ctx->device));
    SurState& S = *ctx->sur;
    if (!ctx->cfb || cfb_n_inst(ctx->cfb) != n || !ctx->arena.find("cfb_lnphi"))
        return fail(ctx, SGL_ERR_STATE, "sgl_sur_nodes_exact: the batched solver does not hold one solved instance per plane");
    for (int j = 0; j < n; ++j) {
        const int p = planes[j];
        if (p < 0 || p >= S.n_planes) return fail(ctx, SGL_ERR_VALUE, "sgl_sur_nodes_exact: plane out of range");
        long long off;
        int enk;
        double edk, ek0;
        cfb_inst_grid(ctx->cfb, j, &off, &enk, &edk, &ek0);
        const SurPlane& P = S.planes[(size_t)p];
        const int lo = node_lo ? node_lo[j] : 0;
        if (lo < 0 || lo + enk > S.nq || edk != P.hq || !(P.dz > 0))
            return fail(ctx, SGL_ERR_VALUE, "sgl_sur_nodes_exact: instance " + std::to_string(j) + " is not on plane " +
                                                std::to_string(p) + "'s node grid");
    }
    std::vector<int> lo_v((size_t)n, 0);
    if (node_lo) for (int j = 0; j < n; ++j) lo_v[(size_t)j] = node_lo[j];
    DBUF(d_pl, int, "sur_exact_planes", n);
    DBUF(d_lo, int, "sur_exact_lo", n);
    CKS(upload(ctx, d_pl, (const int*)planes, (size_t)n));
    CKS(upload(ctx, d_lo, lo_v.data(), (size_t)n));
    launch_sur_nodes_exact(n, d_pl, d_lo, (const CfbInst*)ctx->arena.find("cfb_inst"), (const double2*)ctx->arena.find("cfb_lnphi"),
                           (const SurPlane*)ctx->arena.find("sur_planes"), S.nq, Y, 2LL * S.nq * S.n_planes, members,
                           (float)shift, (float)scale, ctx->stream);
    CKLAUNCH();
    return sync_stream(ctx);
}

sgl_status sgl_sur_pdf(sgl_ctx* ctx, int precision, const double* lnmu, int n_lnmu, double* P_out, double* lnphi_out) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->sur) return fail(ctx, SGL_ERR_STATE, "no surrogate sweep set (sgl_sur_set)");
    if (precision != SGL_FP64 && precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    if (n_lnmu < 1 || !lnmu || !P_out) return fail(ctx, SGL_ERR_VALUE, "sgl_sur_pdf: invalid ln mu grid or output");
    for (int m = 0; m < n_lnmu; ++m) if (!std::isfinite(lnmu[m])) return fail(ctx, SGL_ERR_VALUE, "non-finite ln mu");
    CK(cudaSetDevice(ctx->device));
    SurState& S = *ctx->sur;
    DBUF(lnphi, double2, "sur_lnphi", std::max<long long>(1, S.total_k));
    void* phi = ctx->arena.get("sur_phi", (size_t)std::max<long long>(1, S.total_k) * 2 * (precision == SGL_FP64 ? 8 : 4));
    DBUF(d_lnmu, double, "sur_lnmu", n_lnmu);
    DBUF(d_P, double, "sur_P", (long long)S.n_inst * n_lnmu);
    if (!phi) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (sur phi)");
    CKS(upload(ctx, d_lnmu, lnmu, (size_t)n_lnmu));
    launch_cfb_pdf(precision, (const CfbInst*)ctx->arena.find("sur_inst"), S.n_inst, lnphi, S.total_k,
                   (const long long*)ctx->arena.find("sur_koffs"), phi, d_lnmu, n_lnmu, d_P, ctx->stream);
    CKLAUNCH();
    CK(cudaMemcpyAsync(P_out, d_P, (size_t)S.n_inst * n_lnmu * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (lnphi_out)
        CK(cudaMemcpyAsync(lnphi_out, lnphi, (size_t)S.total_k * 16, cudaMemcpyDeviceToHost, ctx->stream));
    CKS(sync_stream(ctx));
    for (long long e = 0; e < (long long)S.n_inst * n_lnmu; ++e)
        if (!std::isfinite(P_out[e])) return fail(ctx, SGL_ERR_NONFINITE, "surrogate sweep PDF returned non-finite values");
    return SGL_OK;
}

}  // extern "C"
