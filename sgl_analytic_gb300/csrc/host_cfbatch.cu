// Batched plain CF solver: many instances (cosmology x source redshift x closure) with uneven plane
// counts and k grids, solved by one persistent launch, then inverted to dP/dln mu.  The device work
// list, the tile autotuner and the CUDA-graph capture of a whole step live here; the kernels are in
// cfbatch.cu.
//
// No counterpart in the reference, which solves one pipeline.run per instance
// (pipeline.py:114-274).
#include <chrono>
#include <cmath>
#include <numeric>

#include "host.cuh"

struct CfbState {
    int n_inst = 0, n_planes = 0, nstate = 0;
    int shape_class = 0;                       // log2 buckets of the largest k grid and the mean cells
    long long n_cells = 0, total_k = 0;
    std::vector<CfbInst> inst;
    std::vector<double> cost;                  // per instance: cells x k (+ chain) work
    std::vector<int> order;                    // instances by cost, longest first
    // tuned launch shape per precision: k-points per work item (= threads per CTA), CTAs per SM
    int kt[2] = {128, 128}, cps[2] = {0, 0};
    bool tuned[2] = {false, false};
    // the captured step per (precision, n_lnmu) and its item list
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_nm[2] = {0, 0}, graph_kt[2] = {0, 0}, graph_cps[2] = {0, 0};
};

void cfb_state_free(CfbState* s) {
    if (!s) return;
    for (auto& g : s->graph) if (g) cudaGraphExecDestroy(g);
    delete s;
}

int cfb_n_inst(const CfbState* s) { return s ? s->n_inst : 0; }

void cfb_inst_grid(const CfbState* s, int i, long long* k_off, int* nk, double* dk, double* k0) {
    const CfbInst& I = s->inst[(size_t)i];
    *k_off = I.k_off;
    *nk = I.nk;
    *dk = I.dk;
    *k0 = I.k0;
}

namespace sglh {
namespace {

// work items (instance, k tile) for a tile width, instances in `order`
std::vector<int2> cfb_items(const CfbState& S, int kt, const std::vector<int>& order) {
    std::vector<int2> items;
    for (int i : order) {
        const int tiles = (S.inst[(size_t)i].nk + kt - 1) / kt;
        for (int t = 0; t < tiles; ++t) items.push_back(make_int2(i, t));
    }
    return items;
}

sgl_status cfb_launch(sgl_ctx* ctx, int precision, int kt, int cps, const std::vector<int2>& items,
                      const std::string& tag) {
    CfbState& S = *ctx->cfb;
    DBUF(d_items, int2, "cfb_items_" + tag, std::max<size_t>(1, items.size()));
    CKS(upload(ctx, d_items, items.data(), items.size()));
    DBUF(counter, int, "cfb_counter", 1);
    DBUF(out, double2, "cfb_lnphi", std::max<long long>(1, S.total_k));
    const int res = cfb_resident_ctas(precision, kt);
    if (res < 1) return fail(ctx, SGL_ERR_CUDA, "batched CF kernel: no resident CTA for this tile width");
    const int ctas = kNumSMs * std::max(1, std::min(cps, res));
    launch_cfb_persistent(precision, kt, ctas, (const CfbInst*)ctx->arena.find("cfb_inst"), d_items, (int)items.size(),
                          counter, (const long long*)ctx->arena.find("cfb_pcells"),
                          (const double*)ctx->arena.find("cfb_kap"), (const double*)ctx->arena.find("cfb_w"),
                          (const float*)ctx->arena.find("cfb_kh"), (const float*)ctx->arena.find("cfb_kl"),
                          (const float*)ctx->arena.find("cfb_wf"), (const double*)ctx->arena.find("cfb_vpD"),
                          (const double*)ctx->arena.find("cfb_vpK"), (const double*)ctx->arena.find("cfb_vpw"),
                          S.nstate, out, ctx->stream);
    CKLAUNCH();
    return SGL_OK;
}

// The launch shape.  FP64 (the parity path, whose FP64 pipe makes every term slow here) takes a fixed
// shape: 128 k-points per item, as many CTAs per SM as fit.  The mixed path times each (tile width,
// CTAs per SM) allowed by occupancy on a sample of the batch and keeps the fastest: instances evenly
// spread in cost order (at most 256), then every s-th of their work items so that a timed launch holds
// about kTuneTerms cell-k terms, the same fraction for every tile width; a tune costs about a second.
sgl_status cfb_tune(sgl_ctx* ctx, int precision) {
    CfbState& S = *ctx->cfb;
    const int P = precision == SGL_FP64 ? 0 : 1;
    if (precision == SGL_FP64) {
        S.kt[P] = 128;
        S.cps[P] = std::max(1, cfb_resident_ctas(precision, 128));
        S.tuned[P] = true;
        ctx->cfb_shapes[2LL * S.shape_class + P] = {S.kt[P], S.cps[P]};
        return SGL_OK;
    }
    constexpr double kTuneTerms = 2e10;
    std::vector<int> sample;
    const size_t stride = std::max<size_t>(1, S.order.size() / 256);
    double scost = 0.0;
    for (size_t i = 0; i < S.order.size(); i += stride) {
        sample.push_back(S.order[i]);
        scost += S.cost[(size_t)S.order[i]];
    }
    const size_t istride = scost > kTuneTerms ? (size_t)std::ceil(scost / kTuneTerms) : 1;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    double best = 1e300;
    for (int kt : {64, 128, 256}) {
        const int res = cfb_resident_ctas(precision, kt);
        std::vector<int2> items = cfb_items(S, kt, sample);
        if (istride > 1) {
            std::vector<int2> sub;
            for (size_t q = 0; q < items.size(); q += istride) sub.push_back(items[q]);
            items.swap(sub);
        }
        for (int cps : {1, 2, 4, 8, 16}) {
            if (cps > res) continue;
            CKS(cfb_launch(ctx, precision, kt, cps, items, "tune"));       // warm
            cudaEventRecord(a, ctx->stream);
            CKS(cfb_launch(ctx, precision, kt, cps, items, "tune"));
            cudaEventRecord(b, ctx->stream);
            CK(cudaEventSynchronize(b));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (ms < best) { best = ms; S.kt[P] = kt; S.cps[P] = cps; }
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    S.tuned[P] = true;
    ctx->cfb_shapes[2LL * S.shape_class + P] = {S.kt[P], S.cps[P]};
    return sync_stream(ctx);
}

// Validates a batch's instance table and uploads it (instances, k offsets, plane offsets, vp chain
// tables); the cells follow from the caller
sgl_status cfb_tables(sgl_ctx* ctx, int n_inst, const int32_t* inst_plane0, const int64_t* plane_cells,
                      const int32_t* nk, const double* dk, const int32_t* closure, const double* V, int nstate,
                      const double* vp_D, const double* vp_K, const double* vp_w) {
    if (!ctx) return SGL_ERR_VALUE;
    if (n_inst < 1 || !inst_plane0 || !plane_cells || !nk || !dk || !closure || !V)
        return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: invalid sizes or NULL arrays");
    if (inst_plane0[0] != 0) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: inst_plane0[0] must be 0");
    const int n_planes = inst_plane0[n_inst];
    if (n_planes < 1 || plane_cells[0] != 0) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: invalid plane offsets");
    for (int i = 0; i < n_inst; ++i) {
        if (inst_plane0[i + 1] <= inst_plane0[i]) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: an instance has no plane");
        if (nk[i] < 2 || !(dk[i] > 0) || !std::isfinite(dk[i]) || !std::isfinite(V[i]) || (closure[i] != 0 && closure[i] != 1))
            return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: invalid k grid, V or closure of instance " + std::to_string(i));
    }
    for (int p = 0; p < n_planes; ++p)
        if (plane_cells[p + 1] < plane_cells[p]) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: plane_cells not ascending");
    const long long nc = plane_cells[n_planes];
    if (nc < 1) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: no cells");
    int n_vp = 0;
    for (int i = 0; i < n_inst; ++i) n_vp += closure[i] == 1;
    if (n_vp > 0 && (nstate < 2 || nstate > 8 || !vp_D || !vp_K || !vp_w))
        return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: vp instances need 2..8 chain states and their tables");
    CK(cudaSetDevice(ctx->device));
    CKS(sync_stream(ctx));
    if (ctx->cfb) cfb_state_free(ctx->cfb);
    ctx->cfb = new CfbState();
    CfbState& S = *ctx->cfb;
    S.n_inst = n_inst; S.n_planes = n_planes; S.nstate = n_vp > 0 ? nstate : 0; S.n_cells = nc;
    S.inst.resize((size_t)n_inst);
    S.cost.resize((size_t)n_inst);
    long long koff = 0;
    int slot = 0;
    std::vector<long long> k_offs((size_t)n_inst + 1, 0);
    for (int i = 0; i < n_inst; ++i) {
        CfbInst& I = S.inst[(size_t)i];
        I.p0 = inst_plane0[i]; I.p1 = inst_plane0[i + 1];
        I.c0 = plane_cells[I.p0]; I.c1 = plane_cells[I.p1];
        I.k_off = koff; I.nk = nk[i]; I.dk = dk[i]; I.V = V[i]; I.closure = closure[i];
        I.vp_slot = closure[i] == 1 ? slot++ : -1; I.geom = 0; I.k0 = 0.0;
        k_offs[(size_t)i] = koff;
        koff += nk[i];
        // work: cells x k, the chain about 2 S^2 cell-terms per plane
        S.cost[(size_t)i] = (double)nk[i] * ((double)(I.c1 - I.c0) + (closure[i] == 1 ? 2.0 * nstate * nstate * (I.p1 - I.p0) : 0.0));
    }
    k_offs[(size_t)n_inst] = koff;
    S.total_k = koff;
    // batches of the same shape class (largest k grid, mean cells per instance, both in powers of
    // two) reuse the launch shapes the autotuner found for the first of them
    {
        int max_nk = 0;
        for (int i = 0; i < n_inst; ++i) max_nk = std::max(max_nk, nk[i]);
        const int kb = (int)std::ceil(std::log2((double)max_nk));
        const int cb = (int)std::ceil(std::log2(std::max(1.0, (double)nc / n_inst)));
        S.shape_class = 100 * kb + cb;
        for (int q = 0; q < 2; ++q) {
            auto it = ctx->cfb_shapes.find(2LL * S.shape_class + q);
            if (it != ctx->cfb_shapes.end()) { S.kt[q] = it->second.first; S.cps[q] = it->second.second; S.tuned[q] = true; }
        }
    }
    S.order.resize((size_t)n_inst);
    std::iota(S.order.begin(), S.order.end(), 0);
    std::stable_sort(S.order.begin(), S.order.end(), [&](int x, int y) { return S.cost[(size_t)x] > S.cost[(size_t)y]; });
    DBUF(d_inst, CfbInst, "cfb_inst", n_inst);
    DBUF(d_koffs, long long, "cfb_koffs", n_inst + 1);
    DBUF(d_pc, long long, "cfb_pcells", n_planes + 1);
    DBUF(d_vpD, double, "cfb_vpD", std::max(1, n_planes * std::max(1, S.nstate)));
    DBUF(d_vpK, double, "cfb_vpK", std::max(1, n_vp * S.nstate * S.nstate));
    DBUF(d_vpw, double, "cfb_vpw", std::max(1, n_vp * S.nstate));
    CKS(upload(ctx, d_inst, S.inst.data(), S.inst.size()));
    CKS(upload(ctx, d_koffs, k_offs.data(), k_offs.size()));
    CKS(upload(ctx, d_pc, (const long long*)plane_cells, (size_t)n_planes + 1));
    if (n_vp > 0) {
        CKS(upload(ctx, d_vpD, vp_D, (size_t)n_planes * S.nstate));
        CKS(upload(ctx, d_vpK, vp_K, (size_t)n_vp * S.nstate * S.nstate));
        CKS(upload(ctx, d_vpw, vp_w, (size_t)n_vp * S.nstate));
    }
    return sync_stream(ctx);          // k_offs goes out of scope
}

}  // namespace
}  // namespace sglh

extern "C" {

sgl_status sgl_cfb_set(sgl_ctx* ctx, int n_inst, const int32_t* inst_plane0, const int64_t* plane_cells,
                       const double* kap, const double* w, const int32_t* nk, const double* dk, const int32_t* closure,
                       const double* V, int nstate, const double* vp_D, const double* vp_K, const double* vp_w) {
    if (!ctx) return SGL_ERR_VALUE;
    CKS(cfb_tables(ctx, n_inst, inst_plane0, plane_cells, nk, dk, closure, V, nstate, vp_D, vp_K, vp_w));
    CfbState& S = *ctx->cfb;
    const long long nc = S.n_cells;
    if (!kap || !w) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set: no cells");
    std::vector<float> kh((size_t)nc), kl((size_t)nc), wf((size_t)nc);
    for (long long c = 0; c < nc; ++c) {
        const ff f = ff_from_double(kap[c]);
        kh[(size_t)c] = f.hi; kl[(size_t)c] = f.lo; wf[(size_t)c] = (float)w[c];
    }
    DBUF(d_kap, double, "cfb_kap", nc);
    DBUF(d_w, double, "cfb_w", nc);
    DBUF(d_kh, float, "cfb_kh", nc);
    DBUF(d_kl, float, "cfb_kl", nc);
    DBUF(d_wf, float, "cfb_wf", nc);
    CKS(upload(ctx, d_kap, kap, (size_t)nc));
    CKS(upload(ctx, d_w, w, (size_t)nc));
    CKS(upload(ctx, d_kh, kh.data(), kh.size()));
    CKS(upload(ctx, d_kl, kl.data(), kl.size()));
    CKS(upload(ctx, d_wf, wf.data(), wf.size()));
    return sync_stream(ctx);          // the host staging vectors go out of scope
}

sgl_status sgl_cfb_set_separable(sgl_ctx* ctx, int nm, int nb, const double* F, const double* g, int n_inst,
                                 const int32_t* inst_plane0, const int32_t* nk, const double* dk, const double* k0,
                                 int geom, const double* V, const double* u, const double* v) {
    if (!ctx) return SGL_ERR_VALUE;
    if (nm < 1 || nb < 1 || !F || !g || !u || !v || n_inst < 1 || !inst_plane0)
        return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set_separable: invalid template or NULL arrays");
    if (inst_plane0[0] != 0 || inst_plane0[n_inst] < 1) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set_separable: invalid plane offsets");
    const int n_planes = inst_plane0[n_inst];
    const long long per = (long long)nm * nb;
    std::vector<int64_t> pc((size_t)n_planes + 1);
    for (int p = 0; p <= n_planes; ++p) pc[(size_t)p] = per * p;
    std::vector<int32_t> closure((size_t)n_inst, 0);
    if (geom && !k0) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set_separable: log-spaced k points need k0");
    if (k0)
        for (int i = 0; i < n_inst; ++i)
            if (!std::isfinite(k0[i]) || (!geom && !(k0[i] >= 0)) || (geom && k0[i] + (nk[i] - 1) * dk[i] > 700.0))
                return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_set_separable: invalid k0");
    CKS(cfb_tables(ctx, n_inst, inst_plane0, pc.data(), nk, dk, closure.data(), V, 0, nullptr, nullptr, nullptr));
    const long long nc = ctx->cfb->n_cells;
    if (k0) {
        CfbState& S = *ctx->cfb;
        for (int i = 0; i < n_inst; ++i) {
            S.inst[(size_t)i].k0 = k0[i];
            S.inst[(size_t)i].geom = geom ? 1 : 0;
        }
        DBUF(d_inst, CfbInst, "cfb_inst", n_inst);
        CKS(upload(ctx, d_inst, S.inst.data(), S.inst.size()));
    }
    for (long long e = 0; e < per; ++e) if (!std::isfinite(F[e])) return fail(ctx, SGL_ERR_VALUE, "non-finite template F");
    for (int b = 0; b < nb; ++b) if (!std::isfinite(g[b])) return fail(ctx, SGL_ERR_VALUE, "non-finite template g");
    for (long long e = 0; e < (long long)n_planes * nm; ++e)
        if (!std::isfinite(u[e]) || !std::isfinite(v[e])) return fail(ctx, SGL_ERR_VALUE, "non-finite plane factors");
    DBUF(d_F, double, "cfb_tF", per);
    DBUF(d_g, double, "cfb_tg", nb);
    DBUF(d_u, double, "cfb_tu", (long long)n_planes * nm);
    DBUF(d_v, double, "cfb_tv", (long long)n_planes * nm);
    DBUF(d_kap, double, "cfb_kap", nc);
    DBUF(d_w, double, "cfb_w", nc);
    DBUF(d_kh, float, "cfb_kh", nc);
    DBUF(d_kl, float, "cfb_kl", nc);
    DBUF(d_wf, float, "cfb_wf", nc);
    CKS(upload(ctx, d_F, F, (size_t)per));
    CKS(upload(ctx, d_g, g, (size_t)nb));
    CKS(upload(ctx, d_u, u, (size_t)n_planes * nm));
    CKS(upload(ctx, d_v, v, (size_t)n_planes * nm));
    launch_cfb_fill_separable(nc, nm, nb, d_F, d_g, d_u, d_v, d_kap, d_w, d_kh, d_kl, d_wf, ctx->stream);
    CKLAUNCH();
    return sync_stream(ctx);
}

sgl_status sgl_cfb_tune(sgl_ctx* ctx, int precision, int* kt, int* ctas_per_sm) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->cfb) return fail(ctx, SGL_ERR_STATE, "sgl_cfb_tune: no batch set");
    if (precision != SGL_FP64 && precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    CK(cudaSetDevice(ctx->device));
    CKS(cfb_tune(ctx, precision));
    const int P = precision == SGL_FP64 ? 0 : 1;
    if (kt) *kt = ctx->cfb->kt[P];
    if (ctas_per_sm) *ctas_per_sm = ctx->cfb->cps[P];
    return SGL_OK;
}

sgl_status sgl_cfb_lnphi(sgl_ctx* ctx, int precision, double* out) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->cfb) return fail(ctx, SGL_ERR_STATE, "sgl_cfb_lnphi: no batch set");
    if (precision != SGL_FP64 && precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    CK(cudaSetDevice(ctx->device));
    CfbState& S = *ctx->cfb;
    const int P = precision == SGL_FP64 ? 0 : 1;
    if (!S.tuned[P]) CKS(cfb_tune(ctx, precision));
    const std::vector<int2> items = cfb_items(S, S.kt[P], S.order);
    CKS(cfb_launch(ctx, precision, S.kt[P], S.cps[P], items, "run"));
    if (out) CK(cudaMemcpyAsync(out, ctx->arena.find("cfb_lnphi"), (size_t)S.total_k * 16, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_stream(ctx);
}

sgl_status sgl_cfb_pdf(sgl_ctx* ctx, int precision, const double* lnmu, int n_lnmu, double* P_out, int use_graph,
                       double* ms_out) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->cfb) return fail(ctx, SGL_ERR_STATE, "sgl_cfb_pdf: no batch set");
    if (precision != SGL_FP64 && precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    if (n_lnmu < 1 || !lnmu || !P_out) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_pdf: invalid ln mu grid or output");
    for (int m = 0; m < n_lnmu; ++m) if (!std::isfinite(lnmu[m])) return fail(ctx, SGL_ERR_VALUE, "non-finite ln mu");
    CK(cudaSetDevice(ctx->device));
    CfbState& S = *ctx->cfb;
    for (const CfbInst& I : S.inst)
        if (I.k0 != 0.0 || I.geom) return fail(ctx, SGL_ERR_VALUE, "sgl_cfb_pdf: the inversion needs k grids n dk");
    const int P = precision == SGL_FP64 ? 0 : 1;
    if (!S.tuned[P]) CKS(cfb_tune(ctx, precision));
    // every buffer of the step exists before a capture (no allocation inside it)
    const std::vector<int2> items = cfb_items(S, S.kt[P], S.order);
    DBUF(d_items, int2, std::string("cfb_items_run") + (P ? "m" : "d"), std::max<size_t>(1, items.size()));
    DBUF(counter, int, "cfb_counter", 1);
    DBUF(lnphi, double2, "cfb_lnphi", std::max<long long>(1, S.total_k));
    void* phi = ctx->arena.get("cfb_phi", (size_t)std::max<long long>(1, S.total_k) * 2 * (P ? 4 : 8));
    DBUF(d_lnmu, double, "cfb_lnmu", n_lnmu);
    DBUF(d_P, double, "cfb_P", (long long)S.n_inst * n_lnmu);
    if (!phi) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (cfb phi)");
    const int res = cfb_resident_ctas(precision, S.kt[P]);
    const int ctas = kNumSMs * std::max(1, std::min(S.cps[P], std::max(1, res)));
    const cudaStream_t st = ctx->stream;
    auto enqueue = [&]() {
        launch_cfb_persistent(precision, S.kt[P], ctas, (const CfbInst*)ctx->arena.find("cfb_inst"), d_items,
                              (int)items.size(), counter, (const long long*)ctx->arena.find("cfb_pcells"),
                              (const double*)ctx->arena.find("cfb_kap"), (const double*)ctx->arena.find("cfb_w"),
                              (const float*)ctx->arena.find("cfb_kh"), (const float*)ctx->arena.find("cfb_kl"),
                              (const float*)ctx->arena.find("cfb_wf"), (const double*)ctx->arena.find("cfb_vpD"),
                              (const double*)ctx->arena.find("cfb_vpK"), (const double*)ctx->arena.find("cfb_vpw"),
                              S.nstate, lnphi, st);
        launch_cfb_pdf(precision, (const CfbInst*)ctx->arena.find("cfb_inst"), S.n_inst, lnphi, S.total_k,
                       (const long long*)ctx->arena.find("cfb_koffs"), phi, d_lnmu, n_lnmu, d_P, st);
    };
    CKS(upload(ctx, d_items, items.data(), items.size()));
    CKS(upload(ctx, d_lnmu, lnmu, (size_t)n_lnmu));
    const bool reuse = use_graph && S.graph[P] && S.graph_nm[P] == n_lnmu && S.graph_kt[P] == S.kt[P] &&
                       S.graph_cps[P] == S.cps[P];
    if (use_graph && !reuse) {
        // capture the whole step once: counter reset, persistent solve, Phi, inversion
        CKS(sync_stream(ctx));
        if (S.graph[P]) { cudaGraphExecDestroy(S.graph[P]); S.graph[P] = nullptr; }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        enqueue();
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (ce != cudaSuccess) return fail(ctx, SGL_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        const cudaError_t ie = cudaGraphInstantiate(&S.graph[P], g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) { S.graph[P] = nullptr; return fail(ctx, SGL_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie)); }
        S.graph_nm[P] = n_lnmu; S.graph_kt[P] = S.kt[P]; S.graph_cps[P] = S.cps[P];
    }
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    cudaEventRecord(a, st);
    if (use_graph) CK(cudaGraphLaunch(S.graph[P], st));
    else enqueue();
    cudaEventRecord(b, st);
    CKLAUNCH();
    CK(cudaMemcpyAsync(P_out, d_P, (size_t)S.n_inst * n_lnmu * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKS(sync_stream(ctx));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms_out) *ms_out = ms;
    for (long long e = 0; e < (long long)S.n_inst * n_lnmu; ++e)
        if (!std::isfinite(P_out[e])) return fail(ctx, SGL_ERR_NONFINITE, "batched PDF returned non-finite values");
    return SGL_OK;
}

}  // extern "C"
