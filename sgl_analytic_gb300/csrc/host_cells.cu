// Binned-cell deposit (sgl_cells_*): the population build's Cells accumulator (sgl_full.py:1282-1533)
// with its lattices and xi_lin node resident in device memory.  The host side validates, stages each
// batch of objects, keeps the per-object totals (N, dropped, lin) in the reference's order, and closes
// an xi node: occupied rows found on the device, the Gram matrix reduced there, its 42 x 42
// eigendecomposition by cyclic Jacobi here, the projection onto the kept modes on the device again.
#include "host.cuh"

struct CellsState {
    CellsGeom geom{};
    int nshell = 0, nord = 0, n_sm = 0;
    std::vector<double> edges, kmc, gmc;
    long long nfine = 0, ncoarse = 0;
    bool xi_on = false, pos = false, node_open = false;
    int nkp = 0, mm = 0;
    std::vector<double> kp, c;
    double dchi = 0.0;
    struct Group {
        int m = 0, nrow = 0;
        std::vector<int> idx;
        std::vector<double> rows, W, v0;
    };
    std::vector<Group> groups;            // of the node closed last
};

void cells_state_free(CellsState* s) { delete s; }

namespace {

constexpr double kXiSvdTol = 1e-6;        // sgl_full.py:2436
constexpr int kGramChunk = 128;
constexpr int kMaxEdges = 6144;           // the four edge lists share one CTA's 48 KB of shared memory

// the first log-spaced entry and the log step of a signed-log (-pos[::-1], pos) or geometric edge list;
// only the kernels' bin guess uses them (the bracket search is exact for any guess)
void log_params(const double* e, int n, bool signed_list, double& lo, double& dl) {
    const int i0 = signed_list ? n / 2 : 0;
    const int cnt = n - i0;
    lo = e[i0];
    dl = (cnt > 1 && lo > 0 && e[n - 1] > lo) ? std::log(e[n - 1] / lo) / (cnt - 1) : 0.0;
    if (!(lo > 0) || !(dl > 0) || !std::isfinite(dl)) { lo = 1.0; dl = 1.0; }
}

bool ascending(const double* e, int n) {
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(e[i]) || (i > 0 && !(e[i] > e[i - 1]))) return false;
    return true;
}

// signed geometric bin centres (sgl_full.py:466-468)
std::vector<double> centres_signed(const std::vector<double>& e) {
    std::vector<double> c(e.size() - 1);
    for (size_t i = 0; i + 1 < e.size(); ++i) {
        const double p = e[i] * e[i + 1];
        c[i] = p > 0 ? (e[i + 1] > 0 ? 1.0 : -1.0) * std::sqrt(std::fabs(p)) : 0.0;
    }
    return c;
}

// eigenvalues (descending) and eigenvectors (columns, V[j * n + q]) of a symmetric n x n matrix by cyclic
// Jacobi rotations
void jacobi_eigh(std::vector<double> A, int n, std::vector<double>& ev, std::vector<double>& V) {
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int p = 0; p < n; ++p) {
            diag += A[(size_t)p * n + p] * A[(size_t)p * n + p];
            for (int q = p + 1; q < n; ++q) off += A[(size_t)p * n + q] * A[(size_t)p * n + q];
        }
        if (off <= 1e-34 * diag || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[(size_t)p * n + q];
                if (apq == 0.0) continue;
                const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < n; ++k) {
                    const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = cs * akp - sn * akq;
                    A[(size_t)k * n + q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = cs * apk - sn * aqk;
                    A[(size_t)q * n + k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = cs * vkp - sn * vkq;
                    V[(size_t)k * n + q] = sn * vkp + cs * vkq;
                }
            }
    }
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return A[(size_t)a * n + a] > A[(size_t)b * n + b]; });
    ev.resize(n);
    std::vector<double> Vs((size_t)n * n);
    for (int q = 0; q < n; ++q) {
        ev[q] = A[(size_t)order[q] * n + order[q]];
        for (int k = 0; k < n; ++k) Vs[(size_t)k * n + q] = V[(size_t)k * n + order[q]];
    }
    V.swap(Vs);
}

CellsState* need(sgl_ctx* ctx) { return ctx ? ctx->cells : nullptr; }

}  // namespace

extern "C" {

sgl_status sgl_cells_init(sgl_ctx* ctx, int nshell, int nord, int nekf, const double* ekf, int negf,
                          const double* egf, int nekc, const double* ekc, int negc, const double* egc,
                          double g_clip, double k_max_fine) {
    if (!ctx) return SGL_ERR_VALUE;
    if (nshell < 1 || nord < 0 || nord > 15 || !ekf || !egf || !ekc || !egc)
        return fail(ctx, SGL_ERR_VALUE, "sgl_cells_init: need nshell >= 1, 0 <= nord <= 15 and four edge lists");
    if (nekf < 2 || negf < 2 || nekc < 2 || negc < 2 || !ascending(ekf, nekf) || !ascending(egf, negf) ||
        !ascending(ekc, nekc) || !ascending(egc, negc))
        return fail(ctx, SGL_ERR_VALUE, "sgl_cells_init: edge lists must be finite, strictly ascending, >= 2 entries");
    if ((long long)nekf + negf + nekc + negc > kMaxEdges)
        return fail(ctx, SGL_ERR_UNSUPPORTED, "sgl_cells_init: more than 6144 edges in all");
    if (!std::isfinite(g_clip) || !(k_max_fine > 0))
        return fail(ctx, SGL_ERR_VALUE, "sgl_cells_init: g_clip must be finite and k_max_fine positive");
    CK(cudaSetDevice(ctx->device));
    delete ctx->cells;
    ctx->cells = new CellsState();
    CellsState& S = *ctx->cells;
    S.nshell = nshell;
    S.nord = nord;
    CellsGeom& g = S.geom;
    g.nekf = nekf; g.negf = negf; g.nekc = nekc; g.negc = negc;
    log_params(ekf, nekf, true, g.kf_lo, g.kf_dl);
    log_params(egf, negf, false, g.gf_lo, g.gf_dl);
    log_params(ekc, nekc, true, g.kc_lo, g.kc_dl);
    log_params(egc, negc, false, g.gc_lo, g.gc_dl);
    g.g_clip = g_clip;
    g.k_max_fine = k_max_fine;
    g.nord = nord;
    S.edges.insert(S.edges.end(), ekf, ekf + nekf);
    S.edges.insert(S.edges.end(), egf, egf + negf);
    S.edges.insert(S.edges.end(), ekc, ekc + nekc);
    S.edges.insert(S.edges.end(), egc, egc + negc);
    S.kmc = centres_signed(std::vector<double>(ekc, ekc + nekc));
    S.gmc.resize(negc - 1);
    for (int i = 0; i + 1 < negc; ++i) S.gmc[i] = std::sqrt(egc[i] * egc[i + 1]);
    S.nfine = (long long)(nekf - 1) * (negf - 1);
    S.ncoarse = (long long)(nekc - 1) * (negc - 1);
    CK(cudaDeviceGetAttribute(&S.n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
    const long long nHc = (long long)nshell * (nord + 1) * S.ncoarse;
    DBUF(d_e, double, "cells_edges", S.edges.size());
    DBUF(d_H0, double, "cells_H0", S.nfine);
    DBUF(d_H0k, double, "cells_H0k", S.nfine);
    DBUF(d_H0g, double, "cells_H0g", S.nfine);
    DBUF(d_Hc, double, "cells_Hc", nHc);
    CKS(upload(ctx, d_e, S.edges.data(), S.edges.size()));
    CK(cudaMemsetAsync(d_H0, 0, sizeof(double) * S.nfine, ctx->stream));
    CK(cudaMemsetAsync(d_H0k, 0, sizeof(double) * S.nfine, ctx->stream));
    CK(cudaMemsetAsync(d_H0g, 0, sizeof(double) * S.nfine, ctx->stream));
    CK(cudaMemsetAsync(d_Hc, 0, sizeof(double) * nHc, ctx->stream));
    return sync_stream(ctx);
}

sgl_status sgl_cells_xi_init(sgl_ctx* ctx, int nkp, const double* kp, const double* c, int mmax, int pos) {
    CellsState* S = need(ctx);
    if (!S) return ctx ? fail(ctx, SGL_ERR_STATE, "sgl_cells_xi_init: call sgl_cells_init first") : SGL_ERR_VALUE;
    if (nkp < 1 || nkp > 64 || !kp || !c || mmax < 0 || mmax > 2)
        return fail(ctx, SGL_ERR_VALUE, "sgl_cells_xi_init: need 1 <= nkp <= 64 k_perp nodes and 0 <= mmax <= 2");
    if (S->geom.nekc + S->geom.negc > kCellsXiMaxEdges)
        return fail(ctx, SGL_ERR_UNSUPPORTED, "sgl_cells_xi_init: the xi_lin term takes at most 1024 coarse edges in all");
    for (int j = 0; j < nkp; ++j)
        if (!(kp[j] > 0) || !std::isfinite(kp[j]) || !(c[j] >= 0) || !std::isfinite(c[j]))
            return fail(ctx, SGL_ERR_VALUE, "sgl_cells_xi_init: k_perp nodes must be positive and weights c >= 0, finite");
    S->xi_on = true;
    S->pos = pos != 0;
    S->nkp = nkp;
    S->mm = mmax;
    S->kp.assign(kp, kp + nkp);
    S->c.assign(c, c + nkp);
    S->node_open = false;
    DBUF(d_kp, double, "cells_kp", nkp);
    CKS(upload(ctx, d_kp, kp, (size_t)nkp));
    return sync_stream(ctx);
}

sgl_status sgl_cells_xi_begin(sgl_ctx* ctx, double dchi) {
    CellsState* S = need(ctx);
    if (!S || !S->xi_on) return ctx ? fail(ctx, SGL_ERR_STATE, "sgl_cells_xi_begin: no xi_lin term (sgl_cells_xi_init)") : SGL_ERR_VALUE;
    if (!(dchi > 0) || !std::isfinite(dchi)) return fail(ctx, SGL_ERR_VALUE, "sgl_cells_xi_begin: dchi must be positive");
    const long long nHx = S->ncoarse * (S->mm + 1) * S->nkp;
    DBUF(d_Hx, double, "cells_Hx", nHx);
    DBUF(d_lx, double, "cells_lx", 2 * S->nkp);
    CK(cudaMemsetAsync(d_Hx, 0, sizeof(double) * nHx, ctx->stream));
    CK(cudaMemsetAsync(d_lx, 0, sizeof(double) * 2 * S->nkp, ctx->stream));
    if (S->pos) {
        DBUF(d_Wb, double, "cells_Wb", S->ncoarse);
        CK(cudaMemsetAsync(d_Wb, 0, sizeof(double) * S->ncoarse, ctx->stream));
    }
    S->dchi = dchi;
    S->node_open = true;
    S->groups.clear();
    return SGL_OK;
}

sgl_status sgl_cells_add(sgl_ctx* ctx, int n_obj, const int64_t* off, const double* K, const double* G,
                         const double* W, const double* R, const int32_t* shell, const double* beta,
                         const unsigned char* tang, double* sums) {
    CellsState* S = need(ctx);
    if (!S) return ctx ? fail(ctx, SGL_ERR_STATE, "sgl_cells_add: call sgl_cells_init first") : SGL_ERR_VALUE;
    if (n_obj < 0 || !off || (n_obj > 0 && (!shell || !beta || !sums)))
        return fail(ctx, SGL_ERR_VALUE, "sgl_cells_add: invalid object arrays");
    if (n_obj == 0) return SGL_OK;
    if (off[0] != 0) return fail(ctx, SGL_ERR_VALUE, "sgl_cells_add: off[0] must be 0");
    for (int o = 0; o < n_obj; ++o) {
        if (off[o + 1] < off[o]) return fail(ctx, SGL_ERR_VALUE, "sgl_cells_add: offsets must be non-decreasing");
        if (shell[o] < 0 || shell[o] >= S->nshell) return fail(ctx, SGL_ERR_VALUE, "sgl_cells_add: shell out of range");
        if (!std::isfinite(beta[o])) return fail(ctx, SGL_ERR_VALUE, "sgl_cells_add: beta must be finite");
    }
    const long long n = off[n_obj];
    if (n > 0 && (!K || !G || !W)) return fail(ctx, SGL_ERR_VALUE, "sgl_cells_add: NULL point arrays");
    if (S->xi_on) {
        if (!S->node_open) return fail(ctx, SGL_ERR_STATE, "xi deposit outside xi_begin / xi_end");
        if (n > 0 && !R) return fail(ctx, SGL_ERR_UNSUPPORTED, "the xi_lin term needs each point's lens distance R");
    }
    CK(cudaSetDevice(ctx->device));
    const int no = S->nord + 1;
    std::vector<double> betas((size_t)n_obj * no);
    for (int o = 0; o < n_obj; ++o)
        for (int q = 0; q < no; ++q) betas[(size_t)o * no + q] = std::pow(beta[o], (double)q);
    std::vector<unsigned char> tg((size_t)n_obj, 1);
    if (tang)
        for (int o = 0; o < n_obj; ++o) tg[o] = tang[o] ? 1 : 0;
    DBUF(d_K, double, "cells_in_K", std::max(1LL, n));
    DBUF(d_G, double, "cells_in_G", std::max(1LL, n));
    DBUF(d_W, double, "cells_in_W", std::max(1LL, n));
    DBUF(d_off, long long, "cells_in_off", n_obj + 1);
    DBUF(d_sh, int, "cells_in_shell", n_obj);
    DBUF(d_b, double, "cells_in_betas", (size_t)n_obj * no);
    DBUF(d_sums, double, "cells_sums", 3LL * n_obj);
    static_assert(sizeof(long long) == sizeof(int64_t), "offsets");
    CKS(upload(ctx, d_K, K, (size_t)n));
    CKS(upload(ctx, d_G, G, (size_t)n));
    CKS(upload(ctx, d_W, W, (size_t)n));
    CKS(upload(ctx, d_off, reinterpret_cast<const long long*>(off), (size_t)n_obj + 1));
    CKS(upload(ctx, d_sh, shell, (size_t)n_obj));
    CKS(upload(ctx, d_b, betas.data(), betas.size()));
    CK(cudaMemsetAsync(d_sums, 0, sizeof(double) * 3 * n_obj, ctx->stream));
    double* d_e = (double*)ctx->arena.find("cells_edges");
    if (S->xi_on && n > 0) {
        // work items: chunks of at most kXiChunk points that never straddle two objects
        std::vector<CellsXiItem> items;
        for (int o = 0; o < n_obj; ++o)
            for (long long a = off[o]; a < off[o + 1]; a += kXiChunk)
                items.push_back(CellsXiItem{a, (int)std::min<long long>(kXiChunk, off[o + 1] - a), o});
        DBUF(d_R, double, "cells_in_R", n);
        DBUF(d_beta1, double, "cells_in_beta", n_obj);
        DBUF(d_tang, unsigned char, "cells_in_tang", n_obj);
        DBUF(d_items, CellsXiItem, "cells_in_items", items.size());
        CKS(upload(ctx, d_R, R, (size_t)n));
        CKS(upload(ctx, d_beta1, beta, (size_t)n_obj));
        CKS(upload(ctx, d_tang, tg.data(), tg.size()));
        CKS(upload(ctx, d_items, items.data(), items.size()));
        Timed t(ctx, "cells_xi", 0.0, 32.0 * n);
        launch_cells_xi(S->geom, d_e, d_items, (int)items.size(), d_K, d_G, d_W, d_R, d_beta1, d_tang,
                        (const double*)ctx->arena.find("cells_kp"), S->nkp, S->mm,
                        (double*)ctx->arena.find("cells_Hx"), (double*)ctx->arena.find("cells_lx"),
                        S->pos ? (double*)ctx->arena.find("cells_Wb") : nullptr, ctx->stream);
        CKLAUNCH();
    }
    {
        Timed t(ctx, "cells_hist", 0.0, 24.0 * n);
        launch_cells_hist(S->geom, d_e, n, d_K, d_G, d_W, d_off, n_obj, d_sh, d_b, (double*)ctx->arena.find("cells_H0"),
                          (double*)ctx->arena.find("cells_H0k"), (double*)ctx->arena.find("cells_H0g"),
                          (double*)ctx->arena.find("cells_Hc"), d_sums, S->n_sm, ctx->stream);
        CKLAUNCH();
    }
    CK(cudaMemcpyAsync(sums, d_sums, sizeof(double) * 3 * n_obj, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_stream(ctx);
}

sgl_status sgl_cells_xi_shear_tail(sgl_ctx* ctx, double beta, double Gam, double Rm, double n_area) {
    CellsState* S = need(ctx);
    if (!S || !S->node_open) return ctx ? fail(ctx, SGL_ERR_STATE, "sgl_cells_xi_shear_tail: no open xi node") : SGL_ERR_VALUE;
    if (S->mm < 1) return SGL_OK;
    if (!(Rm > 0) || !std::isfinite(beta * Gam * n_area))
        return fail(ctx, SGL_ERR_VALUE, "sgl_cells_xi_shear_tail: Rm must be positive, beta Gam n_area finite");
    CK(cudaSetDevice(ctx->device));
    const double coef = beta * n_area * 2 * M_PI * Gam;
    launch_cells_xi_tail((const double*)ctx->arena.find("cells_kp"), S->nkp, coef, Rm,
                         (double*)ctx->arena.find("cells_lx"), ctx->stream);
    CKLAUNCH();
    return SGL_OK;
}

sgl_status sgl_cells_xi_end(sgl_ctx* ctx, int* n_groups) {
    CellsState* S = need(ctx);
    if (!S || !S->node_open) return ctx ? fail(ctx, SGL_ERR_STATE, "sgl_cells_xi_end: no open xi node") : SGL_ERR_VALUE;
    if (!n_groups) return fail(ctx, SGL_ERR_VALUE, "sgl_cells_xi_end: NULL n_groups");
    CK(cudaSetDevice(ctx->device));
    S->node_open = false;
    S->groups.clear();
    const int nkp = S->nkp, mm = S->mm, ngc = S->geom.negc - 1;
    const int nbins = (int)S->ncoarse;
    const cudaStream_t st = ctx->stream;
    double* d_Hx = (double*)ctx->arena.find("cells_Hx");
    double* d_lx = (double*)ctx->arena.find("cells_lx");
    DBUF(d_flags, unsigned char, "cells_flags", (size_t)nbins * (mm + 1));
    launch_cells_xi_flags(d_Hx, nbins, mm, nkp, d_flags, st);
    CKLAUNCH();
    std::vector<unsigned char> flags((size_t)nbins * (mm + 1));
    std::vector<double> lx(2 * (size_t)nkp), Wb;
    CK(cudaMemcpyAsync(flags.data(), d_flags, flags.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(lx.data(), d_lx, sizeof(double) * lx.size(), cudaMemcpyDeviceToHost, st));
    if (S->pos) {
        Wb.resize((size_t)nbins);
        CK(cudaMemcpyAsync(Wb.data(), ctx->arena.find("cells_Wb"), sizeof(double) * nbins, cudaMemcpyDeviceToHost, st));
    }
    CKS(sync_stream(ctx));
    std::vector<double> sw((size_t)nkp);
    for (int j = 0; j < nkp; ++j) sw[j] = std::sqrt(S->c[j] / S->dchi);
    DBUF(d_sw, double, "cells_sw", nkp);
    DBUF(d_kmc, double, "cells_kmc", S->kmc.size());
    DBUF(d_gmc, double, "cells_gmc", S->gmc.size());
    CKS(upload(ctx, d_sw, sw.data(), sw.size()));
    CKS(upload(ctx, d_kmc, S->kmc.data(), S->kmc.size()));
    CKS(upload(ctx, d_gmc, S->gmc.data(), S->gmc.size()));
    for (int m = 0; m <= mm; ++m) {
        std::vector<int> idx;
        for (int b = 0; b < nbins; ++b)
            if (flags[(size_t)m * nbins + b]) idx.push_back(b);
        if (idx.empty()) {
            // linear-only node: one all-zero bin carries the residual (sgl_full.py:1492-1496)
            bool any = false;
            if (m <= 1)
                for (int j = 0; j < nkp; ++j) any |= lx[(size_t)m * nkp + j] != 0.0;
            if (!any) continue;
            idx.push_back(0);
        }
        const int nidx = (int)idx.size();
        const long long nrows = nidx + 1LL;
        DBUF(d_idx, int, "cells_idx", nidx);
        DBUF(d_A, double, "cells_A", nrows * nkp);
        DBUF(d_part, double, "cells_gram_part", (long long)cells_gram_parts(nrows, kGramChunk) * nkp * nkp);
        DBUF(d_gram, double, "cells_gram", (long long)nkp * nkp);
        CKS(upload(ctx, d_idx, idx.data(), idx.size()));
        const int axis = m == 0 ? 0 : (m == 1 ? 1 : -1);
        launch_cells_xi_rows(d_Hx, mm, nkp, m, d_idx, nidx, axis == 0 ? d_kmc : d_gmc, ngc, axis,
                             d_lx + (m <= 1 ? (size_t)m * nkp : 0), d_sw, d_A, st);
        CKLAUNCH();
        launch_cells_gram(d_A, nrows, nkp, kGramChunk, d_part, d_gram, st);
        CKLAUNCH();
        std::vector<double> gram((size_t)nkp * nkp);
        CK(cudaMemcpyAsync(gram.data(), d_gram, sizeof(double) * gram.size(), cudaMemcpyDeviceToHost, st));
        CKS(sync_stream(ctx));
        std::vector<double> ev, V;
        jacobi_eigh(gram, nkp, ev, V);
        const double S0 = std::sqrt(std::max(ev[0], 0.0));
        std::vector<int> keep;
        if (S0 > 0)
            for (int q = 0; q < nkp; ++q)
                if (std::sqrt(std::max(ev[q], 0.0)) > kXiSvdTol * S0) keep.push_back(q);
        if (keep.empty()) continue;
        const int nk = (int)keep.size();
        std::vector<double> Vk((size_t)nkp * nk);
        for (int j = 0; j < nkp; ++j)
            for (int q = 0; q < nk; ++q) Vk[(size_t)j * nk + q] = V[(size_t)j * nkp + keep[q]];
        DBUF(d_V, double, "cells_V", Vk.size());
        DBUF(d_rows, double, "cells_rows", (long long)nk * nrows);
        CKS(upload(ctx, d_V, Vk.data(), Vk.size()));
        launch_cells_project(d_A, nrows, nkp, d_V, nk, d_rows, st);
        CKLAUNCH();
        CellsState::Group g;
        g.m = m;
        g.nrow = nk;
        g.idx = idx;
        g.rows.resize((size_t)nk * nrows);
        CK(cudaMemcpyAsync(g.rows.data(), d_rows, sizeof(double) * g.rows.size(), cudaMemcpyDeviceToHost, st));
        CKS(sync_stream(ctx));
        for (double v : g.rows)
            if (!std::isfinite(v)) return fail(ctx, SGL_ERR_NONFINITE, "sgl_cells_xi_end: non-finite rows");
        if (m == 0 && S->pos) {
            g.W.resize((size_t)nidx);
            for (int r = 0; r < nidx; ++r) g.W[r] = Wb[(size_t)idx[r]];
            g.v0.resize((size_t)nkp);
            for (int j = 0; j < nkp; ++j) g.v0[j] = V[(size_t)j * nkp];
        }
        S->groups.push_back(std::move(g));
    }
    *n_groups = (int)S->groups.size();
    return SGL_OK;
}

sgl_status sgl_cells_xi_group(sgl_ctx* ctx, int g, int32_t* m, int32_t* nidx, int32_t* nrow, int32_t* idx,
                              double* rows, double* W, double* v0) {
    CellsState* S = need(ctx);
    if (!S) return ctx ? fail(ctx, SGL_ERR_STATE, "sgl_cells_xi_group: call sgl_cells_init first") : SGL_ERR_VALUE;
    if (g < 0 || g >= (int)S->groups.size()) return fail(ctx, SGL_ERR_VALUE, "sgl_cells_xi_group: no such group");
    const CellsState::Group& G = S->groups[(size_t)g];
    if (m) *m = G.m;
    if (nidx) *nidx = (int)G.idx.size();
    if (nrow) *nrow = G.nrow;
    if (idx) std::copy(G.idx.begin(), G.idx.end(), idx);
    if (rows) std::copy(G.rows.begin(), G.rows.end(), rows);
    if (W && !G.W.empty()) std::copy(G.W.begin(), G.W.end(), W);
    if (v0 && !G.v0.empty()) std::copy(G.v0.begin(), G.v0.end(), v0);
    return SGL_OK;
}

sgl_status sgl_cells_read(sgl_ctx* ctx, double* H0, double* H0k, double* H0g, double* Hc) {
    CellsState* S = need(ctx);
    if (!S) return ctx ? fail(ctx, SGL_ERR_STATE, "sgl_cells_read: call sgl_cells_init first") : SGL_ERR_VALUE;
    CK(cudaSetDevice(ctx->device));
    const cudaStream_t st = ctx->stream;
    const size_t nf = sizeof(double) * (size_t)S->nfine;
    if (H0) CK(cudaMemcpyAsync(H0, ctx->arena.find("cells_H0"), nf, cudaMemcpyDeviceToHost, st));
    if (H0k) CK(cudaMemcpyAsync(H0k, ctx->arena.find("cells_H0k"), nf, cudaMemcpyDeviceToHost, st));
    if (H0g) CK(cudaMemcpyAsync(H0g, ctx->arena.find("cells_H0g"), nf, cudaMemcpyDeviceToHost, st));
    if (Hc)
        CK(cudaMemcpyAsync(Hc, ctx->arena.find("cells_Hc"),
                           sizeof(double) * (size_t)S->nshell * (S->nord + 1) * (size_t)S->ncoarse,
                           cudaMemcpyDeviceToHost, st));
    return sync_stream(ctx);
}

}  // extern "C"
