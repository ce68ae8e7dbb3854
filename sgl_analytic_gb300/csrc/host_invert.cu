// The inversion (sgl_full.invert): grid plan with the measured k-reach, Phi = exp(ln Phi),
// the box window, Hankel and kappa transforms, Euler-Maclaurin term, constant-mu path
// integral, normalisation and moments.
//
// Three entry points share the stages below:
//   sgl_pdf        plan the grid from the context's population, Phi = exp(ln Phi), invert;
//   sgl_plan_grid  only the grid plan (vector_grid, tail box, measured reach), for a caller that
//                  evaluates Phi itself;
//   sgl_invert     invert a caller-owned Phi given on such a grid.
#include "host.cuh"

// populations of at most this many cells evaluate ln Phi in FP64 on the mixed path as well
constexpr long long kMixedFp64LambdaCells = 4096;

namespace sglh {

// the reference's invert grid (sgl_full.py:187-262) for one population: every quantity the
// transforms and the path integral need
struct GridPlan {
    long long nk_k = 0, nk_g = 0, n_kap = 0, n_gam = 0;
    double k_k_max = 0, k_g_max = 0, kap_min = 0, kap_max = 0, gam_max = 0, xi_min = 0, xi_max = 0;
    double sigma = 0, g0 = 0, phic[2] = {0, 0};
};

sgl_status check_opts(sgl_ctx* ctx, const sgl_invert_opts* opts, sgl_invert_opts& o) {
    sgl_invert_opts_default(&o);
    if (opts) o = *opts;
    if (o.precision != SGL_FP64 && o.precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    if (o.n_xi_wide < 2 || o.n_k_int < 2 || !(o.phi_tol > 0) || !(o.xi_reach > 0) || o.window < 0 || o.window > 2)
        return fail(ctx, SGL_ERR_VALUE, "invalid inversion options");
    return SGL_OK;
}

// vector_grid (sgl.py:1229-1258) and the tail box of invert (sgl_full.py:191-212) for sigma: the
// box, the output grid and the k steps; k_k_max / k_g_max are the reach probes' start points
void box_for_sigma(const sgl_invert_opts& o, double sigma, GridPlan& G, double& dk_k, double& dk_g) {
    const double sig_xi = 2.0 * sigma;
    G.sigma = sigma;
    G.xi_max = o.xi_reach * sig_xi;
    G.xi_min = -kBoxReach * sig_xi;
    double kap_max = 1.0 - std::exp(-0.5 * G.xi_max);
    const double kap_min = -kBoxReach * sigma;
    double gam_max = kBoxReach * sigma;
    G.g0 = gam_max;
    G.k_k_max = kSigReach / sigma;
    G.k_g_max = kSigReach / sigma;
    long long n_kap = (long long)std::ceil((kap_max - kap_min) / (sigma / kPtsPerSigKap)) + 1;
    long long n_gam = (long long)std::ceil(gam_max / (sigma / kPtsPerSigGam)) + 1;
    double kap_max_new = kap_max, gam_max_new = gam_max;
    if (o.tail_box) { kap_max_new = std::max(kap_max, kTailKapMax); gam_max_new = std::max(G.g0, kTailGamMax); }
    dk_k = 2.0 * M_PI / (kPppK * std::max(std::fabs(kap_min), kap_max));
    dk_g = 2.0 * M_PI / (kPppG * gam_max);
    if (o.tail_box && kTailPppG > 0) dk_g = std::min(dk_g, 2.0 * M_PI / (kTailPppG * gam_max_new));
    if (kap_max_new != kap_max || gam_max_new != gam_max) {
        kap_max = kap_max_new; gam_max = gam_max_new;
        n_kap = (long long)std::ceil((kap_max - kap_min) / (sigma / kPtsPerSigKap)) + 1;
        n_gam = (long long)std::ceil(gam_max / (sigma / kPtsPerSigGam)) + 1;
    }
    G.kap_min = kap_min; G.kap_max = kap_max; G.gam_max = gam_max; G.n_kap = n_kap; G.n_gam = n_gam;
}

// The whole grid plan: the box, then the measured reach (_reach, sgl_full.py:38-47: 20 probes
// k0 * 1.25^j per axis on ln Phi) and the k grid sizes.  With the positive closure installed its
// coarse grid grows with the box, per axis (sgl_full.py:226-238).
sgl_status plan_grid(sgl_ctx* ctx, const sgl_invert_opts& o, GridPlan& G) {
    double sigma;
    CKS(sgl_lam_sigma(ctx, &sigma));
    if (!(sigma > 0) || !std::isfinite(sigma)) return fail(ctx, SGL_ERR_VALUE, "sigma_kappa must be positive");
    double dk_k, dk_g;
    box_for_sigma(o, sigma, G, dk_k, dk_g);
    const int nprobe = (int)std::ceil(std::log(64.0) / std::log(1.25)) + 1;
    double reach[2];
    for (int ax = 0; ax < 2; ++ax) {
        const double k0v = ax == 0 ? G.k_k_max : G.k_g_max;
        std::vector<double> ks(nprobe), re(nprobe), im(nprobe);
        for (int j = 0; j < nprobe; ++j) ks[j] = k0v * std::pow(1.25, (double)j);
        const double zero = 0.0;
        if (ax == 0) CKS(lambda_direct(ctx, ks.data(), nprobe, &zero, 1, re.data(), im.data(), o.precision));
        else CKS(lambda_direct(ctx, &zero, 1, ks.data(), nprobe, re.data(), im.data(), o.precision));
        int pick = -1, amin = 0;
        double best = 1e300;
        for (int j = 0; j < nprobe; ++j) {
            const double phi = std::fabs(std::exp(re[j]));   // |exp(L)| = exp(Re L)
            if (phi <= o.phi_tol && pick < 0) pick = j;
            if (phi < best) { best = phi; amin = j; }
        }
        const int i = pick >= 0 ? pick : amin;
        reach[ax] = ks[i];
        G.phic[ax] = std::exp(re[i]);
    }
    G.k_k_max = reach[0]; G.k_g_max = reach[1];
    G.nk_k = (long long)std::ceil(G.k_k_max / dk_k) + 1;
    G.nk_g = (long long)std::ceil(G.k_g_max / dk_g) + 1;
    if (ctx->vp_on) {
        const double kks = G.k_k_max * sigma, kgs = G.k_g_max * sigma;
        ctx->vp_xi_coarse = (int)std::min(401.0, std::max((double)ctx->vp_xi_coarse, 1.0 + std::ceil(12.65 * std::sqrt(kgs))));
        ctx->vp_xi_coarse_k = (int)std::min(4001.0, std::max({(double)ctx->vp_xi_coarse_k, (double)ctx->vp_xi_coarse,
                                                              1.0 + std::ceil(66.7 * std::sqrt(kks))}));
    }
    return SGL_OK;
}

// Grid limits of this implementation.  Above 2e7 k-points the reference accumulates Phi, the
// Hankel product and the kappa transform over k_kappa row blocks to bound host memory
// (_invert_blocked, sgl_full.py:97-157; "same sums, partial-sum order -> roundoff").  The whole
// grid fits in HBM here, so the same sums run unblocked; allocation failure is reported as such.
// The Phi rows are one grid dimension of the composition kernel, hence the axis limit.
sgl_status check_grid(sgl_ctx* ctx, const GridPlan& G) {
    if ((double)G.n_kap * (double)G.n_gam > kOutGridMax)
        return fail(ctx, SGL_ERR_UNSUPPORTED, "geometric output grid (n_kap * n_gam > OUT_GRID_MAX) not implemented");
    if (G.nk_k > 65535) return fail(ctx, SGL_ERR_UNSUPPORTED, "k_kappa axis longer than 65535 points");
    if (G.nk_k < 2 || G.nk_g < 2) return fail(ctx, SGL_ERR_VALUE, "degenerate k grid");
    if (G.n_kap < 2 || G.n_gam < 2) return fail(ctx, SGL_ERR_VALUE, "degenerate output grid");
    return SGL_OK;
}

// Everything after Phi: the box window, the Hankel and kappa transforms with the Euler-Maclaurin
// endpoint term, the constant-mu path integrals on the wide grid and the caller's grid, the
// normalisation and the moments.  Phi: the context's "phi" buffer (re plane, then im plane) in
// the precision's element type; ctx->ev[0] was recorded before Phi was formed.
sgl_status invert_phi(sgl_ctx* ctx, const sgl_invert_opts& o, const GridPlan& G, void* Phi, const double* xi_out,
                      int n_xi, double* P_out, sgl_invert_meta* meta) {
    const cudaStream_t st = ctx->stream;
    const std::vector<double> kk = linspace(0.0, G.k_k_max, G.nk_k);
    const std::vector<double> kg = linspace(0.0, G.k_g_max, G.nk_g);
    const std::vector<double> kap = linspace(G.kap_min, G.kap_max, G.n_kap);
    const std::vector<double> gam = linspace(0.0, G.gam_max, G.n_gam);
    const int nk = (int)G.nk_k, nkg = (int)G.nk_g, nkap = (int)G.n_kap, ngam = (int)G.n_gam;
    const int P = o.precision;
    const size_t es = elem_size(P);
    // window (sgl_full.py:254-258): 1 always, 2 ("auto") only when the reach did not converge
    const bool use_win = o.window == 1 || (o.window == 2 && std::max(G.phic[0], G.phic[1]) > o.phi_tol);
    if (use_win) {
        std::vector<double> wk(nk), wg(nkg);
        for (int i = 0; i < nk; ++i) {
            const double x = std::fabs(kk[i]) * 2.0 / G.k_k_max;
            const double v = x < 1 ? 2.0 / 3.0 - x * x + x * x * x / 2 : (x < 2 ? (2 - x) * (2 - x) * (2 - x) / 6 : 0.0);
            wk[i] = v / (2.0 / 3.0);
        }
        for (int j = 0; j < nkg; ++j) {
            const double r = std::min(1.0, std::max(0.0, std::fabs(kg[j]) / G.k_g_max));
            wg[j] = std::pow(1 - r, 4) * (4 * r + 1);
        }
        DBUF(d_wk, double, "win_k", nk);
        DBUF(d_wg, double, "win_g", nkg);
        CKS(upload(ctx, d_wk, wk.data(), nk));
        CKS(upload(ctx, d_wg, wg.data(), nkg));
        launch_window(P, Phi, nk, nkg, d_wk, d_wg, st); CKLAUNCH();
    }
    cudaEventRecord(ctx->ev[1], st);
    // ---- transforms: F = Phi @ M (Hankel), P3ext = c CS @ [F | va | vb]
    DBUF(d_kk, double, "inv_kk", nk);
    DBUF(d_kg, double, "inv_kg", nkg);
    DBUF(d_kap, double, "inv_kap", nkap);
    DBUF(d_gam, double, "inv_gam", ngam);
    CKS(upload(ctx, d_kk, kk.data(), nk));
    CKS(upload(ctx, d_kg, kg.data(), nkg));
    CKS(upload(ctx, d_kap, kap.data(), nkap));
    CKS(upload(ctx, d_gam, gam.data(), ngam));
    const int ldF = ngam + 2;
    void* M = ctx->arena.get("inv_M", (size_t)nkg * ldF * es * (P == SGL_FP64 ? 1 : 2));
    void* F = ctx->arena.get("inv_F", 2ULL * nk * ldF * es);
    void* CS = ctx->arena.get("inv_CS", (size_t)nkap * 2 * nk * es);
    void* P3e = ctx->arena.get("inv_P3e", (size_t)nkap * ldF * es);
    DBUF(d_P3, double, "inv_P3", (long long)nkap * ngam);
    if (!M || !F || !CS || !P3e) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (transforms)");
    const double dkg = kg[1] - kg[0], dkk = kk[1] - kk[0];
    // the transform matrices depend on the grid only: kept between PDFs on the same grid
    const std::vector<double> kM{(double)P, (double)nkg, G.k_g_max, (double)ngam, G.gam_max};
    if (!table_current(ctx, "inv_M", kM)) {
        launch_hankel_matrix(P, d_kg, nkg, dkg, d_gam, ngam, ldF, M, st); CKLAUNCH();
        table_built(ctx, "inv_M", kM);
    }
    const std::vector<double> kC{(double)P, (double)nk, G.k_k_max, (double)nkap, G.kap_min, G.kap_max};
    if (!table_current(ctx, "inv_CS", kC)) {
        launch_kappa_matrix(P, d_kk, nk, dkk, d_kap, nkap, CS, st); CKLAUNCH();
        table_built(ctx, "inv_CS", kC);
    }
    // mixed path: the transform sums run in >= 4 K-slices combined in float-float; within a slice
    // the FP32 kernel's compensated blocked accumulation bounds the chain's rounding
    constexpr int kTransformSplit = 4;
    const double c = 1.0 / (2.0 * M_PI * M_PI);
    if (P == SGL_FP64) {
        CKS(gemm_splitk<double>(ctx, gd<double>(2 * nk, ngam, nkg, Phi, nkg, 1, M, ldF, 1, F, ldF), "hankel"));
    } else {
        // F = Phi M_hi + Phi M_lo (split Hankel matrix)
        CKS(gemm_splitk<float>(ctx, gd<float>(2 * nk, ngam, nkg, Phi, nkg, 1, M, ldF, 1, F, ldF), "hankel", kTransformSplit));
        // the M_lo term is a correction of relative size 2^-24: BF16 operands on the tensor cores
        // carry it to ~0.4%, i.e. ~2e-10 of F
        CKS(gemm_splitk_tc(ctx, gd<float>(2 * nk, ngam, nkg, Phi, nkg, 1, (const float*)M + (size_t)nkg * ldF, ldF,
                                          1, F, ldF, 1.0, 1.0), "hankel_lo", 1, 1));
    }
    launch_em_columns(P, Phi, nk, nkg, dkg, F, ldF, ngam, st); CKLAUNCH();
    if (P == SGL_FP64) {
        CKS(gemm_splitk<double>(ctx, gd<double>(nkap, ldF, 2 * nk, CS, 2 * nk, 1, F, ldF, 1, P3e, ldF, c), "kappa"));
    } else {
        CKS(gemm_splitk<float>(ctx, gd<float>(nkap, ldF, 2 * nk, CS, 2 * nk, 1, F, ldF, 1, P3e, ldF, c), "kappa", kTransformSplit));
    }
    float* d_P3f = nullptr;
    if (P == SGL_MIXED) {
        d_P3f = dbuf<float>(ctx, "inv_P3f", (size_t)nkap * ngam);
        if (!d_P3f) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (P3f)");
    }
    launch_p3_finish(P, P3e, nkap, ngam, ldF, d_gam, d_P3, d_P3f, st); CKLAUNCH();
    cudaEventRecord(ctx->ev[2], st);
    // ---- path integral on the wide grid and the output grid in one launch
    const int nw = o.n_xi_wide;
    const std::vector<double> xw = linspace(G.xi_min, G.xi_max, nw);
    std::vector<double> xall(xw);
    xall.insert(xall.end(), xi_out, xi_out + n_xi);
    DBUF(d_x, double, "path_x", xall.size());
    DBUF(d_pi, double, "path_out", xall.size());
    CKS(upload(ctx, d_x, xall.data(), xall.size()));
    const double g_def = std::min(G.g0, G.gam_max);
    {
        Timed t(ctx, "path_integral", 0.0, (double)xall.size() * o.n_k_int * 2 * 4 * 8);
        launch_path_integral(d_P3, d_P3f, nkap, ngam, kap.front(), kap.back(), gam.back(), d_x, (int)xall.size(),
                             G.gam_max, g_def, o.n_k_int, d_pi, st);
    }
    CKLAUNCH();
    cudaEventRecord(ctx->ev[3], st);
    std::vector<double> pall(xall.size());
    CK(cudaMemcpyAsync(pall.data(), d_pi, pall.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKS(sync_stream(ctx));
    CKS(check_dev_err(ctx));
    // ---- normalisation and moments (sgl_full.py:362-372)
    const double* pw = pall.data();
    const double norm = trapz(pw, xw.data(), nw);
    std::vector<double> ps(nw), tmp(nw);
    for (int i = 0; i < nw; ++i) ps[i] = pw[i] / norm;
    for (int i = 0; i < nw; ++i) tmp[i] = xw[i] * ps[i];
    const double mean = trapz(tmp.data(), xw.data(), nw);
    for (int i = 0; i < nw; ++i) { const double d = xw[i] - mean; tmp[i] = d * d * ps[i]; }
    const double var = trapz(tmp.data(), xw.data(), nw);
    for (int i = 0; i < nw; ++i) { const double d = xw[i] - mean; tmp[i] = d * d * d * ps[i]; }
    const double skew = trapz(tmp.data(), xw.data(), nw) / std::pow(var, 1.5);
    std::vector<double> xe(nw);
    for (int i = 0; i < nw; ++i) xe[i] = std::exp(-0.5 * xw[i]);
    for (int i = 0; i < nw; ++i) tmp[i] = xe[i] * ps[i];
    const double md = trapz(tmp.data(), xw.data(), nw);
    for (int i = 0; i < nw; ++i) { const double d = xe[i] - md; tmp[i] = d * d * ps[i]; }
    const double sDL = std::sqrt(trapz(tmp.data(), xw.data(), nw)) / md;
    bool finite = std::isfinite(norm) && norm != 0.0;
    for (int i = 0; i < n_xi; ++i) {
        P_out[i] = pall[(size_t)nw + i] / norm;
        finite = finite && std::isfinite(P_out[i]);
    }
    if (meta) {
        meta->nk_k = G.nk_k; meta->nk_g = G.nk_g; meta->n_kap = G.n_kap; meta->n_gam = G.n_gam;
        meta->k_k_max = G.k_k_max; meta->k_g_max = G.k_g_max; meta->kap_min = G.kap_min; meta->kap_max = G.kap_max;
        meta->gam_max = G.gam_max; meta->xi_min = G.xi_min; meta->xi_max = G.xi_max; meta->sigma = G.sigma;
        meta->phi_at_k_cut = G.phic[0]; meta->phi_at_g_cut = G.phic[1];
        meta->mean = mean; meta->var = var; meta->skew = skew; meta->sigmaDL = sDL; meta->norm = norm;
        float a = 0, b = 0, cc = 0;
        cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
        cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
        cudaEventElapsedTime(&cc, ctx->ev[2], ctx->ev[3]);
        meta->ms_lambda = a; meta->ms_transform = b; meta->ms_path = cc;
        meta->window = use_win ? 1.0 : 0.0;
        meta->xi_coarse = ctx->vp_on ? ctx->vp_xi_coarse : 0.0;
        meta->xi_coarse_k = ctx->vp_on ? ctx->vp_xi_coarse_k : 0.0;
    }
    if (!finite) return fail(ctx, SGL_ERR_NONFINITE, "PDF inversion returned non-finite values");
    return SGL_OK;
}

sgl_status check_xi_out(sgl_ctx* ctx, const double* xi_out, int n_xi, const double* P_out) {
    if (n_xi < 0 || (n_xi > 0 && (!xi_out || !P_out))) return fail(ctx, SGL_ERR_VALUE, "invalid output grid");
    for (int i = 0; i < n_xi; ++i) if (!std::isfinite(xi_out[i])) return fail(ctx, SGL_ERR_VALUE, "non-finite xi_out");
    return SGL_OK;
}

}  // namespace sglh

extern "C" {

void sgl_invert_opts_default(sgl_invert_opts* o) {
    if (!o) return;
    o->precision = SGL_FP64;
    o->tail_box = 1;
    o->phi_tol = 1e-8;
    o->n_xi_wide = 500;
    o->n_k_int = 2400;
    o->xi_reach = 24.0;
    o->window = 0;
}

sgl_status sgl_pdf(sgl_ctx* ctx, const double* xi_out, int n_xi, const sgl_invert_opts* opts, double* P_out,
                   sgl_invert_meta* meta) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->has_cells) return fail(ctx, SGL_ERR_STATE, "cells not set");
    CKS(check_xi_out(ctx, xi_out, n_xi, P_out));
    sgl_invert_opts o;
    CKS(check_opts(ctx, opts, o));
    CK(cudaSetDevice(ctx->device));
    CKS(sync_stream(ctx));
    GridPlan G;
    CKS(plan_grid(ctx, o, G));
    CKS(check_grid(ctx, G));
    const std::vector<double> kk = linspace(0.0, G.k_k_max, G.nk_k);
    const std::vector<double> kg = linspace(0.0, G.k_g_max, G.nk_g);
    const int nk = (int)G.nk_k, nkg = (int)G.nk_g;
    const size_t es = elem_size(o.precision);
    cudaEventRecord(ctx->ev[0], ctx->stream);
    // ---- Phi = exp(ln Phi) on the full grid
    void* Phi = ctx->arena.get("phi", 2ULL * nk * nkg * es);
    if (!Phi) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (phi)");
    if (o.precision == SGL_MIXED && (long long)ctx->w0.size() <= kMixedFp64LambdaCells) {
        // few cells: ln Phi is a sum of few large terms whose FP32 rounding does not average out (on a
        // 300-cell population carrying the weight of 80k the mixed tail error was 1.2e-3 with FP32
        // Lambda, 7.6e-4 with FP64 Lambda and FP32 transforms); for so few cells FP64 Lambda is cheap
        const long long npt = (long long)nk * nkg;
        DBUF(stage, double, "phi_in", 2 * npt);
        CKS(lambda_eval(ctx, SGL_FP64, kk.data(), nk, kg.data(), nkg, 1, stage, stage + npt));
        launch_phi_to_f32(stage, 2 * npt, (float*)Phi, ctx->stream);
        CKLAUNCH();
    } else {
        CKS(lambda_eval(ctx, o.precision, kk.data(), nk, kg.data(), nkg, 1, Phi, (char*)Phi + (size_t)nk * nkg * es));
    }
    return invert_phi(ctx, o, G, Phi, xi_out, n_xi, P_out, meta);
}

sgl_status sgl_plan_grid(sgl_ctx* ctx, const sgl_invert_opts* opts, sgl_grid* grid) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->has_cells) return fail(ctx, SGL_ERR_STATE, "cells not set");
    if (!grid) return fail(ctx, SGL_ERR_VALUE, "grid is NULL");
    sgl_invert_opts o;
    CKS(check_opts(ctx, opts, o));
    CK(cudaSetDevice(ctx->device));
    CKS(sync_stream(ctx));
    GridPlan G;
    CKS(plan_grid(ctx, o, G));
    CKS(check_grid(ctx, G));
    grid->nk_k = G.nk_k; grid->nk_g = G.nk_g; grid->n_kap = G.n_kap; grid->n_gam = G.n_gam;
    grid->k_k_max = G.k_k_max; grid->k_g_max = G.k_g_max; grid->kap_min = G.kap_min; grid->kap_max = G.kap_max;
    grid->gam_max = G.gam_max; grid->sigma = G.sigma;
    grid->phi_at_k_cut = G.phic[0]; grid->phi_at_g_cut = G.phic[1];
    return SGL_OK;
}

sgl_status sgl_invert(sgl_ctx* ctx, const double* phi_re, const double* phi_im, int phi_on_device, const sgl_grid* grid,
                      const double* xi_out, int n_xi, const sgl_invert_opts* opts, double* P_out, sgl_invert_meta* meta) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!grid || !phi_re || !phi_im) return fail(ctx, SGL_ERR_VALUE, "grid or Phi is NULL");
    CKS(check_xi_out(ctx, xi_out, n_xi, P_out));
    sgl_invert_opts o;
    CKS(check_opts(ctx, opts, o));
    if (!(grid->sigma > 0) || !std::isfinite(grid->sigma) || !(grid->k_k_max > 0) || !(grid->k_g_max > 0) ||
        !std::isfinite(grid->k_k_max) || !std::isfinite(grid->k_g_max))
        return fail(ctx, SGL_ERR_VALUE, "invalid grid (sigma and the k extents must be positive and finite)");
    CK(cudaSetDevice(ctx->device));
    CKS(sync_stream(ctx));
    // the box follows sigma as in sgl_pdf; the k extents, the k sizes and the output grid sizes
    // are the caller's (a grid from sgl_plan_grid reproduces sgl_pdf exactly)
    GridPlan G;
    double dk_k, dk_g;
    box_for_sigma(o, grid->sigma, G, dk_k, dk_g);
    G.nk_k = grid->nk_k; G.nk_g = grid->nk_g; G.n_kap = grid->n_kap; G.n_gam = grid->n_gam;
    G.k_k_max = grid->k_k_max; G.k_g_max = grid->k_g_max;
    G.kap_min = grid->kap_min; G.kap_max = grid->kap_max; G.gam_max = grid->gam_max;
    G.phic[0] = grid->phi_at_k_cut; G.phic[1] = grid->phi_at_g_cut;
    if (!(G.kap_max > G.kap_min) || !(G.gam_max > 0)) return fail(ctx, SGL_ERR_VALUE, "invalid output box");
    CKS(check_grid(ctx, G));
    const long long npt = G.nk_k * G.nk_g;
    const size_t es = elem_size(o.precision);
    cudaEventRecord(ctx->ev[0], ctx->stream);
    void* Phi = ctx->arena.get("phi", 2ULL * npt * es);
    if (!Phi) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (phi)");
    const cudaMemcpyKind kind = phi_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (o.precision == SGL_FP64) {
        CK(cudaMemcpyAsync(Phi, phi_re, (size_t)npt * 8, kind, ctx->stream));
        CK(cudaMemcpyAsync((char*)Phi + (size_t)npt * 8, phi_im, (size_t)npt * 8, kind, ctx->stream));
    } else {
        DBUF(stage, double, "phi_in", 2 * npt);
        CK(cudaMemcpyAsync(stage, phi_re, (size_t)npt * 8, kind, ctx->stream));
        CK(cudaMemcpyAsync(stage + npt, phi_im, (size_t)npt * 8, kind, ctx->stream));
        launch_phi_to_f32(stage, 2 * npt, (float*)Phi, ctx->stream);
        CKLAUNCH();
    }
    return invert_phi(ctx, o, G, Phi, xi_out, n_xi, P_out, meta);
}

}  // extern "C"
