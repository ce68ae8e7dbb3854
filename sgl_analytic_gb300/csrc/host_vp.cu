// The positive (vp) Cox closure: closure upload and run sorting (sgl_vp_set), ln R on a tensor
// grid, and the xi term it replaces (Closure.qxi: unwrapped ln R minus the shear term).
#include "host.cuh"

namespace sglh {

void unwrap_line(double* p, int n, long long stride) {
    double corr = 0.0;
    for (int i = 1; i < n; ++i) {
        const double dd = p[(long long)i * stride] - (p[(long long)(i - 1) * stride] - corr);
        double ddmod = std::fmod(dd + M_PI, 2.0 * M_PI);
        if (ddmod < 0) ddmod += 2.0 * M_PI;
        ddmod -= M_PI;
        if (ddmod == -M_PI && dd > 0) ddmod = M_PI;
        double pc = ddmod - dd;
        if (std::fabs(dd) < M_PI) pc = 0.0;
        corr += pc;
        p[(long long)i * stride] += corr;
    }
}

// ln R on kv x qv into device planes (tables, z buffer from the arena; rows in passes of <= 8 GiB z)
sgl_status vp_lnR_device(sgl_ctx* ctx, int precision, const double* d_kv, int nk, const double* d_qv, int nq,
                         double* d_re, double* d_im) {
    const VpDevice& D = ctx->vpd;
    void* tables = ctx->arena.get("vp_tables", vp_table_bytes(precision, D.U, nk, nq));
    const int rows = vp_rows_per_pass(D.nsh, nk, nq, (size_t)8 << 30);
    const int pieces = rows == nk ? vp_pieces(D.nsh, rows, nq) : 1;     // split runs only in a single pass
    void* zb = ctx->arena.get("vp_z", (size_t)D.nsh * 49 * 16 * (size_t)rows * nq * pieces);
    if (!tables || !zb) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (vp)");
    const double pts = (double)nk * nq;
    Timed t(ctx, precision == SGL_FP64 ? "vp_lnR_f64" : "vp_lnR_mixed", pts * (double)D.ncells * 12.0,
            pts * D.nsh * 49 * 16.0 * 2);
    launch_vp_lnR(precision, D, d_kv, nk, d_qv, nq, tables, (double2*)zb, rows, d_re, d_im, ctx->stream, pieces);
    CKLAUNCH();
    return SGL_OK;
}

// vp closure term on kk x kg (Closure.qxi, pos_closure.py:690-705): ln R, its imaginary part
// unwrapped along k_kappa at the first k_gamma column and then along k_gamma, minus
// shear_var kg^2 / 4.  Device planes out.
sgl_status vp_qxi(sgl_ctx* ctx, int precision, const double* d_kk, int nk, const double* d_kg, const double* h_kg,
                  int nkg, double* d_re, double* d_im) {
    const cudaStream_t st = ctx->stream;
    CKS(vp_lnR_device(ctx, precision, d_kk, nk, d_kg, nkg, d_re, d_im));
    const long long npt = (long long)nk * nkg;
    std::vector<double> im((size_t)npt), re((size_t)npt);
    CK(cudaMemcpyAsync(im.data(), d_im, npt * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(re.data(), d_re, npt * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKS(sync_stream(ctx));
    unwrap_line(im.data(), nk, nkg);                              // first column along k_kappa
    for (int i = 0; i < nk; ++i) unwrap_line(im.data() + (long long)i * nkg, nkg, 1);
    for (long long e2 = 0; e2 < npt; ++e2) {
        const double q = h_kg[e2 % nkg];
        re[(size_t)e2] -= 0.25 * ctx->vp_shear * q * q;
    }
    CKS(upload(ctx, d_re, re.data(), (size_t)npt));
    CKS(upload(ctx, d_im, im.data(), (size_t)npt));
    CKS(sync_stream(ctx));
    return SGL_OK;
}

}  // namespace sglh

extern "C" {

sgl_status sgl_vp_set(sgl_ctx* ctx, int nstate, const double* u, const double* w, int n_shells, const double* K,
                      int n_unique, const double* ku, const double* gu, int64_t n_cells, const int32_t* cu,
                      const double* cw, int n_groups, const int64_t* gstart, const int32_t* sh_g, const double* ga,
                      const double* gb, const double* gc, const int32_t* glo, const int32_t* ghi, double shear_var) {
    if (!ctx) return SGL_ERR_VALUE;
    if (n_shells == 0) { ctx->vp_on = false; return SGL_OK; }
    if (nstate != 48) return fail(ctx, SGL_ERR_UNSUPPORTED, "vp closure: only the 48-state chain is built");
    if (n_shells < 0 || n_unique < 1 || n_cells < 0 || n_groups < 0 || !u || !w || !ku || !gu || !gstart || !sh_g ||
        (n_shells > 1 && !K) || (n_cells > 0 && (!cu || !cw)) || (n_groups > 0 && (!ga || !gb || !gc || !glo || !ghi)))
        return fail(ctx, SGL_ERR_VALUE, "vp closure: missing arrays");
    if (!std::isfinite(shear_var) || shear_var < 0) return fail(ctx, SGL_ERR_VALUE, "vp closure: shear_var must be finite, >= 0");
    for (int j = 0; j < nstate; ++j)
        if (!std::isfinite(u[j]) || !std::isfinite(w[j]) || (j > 0 && !(u[j] > u[j - 1])))
            return fail(ctx, SGL_ERR_VALUE, "vp closure: state nodes must be finite and increasing");
    for (long long e = 0; e < (long long)(n_shells - 1) * nstate * nstate; ++e)
        if (!std::isfinite(K[e])) return fail(ctx, SGL_ERR_VALUE, "vp closure: non-finite transition matrix");
    for (int i = 0; i < n_unique; ++i)
        if (!std::isfinite(ku[i]) || !std::isfinite(gu[i])) return fail(ctx, SGL_ERR_VALUE, "vp closure: non-finite cell");
    for (int64_t c = 0; c < n_cells; ++c)
        if (cu[c] < 0 || cu[c] >= n_unique || !std::isfinite(cw[c]))
            return fail(ctx, SGL_ERR_VALUE, "vp closure: cell index out of range or non-finite weight");
    if (sh_g[0] != 0 || sh_g[n_shells] != n_groups) return fail(ctx, SGL_ERR_VALUE, "vp closure: shell offsets must span the groups");
    for (int s = 0; s < n_shells; ++s)
        if (sh_g[s + 1] < sh_g[s]) return fail(ctx, SGL_ERR_VALUE, "vp closure: shell offsets must be non-decreasing");
    if (gstart[0] != 0 || gstart[n_groups] != n_cells) return fail(ctx, SGL_ERR_VALUE, "vp closure: group offsets must span the cells");
    for (int g = 0; g < n_groups; ++g) {
        if (gstart[g + 1] < gstart[g]) return fail(ctx, SGL_ERR_VALUE, "vp closure: group offsets must be non-decreasing");
        if (!std::isfinite(ga[g]) || !std::isfinite(gb[g])) return fail(ctx, SGL_ERR_VALUE, "vp closure: non-finite rate");
        if (glo[g] < 0 || ghi[g] >= nstate || glo[g] > ghi[g]) return fail(ctx, SGL_ERR_VALUE, "vp closure: bad rate interval");
        // rate intervals (pos_closure_fused.py:18-48): c = 0 on all states, or c = -1 on an interval
        // that reaches one end of the state grid
        if (gc[g] == -1.0) {
            if (ghi[g] != nstate - 1 && glo[g] != 0)
                return fail(ctx, SGL_ERR_VALUE, "vp closure: clipped rate support must reach an end of the state grid");
        } else if (gc[g] != 0.0) {
            return fail(ctx, SGL_ERR_VALUE, "vp closure: rate offset c must be 0 or -1");
        }
    }
    // zero stationary mean of every rate (pos_closure.py:15): the kernels rely on it
    for (int g = 0; g < n_groups; ++g) {
        double m = 0.0, mx = 0.0;
        for (int j = 0; j < nstate; ++j) {
            double D;
            if (gc[g] == 0.0) D = ga[g] * u[j] + gb[g];
            else if (j < glo[g] || j > ghi[g]) D = -1.0;
            else D = -1.0 + (u[j] - u[ghi[g] == nstate - 1 ? glo[g] : ghi[g]]) * ga[g] + gb[g];
            m += w[j] * D;
            mx = std::max(mx, std::fabs(D));
        }
        if (std::fabs(m) > 1e-11 * std::max(mx, 1e-300) && mx > 0)
            return fail(ctx, SGL_ERR_VALUE, "vp closure: a group's rate does not keep the mean (E_w[lam] != 1)");
    }
    // runs: per shell, groups ordered linear first, then by the first state they change
    // (left: lo, right: hi + 1); cells concatenated with weights (w a, w b)
    std::vector<int> cu_s, run_kind, run_bound, sh_run{0};
    std::vector<double2> wab;
    std::vector<float2> wabf;
    std::vector<long long> run_cell{0};
    cu_s.reserve((size_t)n_cells); wab.reserve((size_t)n_cells); wabf.reserve((size_t)n_cells);
    for (int sh = 0; sh < n_shells; ++sh) {
        std::vector<std::pair<int, int>> keyed;        // (sort key, group)
        for (int g = sh_g[sh]; g < sh_g[sh + 1]; ++g) {
            if (ga[g] == 0.0 && gb[g] == 0.0 && gc[g] == 0.0) continue;
            if (gstart[g + 1] == gstart[g]) continue;
            int key;
            if (gc[g] == 0.0) key = -1;
            else if (ghi[g] == nstate - 1) key = 2 * glo[g];            // left
            else key = 2 * (ghi[g] + 1) + 1;                            // right
            keyed.emplace_back(key, g);
        }
        std::stable_sort(keyed.begin(), keyed.end(), [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
            return x.first < y.first;
        });
        int cur_key = INT32_MIN;
        for (const auto& kg : keyed) {
            const int g = kg.second;
            if (kg.first != cur_key) {
                if (cur_key != INT32_MIN) run_cell.push_back((long long)cu_s.size());
                cur_key = kg.first;
                run_kind.push_back(gc[g] == 0.0 ? 0 : (ghi[g] == nstate - 1 ? 1 : 2));
                run_bound.push_back(gc[g] == 0.0 ? 0 : (ghi[g] == nstate - 1 ? glo[g] : ghi[g]));
            }
            for (int64_t c = gstart[g]; c < gstart[g + 1]; ++c) {
                cu_s.push_back(cu[c]);
                const double2 v = make_double2(cw[c] * ga[g], cw[c] * gb[g]);
                wab.push_back(v);
                wabf.push_back(make_float2((float)v.x, (float)v.y));
            }
        }
        if (cur_key != INT32_MIN) run_cell.push_back((long long)cu_s.size());
        sh_run.push_back((int)run_kind.size());
    }
    const int nruns = (int)run_kind.size();
    const long long ncs = (long long)cu_s.size();
    CK(cudaSetDevice(ctx->device));
    VpDevice D;
    D.nsh = n_shells; D.U = n_unique; D.nruns = nruns; D.ncells = ncs;
    DBUF(d_u, double, "vp_u", nstate);
    DBUF(d_w, double, "vp_w", nstate);
    DBUF(d_K, double, "vp_K", std::max<long long>(1, (long long)(n_shells - 1) * nstate * nstate));
    DBUF(d_ku, double, "vp_ku", n_unique);
    DBUF(d_gu, double, "vp_gu", n_unique);
    DBUF(d_cu, int, "vp_cu", std::max<long long>(1, ncs));
    DBUF(d_wab, double2, "vp_wab", std::max<long long>(1, ncs));
    DBUF(d_wabf, float2, "vp_wabf", std::max<long long>(1, ncs));
    DBUF(d_rc, long long, "vp_run_cell", nruns + 1);
    DBUF(d_rk, int, "vp_run_kind", 2 * std::max(1, nruns));
    DBUF(d_sr, int, "vp_sh_run", n_shells + 1);
    CKS(upload(ctx, d_u, u, nstate));
    CKS(upload(ctx, d_w, w, nstate));
    if (n_shells > 1) CKS(upload(ctx, d_K, K, (size_t)(n_shells - 1) * nstate * nstate));
    CKS(upload(ctx, d_ku, ku, n_unique));
    CKS(upload(ctx, d_gu, gu, n_unique));
    if (ncs > 0) {
        CKS(upload(ctx, d_cu, cu_s.data(), (size_t)ncs));
        CKS(upload(ctx, d_wab, wab.data(), (size_t)ncs));
        CKS(upload(ctx, d_wabf, wabf.data(), (size_t)ncs));
    }
    CKS(upload(ctx, d_rc, run_cell.data(), run_cell.size()));
    if (nruns > 0) {
        CKS(upload(ctx, d_rk, run_kind.data(), (size_t)nruns));
        CKS(upload(ctx, d_rk + nruns, run_bound.data(), (size_t)nruns));
    }
    CKS(upload(ctx, d_sr, sh_run.data(), sh_run.size()));
    CKS(sync_stream(ctx));
    D.u = d_u; D.w = d_w; D.K = d_K; D.ku = d_ku; D.gu = d_gu; D.cu = d_cu; D.wab = d_wab; D.wabf = d_wabf;
    D.run_cell = d_rc; D.run_kind = d_rk; D.run_bound = d_rk + nruns; D.sh_run = d_sr;
    ctx->vpd = D;
    ctx->vp_shear = shear_var;
    ctx->vp_xi_coarse = kXiCoarse;
    ctx->vp_xi_coarse_k = 0;
    ctx->vp_on = true;
    return SGL_OK;
}

sgl_status sgl_vp_lnR(sgl_ctx* ctx, const double* kv, int nk, const double* qv, int nq, int precision,
                      double* out_re, double* out_im) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->vp_on) return fail(ctx, SGL_ERR_STATE, "vp closure not set");
    if (nk < 1 || nq < 1 || !kv || !qv || !out_re || !out_im) return fail(ctx, SGL_ERR_VALUE, "empty grid");
    if (precision != SGL_FP64 && precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    for (int i = 0; i < nk; ++i) if (!std::isfinite(kv[i])) return fail(ctx, SGL_ERR_VALUE, "non-finite k_kappa");
    for (int i = 0; i < nq; ++i) if (!std::isfinite(qv[i])) return fail(ctx, SGL_ERR_VALUE, "non-finite k_gamma");
    CK(cudaSetDevice(ctx->device));
    const long long npt = (long long)nk * nq;
    DBUF(d_kv, double, "vpr_k", nk);
    DBUF(d_qv, double, "vpr_q", nq);
    DBUF(d_o, double, "vpr_out", 2 * npt);
    CKS(upload(ctx, d_kv, kv, nk));
    CKS(upload(ctx, d_qv, qv, nq));
    CKS(vp_lnR_device(ctx, precision, d_kv, nk, d_qv, nq, d_o, d_o + npt));
    CK(cudaMemcpyAsync(out_re, d_o, npt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(out_im, d_o + npt, npt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CKS(sync_stream(ctx));
    for (long long p = 0; p < npt; ++p)
        if (!std::isfinite(out_re[p]) || !std::isfinite(out_im[p])) return fail(ctx, SGL_ERR_NONFINITE, "non-finite ln R");
    return SGL_OK;
}

}  // extern "C"
