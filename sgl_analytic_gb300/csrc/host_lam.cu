// Population plans and ln Phi: the cell compaction and separable plan (Lam.__init__,
// _sep_gamma_nodes), the xi_lin group plans, and ln Phi on a tensor grid (Lam.__call__ /
// _direct_call: separable Psi_1, the gauss Psi_2 term with its coarse-grid spline).
#include "host.cuh"

namespace sglh {

// numpy's summation of a contiguous float64 array (np.sum): runs of at most 128 values summed with
// 8 interleaved partial sums combined pairwise, longer runs split in two at a multiple of 8
double pairwise_sum(const double* a, long long n) {
    if (n < 8) {
        double r = 0.0;
        for (long long i = 0; i < n; ++i) r += a[i];
        return r;
    }
    if (n <= 128) {
        double r[8];
        for (int j = 0; j < 8; ++j) r[j] = a[j];
        long long i = 8;
        for (; i < n - (n % 8); i += 8)
            for (int j = 0; j < 8; ++j) r[j] += a[i + j];
        double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
        for (; i < n; ++i) res += a[i];
        return res;
    }
    long long n2 = n / 2;
    n2 -= n2 % 8;
    return pairwise_sum(a, n2) + pairwise_sum(a + n2, n - n2);
}

// ------------------------------------------------------------------ separable plan
// Restates _sep_gamma_nodes (sgl_full.py:2631-2661) for kg_max = key.
sgl_status build_sep(sgl_ctx* ctx, double key, int nk) {
    if (ctx->sep.key == key && ctx->sep_precision_ready >= 0) return SGL_OK;
    HostTimer ht(ctx);
    const long long N = (long long)ctx->w0.size();
    const double* fe = ctx->fe_g.data();
    double t[kSepMg];
    for (int a = 0; a < kSepMg; ++a) {
        const int b = kSepMg - 1 - a;
        t[a] = std::cos((double)(2 * b + 1) * M_PI / (double)(2 * kSepMg));
    }
    // per-cell scratch kept in the context between calls (no fresh pages to fault in)
    SepScratch& S0 = ctx->sep_scratch;
    std::vector<long long>& keyv = S0.keyv;
    std::vector<double>& sl = S0.sl;
    std::vector<double>& sh = S0.sh;
    std::vector<char>& direct = S0.direct;
    keyv.resize((size_t)N); sl.resize((size_t)N); sh.resize((size_t)N);
    direct.assign((size_t)N, 0);
    std::atomic<int> below{0};                 // some cell lies below its gamma bin
    parallel_for(N, [&](long long c0, long long c1) {
        for (long long c = c0; c < c1; ++c) {
            const int b = ctx->ig[(size_t)c];
            const double lo = fe[b], hi = fe[b + 1], wd = hi - lo;
            double nsd = std::ceil(key * wd / (2.0 * kSepTheta));
            long long ns = std::max(1LL, (long long)nsd);
            if (ns > kSepSmax) { direct[(size_t)c] = 1; keyv[(size_t)c] = -1; continue; }
            long long j = (long long)((ctx->g0[(size_t)c] - lo) / wd * (double)ns);
            j = std::min(j, ns - 1);
            sl[(size_t)c] = lo + (double)j * wd / (double)ns;
            sh[(size_t)c] = lo + (double)(j + 1) * wd / (double)ns;
            keyv[(size_t)c] = (long long)b * (kSepSmax + 1) + j;
            if (j < 0) below = 1;
        }
    });
    ht.lap("sep_keys");
    // order: sep cells by sub-bin (the reference's np.unique over the sub-bins' lower edges
    // rounded to 14 decimals, ascending), then direct cells in original order.  A cell whose
    // gamma lies below its bin (possible in the reference's populations) gets a negative sub-bin
    // index, as in the reference (truncation toward zero, no lower clamp): its sub-bin lies below
    // the bin.  Without such cells, (bin, sub-bin) order is the lower-edge order and a stable
    // counting sort over the small key range gives it; with them, the sub-bins are ranked by
    // their rounded lower edges.
    std::vector<long long>& order = S0.order;
    order.resize((size_t)N);
    long long n_sep = 0;
    for (long long c = 0; c < N; ++c) n_sep += !direct[(size_t)c];
    if (!below) {
        long long kmax = -1;
        for (long long c = 0; c < N; ++c) kmax = std::max(kmax, keyv[(size_t)c]);
        std::vector<long long> cnt((size_t)(kmax + 2), 0);
        for (long long c = 0; c < N; ++c) if (!direct[(size_t)c]) ++cnt[(size_t)keyv[(size_t)c] + 1];
        for (size_t i = 1; i < cnt.size(); ++i) cnt[i] += cnt[i - 1];
        for (long long c = 0, d = n_sep; c < N; ++c) {
            if (direct[(size_t)c]) order[(size_t)d++] = c;
            else order[(size_t)cnt[(size_t)keyv[(size_t)c]]++] = c;
        }
    } else {
        std::vector<long long> edge((size_t)N, 0);
        long long d = 0, e = n_sep;
        for (long long c = 0; c < N; ++c) {
            if (direct[(size_t)c]) { order[(size_t)e++] = c; continue; }
            edge[(size_t)c] = std::llrint(sl[(size_t)c] * 1e14);
            order[(size_t)d++] = c;
        }
        std::stable_sort(order.begin(), order.begin() + n_sep,
                         [&](long long a, long long b) { return edge[(size_t)a] < edge[(size_t)b]; });
        // dense group keys in that order
        long long key = -1, prev_edge = 0;
        for (long long i = 0; i < n_sep; ++i) {
            const long long c = order[(size_t)i];
            if (i == 0 || edge[(size_t)c] != prev_edge) { ++key; prev_edge = edge[(size_t)c]; }
            keyv[(size_t)c] = key;
        }
    }
    const long long n_dir = N - n_sep;

    ht.lap("sep_sort");
    std::vector<double>& kap = S0.kap;
    std::vector<double>& w = S0.w;
    std::vector<double>& wl = S0.wl;
    std::vector<float>& kh = S0.kh;
    std::vector<float>& kl = S0.kl;
    std::vector<float>& wf = S0.wf;
    std::vector<float>& wlf = S0.wlf;
    std::vector<int>& grp = S0.grp;
    kap.resize((size_t)N); w.resize((size_t)N); kh.resize((size_t)N); kl.resize((size_t)N); wf.resize((size_t)N);
    grp.resize((size_t)N);
    wl.assign((size_t)N * 8, 0.0);
    wlf.assign((size_t)N * 8, 0.f);
    std::vector<double> nodes;
    std::vector<int> gcol0, gncol;
    int ng = -1;
    long long prev = -2;
    double maxnode = 0.0;
    for (long long i = 0; i < n_sep; ++i) {
        const long long c = order[(size_t)i];
        if (keyv[(size_t)c] != prev) {
            ++ng; prev = keyv[(size_t)c];
            gcol0.push_back(ng * kSepMg); gncol.push_back(kSepMg);
            const double lo_s = sl[(size_t)c], hi_s = sh[(size_t)c];
            for (int a = 0; a < kSepMg; ++a) {
                const double v = 0.5 * (lo_s + hi_s) + (0.5 * (hi_s - lo_s)) * t[a];
                nodes.push_back(v);
                maxnode = std::max(maxnode, v);
            }
        }
        grp[(size_t)i] = ng;
    }
    ht.lap("sep_groups");
    // Lagrange weights of each separable cell at its sub-bin's Chebyshev nodes
    parallel_for(n_sep, [&](long long i0, long long i1) {
        for (long long i = i0; i < i1; ++i) {
            const long long c = order[(size_t)i];
            const double lo_s = sl[(size_t)c], hi_s = sh[(size_t)c];
            const double u = ((2.0 * ctx->g0[(size_t)c] - lo_s) - hi_s) / (hi_s - lo_s);
            for (int a = 0; a < kSepMg; ++a) {
                double L = 1.0;
                for (int b2 = 0; b2 < kSepMg; ++b2)
                    if (b2 != a) L = L * ((u - t[b2]) / (t[a] - t[b2]));
                wl[(size_t)i * 8 + a] = ctx->w0[(size_t)c] * L;
            }
        }
    });
    const int n_sep_groups = ng + 1;
    const int n_cols_sep = n_sep_groups * kSepMg;
    for (long long i = n_sep; i < N; ++i) {
        const long long c = order[(size_t)i];
        ++ng;
        gcol0.push_back(n_cols_sep + (int)(i - n_sep));
        gncol.push_back(1);
        grp[(size_t)i] = ng;
        wl[(size_t)i * 8] = ctx->w0[(size_t)c];
        nodes.push_back(ctx->g0[(size_t)c]);
    }
    const int n_groups = ng + 1;
    parallel_for(N, [&](long long i0, long long i1) {
        for (long long i = i0; i < i1; ++i) {
            const long long c = order[(size_t)i];
            kap[(size_t)i] = ctx->k0[(size_t)c];
            w[(size_t)i] = ctx->w0[(size_t)c];
            const ff f = ff_from_double(kap[(size_t)i]);
            kh[(size_t)i] = f.hi; kl[(size_t)i] = f.lo;
            wf[(size_t)i] = (float)w[(size_t)i];
            for (int a = 0; a < 8; ++a) wlf[(size_t)i * 8 + a] = (float)wl[(size_t)i * 8 + a];
        }
    });
    ht.lap("sep_weights");
    // chunks of whole groups: one wave of ~8 CTAs per SM over (row tiles x chunks); the mixed
    // sweep's 4-warp CTAs are latency-bound, so residency is what feeds its pipes
    const int row_tiles = std::max(1, ceil_div(nk, 128));
    int nchunks = std::max(1, std::min(n_groups, 8 * kNumSMs / row_tiles));
    const long long target = std::max(1LL, (N + nchunks - 1) / nchunks);
    std::vector<int> cb{0};
    long long acc = 0;
    for (long long i = 0; i < N; ++i) {
        if (i > 0 && grp[(size_t)i] != grp[(size_t)i - 1] && acc >= target) { cb.push_back((int)i); acc = 0; }
        ++acc;
    }
    cb.push_back((int)N);

    SepHost& S = ctx->sep;
    S.key = key; S.version++; S.n_cells = (int)N; S.n_groups = n_groups; S.n_cols_sep = n_cols_sep;
    S.n_cols = n_cols_sep + (int)n_dir; S.n_direct = (int)n_dir; S.chunk_begin = cb; S.max_sep_node = maxnode;

    ht.lap("sep_chunks");
    DBUF(d_kap, double, "sep_kap", N);
    DBUF(d_w, double, "sep_w", N);
    DBUF(d_wl, double, "sep_wl", N * 8);
    DBUF(d_kh, float, "sep_kh", N);
    DBUF(d_kl, float, "sep_kl", N);
    DBUF(d_wf, float, "sep_wf", N);
    DBUF(d_wlf, float, "sep_wlf", N * 8);
    DBUF(d_grp, int, "sep_grp", N);
    DBUF(d_gc0, int, "sep_gcol0", n_groups);
    DBUF(d_gnc, int, "sep_gncol", n_groups);
    DBUF(d_cb, int, "sep_chunks", cb.size());
    DBUF(d_nodes, double, "sep_nodes", nodes.size());
    CKS(upload(ctx, d_kap, kap.data(), kap.size()));
    CKS(upload(ctx, d_w, w.data(), w.size()));
    CKS(upload(ctx, d_wl, wl.data(), wl.size()));
    CKS(upload(ctx, d_kh, kh.data(), kh.size()));
    CKS(upload(ctx, d_kl, kl.data(), kl.size()));
    CKS(upload(ctx, d_wf, wf.data(), wf.size()));
    CKS(upload(ctx, d_wlf, wlf.data(), wlf.size()));
    CKS(upload(ctx, d_grp, grp.data(), grp.size()));
    CKS(upload(ctx, d_gc0, gcol0.data(), gcol0.size()));
    CKS(upload(ctx, d_gnc, gncol.data(), gncol.size()));
    CKS(upload(ctx, d_cb, cb.data(), cb.size()));
    CKS(upload(ctx, d_nodes, nodes.data(), nodes.size()));
    CK(cudaStreamSynchronize(ctx->stream));   // host staging vectors go out of scope
    ctx->pinned_off = 0;
    SepDevice& D = ctx->sepd;
    D.n_cells = (int)N; D.n_groups = n_groups; D.n_cols = S.n_cols; D.n_cols_sep = n_cols_sep;
    D.nchunks = (int)cb.size() - 1;
    D.kap = d_kap; D.w = d_w; D.wl = d_wl; D.kap_hi = d_kh; D.kap_lo = d_kl; D.w_f = d_wf; D.wl_f = d_wlf;
    D.grp = d_grp; D.gcol0 = d_gc0; D.gncol = d_gnc; D.chunk_begin = d_cb;
    ctx->sep_precision_ready = 1;
    ht.lap("sep_upload");
    return SGL_OK;
}

// ------------------------------------------------------------------ spline (not-a-knot)
// Cubic B-spline basis at s for knots t (ncoef coefficients): interval l and 4 values.
void bspline_basis_host(const std::vector<double>& t, int ncoef, double s, int& l0, double N[4]) {
    int lo = 3, hi = ncoef - 1;
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (t[(size_t)mid] <= s) lo = mid; else hi = mid - 1; }
    const int l = lo;
    double left[4], right[4];
    N[0] = 1.0;
    for (int j = 1; j <= 3; ++j) {
        left[j] = s - t[(size_t)(l + 1 - j)];
        right[j] = t[(size_t)(l + j)] - s;
        double saved = 0.0;
        for (int r = 0; r < j; ++r) {
            const double temp = N[r] / (right[r + 1] + left[j - r]);
            N[r] = saved + right[r + 1] * temp;
            saved = left[j - r] * temp;
        }
        N[j] = saved;
    }
    l0 = l - 3;
}

// Knots of the not-a-knot cubic interpolant on s = linspace(0, 1, n) and the inverse of its
// collocation matrix (coefficients = Minv @ values), as make_interp_spline(s, y, k=3) builds.
bool spline_setup(SplineHost& S, int n) {
    if (S.n == n) return true;
    const std::vector<double> s = linspace(0.0, 1.0, n);
    std::vector<double> t;
    for (int i = 0; i < 4; ++i) t.push_back(s[0]);
    for (int i = 2; i < n - 2; ++i) t.push_back(s[(size_t)i]);
    for (int i = 0; i < 4; ++i) t.push_back(s[(size_t)n - 1]);
    std::vector<double> A((size_t)n * n, 0.0), I((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) {
        int l0; double N[4];
        bspline_basis_host(t, n, s[(size_t)i], l0, N);
        for (int a = 0; a < 4; ++a) A[(size_t)i * n + l0 + a] = N[a];
        I[(size_t)i * n + i] = 1.0;
    }
    // Gauss-Jordan with partial pivoting
    for (int col = 0; col < n; ++col) {
        int piv = col;
        for (int r = col + 1; r < n; ++r) if (std::fabs(A[(size_t)r * n + col]) > std::fabs(A[(size_t)piv * n + col])) piv = r;
        if (A[(size_t)piv * n + col] == 0.0) return false;
        if (piv != col)
            for (int k = 0; k < n; ++k) { std::swap(A[(size_t)piv * n + k], A[(size_t)col * n + k]); std::swap(I[(size_t)piv * n + k], I[(size_t)col * n + k]); }
        const double d = A[(size_t)col * n + col];
        for (int k = 0; k < n; ++k) { A[(size_t)col * n + k] /= d; I[(size_t)col * n + k] /= d; }
        for (int r = 0; r < n; ++r) {
            if (r == col) continue;
            const double f = A[(size_t)r * n + col];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) { A[(size_t)r * n + k] -= f * A[(size_t)col * n + k]; I[(size_t)r * n + k] -= f * I[(size_t)col * n + k]; }
        }
    }
    S.n = n; S.knots = t; S.minv = I;
    return true;
}

// ------------------------------------------------------------------ xi_lin term on a grid
// Exact Psi_2 on kk x kg (device in/out, double planes).  1-D fast paths for the probes.
sgl_status xi_eval(sgl_ctx* ctx, int precision, const double* d_kk, const double* h_kk, int nk, const double* d_kg,
                   const double* h_kg, int nkg, double* d_re, double* d_im) {
    XiHost& X = ctx->xi;
    const cudaStream_t st = ctx->stream;
    if (nkg == 1 && h_kg[0] == 0.0 && X.R0 > 0) {
        DBUF(d_part, double, "xi_line_part", 2LL * kLineChunks * nk);
        launch_xi_line_k(ctx->xid, d_kk, nk, d_re, d_im, d_part, st); CKLAUNCH(); return SGL_OK;
    }
    if (nk == 1 && h_kk[0] == 0.0 && (X.Rm[0] + X.Rm[1] + X.Rm[2]) > 0) {
        DBUF(d_part, double, "xi_line_part", 2LL * kLineChunks * nkg);
        launch_xi_line_g(ctx->xid, d_kg, nkg, d_re, d_im, d_part, st); CKLAUNCH(); return SGL_OK;
    }
    if (precision == SGL_MIXED && xi_fused_fits(ctx->xid.r_max, nk, X.n_gmc)) {
        // fused tcgen05 form: per (group, tile of <= 8 k_gamma columns) one CTA builds T in shared
        // memory, contracts it with the packed E in TMEM and squares in its epilogue
        const int ng = X.n_groups;
        std::vector<int> jt(ng);
        std::vector<long long> pre(3LL * ng + 2, 0);      // cta_prefix | padded-p prefix | E offsets
        long long* cta_prefix = pre.data();
        long long* pp_prefix = pre.data() + ng + 1;
        long long* e_off = pre.data() + 2 * (ng + 1);
        double fl = 0.0;
        for (int g = 0; g < ng; ++g) {
            jt[g] = xi_fused_jt(X.r[g]);
            cta_prefix[g + 1] = cta_prefix[g] + (nkg + jt[g] - 1) / jt[g];
            e_off[g] = pp_prefix[g] * 512;                  // 32 KB of packed E per 16 p
            pp_prefix[g + 1] = pp_prefix[g] + 16LL * ((X.nP[g] + 15) / 16);
            fl += 2.0 * (2.0 * nk) * ((double)X.r[g] * nkg) * X.nP[g];
        }
        DBUF(d_jt, int, "xf_jt", ng);
        DBUF(d_pre, long long, "xf_prefix", pre.size());
        CKS(upload(ctx, d_jt, jt.data(), (size_t)ng));
        CKS(upload(ctx, d_pre, pre.data(), pre.size()));
        float* J = (float*)ctx->arena.get("xi_J", 4ULL * X.n_gmc * nkg * sizeof(float));
        if (!J) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (xi)");
        DBUF(Epk, float, "xf_E", std::max<long long>(1, pp_prefix[ng] * 512));
        DBUF(part, float2, "xf_part", (long long)ng * nkg * nk);
        DBUF(d_Vf, float, "xi_Vf", (long long)X.total_rows * nkg);
        DBUF(d_kres, float2, "xi_kres", (long long)nk * X.total_rows);
        DBUF(d_hq, float2, "xi_hq", (long long)X.total_rows * nkg);
        DBUF(d_J64, double, "xi_J64", 4LL * X.n_gmc * nkg);
        const long long* d_pp = (const long long*)ctx->arena.find("xi_pprefix");
        int* err = dev_err_flag(ctx);
        if (!err) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (error flag)");
        launch_bessel_tables(SGL_MIXED, ctx->xid.gmc, X.n_gmc, d_kg, nkg, J, st); CKLAUNCH();
        launch_xi_E_pack(ctx->xid, d_kk, nk, d_pre + (ng + 1), pp_prefix[ng], d_pp, d_pre + 2 * (ng + 1), Epk, st);
        CKLAUNCH();
        launch_bessel_tables(SGL_FP64, ctx->xid.gmc, X.n_gmc, d_kg, nkg, d_J64, st); CKLAUNCH();
        launch_xi_V_mixed(ctx->xid, d_J64 + 3LL * X.n_gmc * nkg, nkg, d_Vf, X.total_rows, d_kk, nk, d_kg, d_kres, d_hq,
                          st, 1);
        CKLAUNCH();
        {
            Timed t(ctx, "xi_fused", fl, 0.0);
            launch_xi_fused(ctx->xid, d_pp, d_pp + (ng + 1), d_jt, d_pre, cta_prefix[ng], d_pre + 2 * (ng + 1), Epk, J,
                            d_Vf, d_kres, d_hq, nk, nkg, part, err, d_re, d_im, st);
        }
        CKLAUNCH();
        return SGL_OK;
    }
    const size_t es = elem_size(precision);
    // offsets
    std::vector<long long> T_off(X.n_groups), E_off(X.n_groups), G_off(X.n_groups);
    long long tT = 0, tE = 0, tG = 0;
    for (int g = 0; g < X.n_groups; ++g) {
        T_off[g] = tT; E_off[g] = tE; G_off[g] = tG;
        tT += (long long)X.nP[g] * X.r[g] * nkg;
        tE += 2LL * nk * X.nP[g];
        tG += 2LL * nk * X.r[g] * nkg;
    }
    DBUF(d_off, long long, "xi_off", 3 * X.n_groups);
    CKS(upload(ctx, d_off, T_off.data(), X.n_groups));
    CKS(upload(ctx, d_off + X.n_groups, E_off.data(), X.n_groups));
    CKS(upload(ctx, d_off + 2 * X.n_groups, G_off.data(), X.n_groups));
    // mixed path: stage A writes the tensor-core GEMM's packed A operand directly
    const bool fused = precision == SGL_MIXED && xi_stageA_pack_fits(ctx->xid.r_max, nkg);
    void* J = ctx->arena.get("xi_J", 4ULL * X.n_gmc * nkg * es);
    void* T = fused ? nullptr : ctx->arena.get("xi_T", (size_t)tT * es);
    void* E = ctx->arena.get("xi_E", (size_t)tE * es);
    void* G = ctx->arena.get("xi_G", (size_t)tG * es);
    if (!J || (!T && !fused) || !E || !G) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (xi)");
    const long long* d_pp = (const long long*)ctx->arena.find("xi_pprefix");
    launch_bessel_tables(precision, ctx->xid.gmc, X.n_gmc, d_kg, nkg, J, st); CKLAUNCH();
    if (!fused) {
        Timed t(ctx, "xi_stageA", 0.0, (double)tT * es);
        launch_xi_stageA(precision, ctx->xid, d_pp, X.total_p, d_off, J, nkg, T, st);
    }
    CKLAUNCH();
    launch_xi_E(precision, ctx->xid, d_kk, nk, d_off + X.n_groups, d_pp, X.total_p, E, st); CKLAUNCH();
    if (fused) {
        // G^T (N x 2nk) = T^T (N x nP) E^T (nP x 2nk); T^T produced packed by stage A
        std::vector<TcGemmDesc> v;
        std::vector<long long> chunk_prefix;
        long long nchunks = 0;
        for (int g = 0; g < X.n_groups; ++g) {
            const int N = X.r[g] * nkg;
            TcGemmDesc t{};
            t.M = N; t.N = 2 * nk; t.K = X.nP[g];
            t.A = nullptr; t.a_rs = 1; t.a_cs = N;
            t.B = (const float*)E + E_off[g]; t.b_rs = 1; t.b_cs = X.nP[g];
            t.C = (float*)G + G_off[g]; t.c_rs = 1; t.c_cs = N;
            t.alpha = 1.f;
            v.push_back(t);
            chunk_prefix.push_back(nchunks);
            nchunks += 4LL * ((X.nP[g] + 15) / 16);
        }
        std::vector<TcPackDesc> pk(2 * v.size());
        int tiles = 0;
        long long quads = 0;
        const long long pfl = tc_gemm_plan(v.data(), (int)v.size(), 2, pk.data(), &tiles, &quads, false);
        DBUF(dd, TcGemmDesc, "tc_desc_xi", v.size());
        DBUF(dpk, TcPackDesc, "tc_pack_xi", pk.size());
        DBUF(dcp, long long, "xi_chunk_prefix", chunk_prefix.size());
        DBUF(packed, float, "tc_packed_xi", std::max<long long>(pfl, 1));
        CKS(upload(ctx, dd, v.data(), v.size()));
        CKS(upload(ctx, dpk, pk.data(), pk.size()));
        CKS(upload(ctx, dcp, chunk_prefix.data(), chunk_prefix.size()));
        int* err = dev_err_flag(ctx);
        if (!err) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (error flag)");
        {
            Timed t(ctx, "xi_stageA", 0.0, (double)pfl * 4.0);
            launch_xi_stageA_pack(ctx->xid, d_pp, (const float*)J, nkg, dcp, nchunks, dd, packed, st);
        }
        CKLAUNCH();
        double fl = 0.0;
        for (auto& g : v) fl += 2.0 * g.M * (double)g.N * g.K;
        {
            Timed t(ctx, "gemm_tc_xi", fl, 0.0);
            launch_tc_gemm(2, dd, (int)v.size(), tiles, dpk, quads, packed, err, st);
        }
        CKLAUNCH();
    } else if (precision == SGL_FP64) {
        std::vector<GemmDesc<double>> v;
        for (int g = 0; g < X.n_groups; ++g) {
            const int N = X.r[g] * nkg;
            v.push_back(gd<double>(2 * nk, N, X.nP[g], (const double*)E + E_off[g], X.nP[g], 1,
                                   (const double*)T + T_off[g], N, 1, (double*)G + G_off[g], N));
        }
        CKS(run_gemms(ctx, v, "xi"));
    } else {
        // tensor cores, transposed so that the 2 nk rows of E fit one tile width:
        // G^T (N x 2nk) = T^T (N x nP) E^T (nP x 2nk)
        std::vector<TcGemmDesc> v;
        for (int g = 0; g < X.n_groups; ++g) {
            const int N = X.r[g] * nkg;
            TcGemmDesc t{};
            t.M = N; t.N = 2 * nk; t.K = X.nP[g];
            t.A = (const float*)T + T_off[g]; t.a_rs = 1; t.a_cs = N;
            t.B = (const float*)E + E_off[g]; t.b_rs = 1; t.b_cs = X.nP[g];
            t.C = (float*)G + G_off[g]; t.c_rs = 1; t.c_cs = N;
            t.alpha = 1.f;
            v.push_back(t);
        }
        CKS(run_tc_gemms(ctx, v, "xi", 2));
    }
    const int nsplit = std::max(1, std::min(X.n_groups, 16));
    DBUF(d_part, double, "xi_sq_part", 2LL * nsplit * nk * nkg);
    if (precision == SGL_MIXED) {
        // compensated m = 0 form: V = U (J0 - 1) in FP64 from an FP64 J0 - 1 table (rounded to FP32
        // where formed), and the float-float correction tables of the square kernel
        DBUF(d_Vf, float, "xi_Vf", (long long)X.total_rows * nkg);
        DBUF(d_kres, float2, "xi_kres", (long long)nk * X.total_rows);
        DBUF(d_hq, float2, "xi_hq", (long long)X.total_rows * nkg);
        DBUF(d_J64, double, "xi_J64", 4LL * X.n_gmc * nkg);
        launch_bessel_tables(SGL_FP64, ctx->xid.gmc, X.n_gmc, d_kg, nkg, d_J64, st); CKLAUNCH();
        launch_xi_V_mixed(ctx->xid, d_J64 + 3LL * X.n_gmc * nkg, nkg, d_Vf, X.total_rows, d_kk, nk, d_kg, d_kres, d_hq,
                          st);
        CKLAUNCH();
        Timed t(ctx, "xi_square", 0.0, (double)tG * es);
        launch_xi_square_mixed(ctx->xid, d_off + 2 * X.n_groups, (const float*)G, nk, nkg, d_Vf, d_kres, d_hq,
                               X.total_rows, nsplit, d_part, d_re, d_im, st);
    } else {
        Timed t(ctx, "xi_square", 0.0, (double)tG * es);
        launch_xi_square(precision, ctx->xid, d_off + 2 * X.n_groups, G, d_kk, nk, d_kg, nkg, nullptr, nsplit, d_part,
                         d_re, d_im, st);
    }
    CKLAUNCH();
    return SGL_OK;
}

// numpy.unwrap along a strided line (period 2 pi, discontinuity pi)
sgl_status xi_any(sgl_ctx* ctx, int precision, const double* d_kk, const double* h_kk, int nk, const double* d_kg,
                  const double* h_kg, int nkg, double* d_re, double* d_im) {
    if (ctx->vp_on) return vp_qxi(ctx, precision, d_kk, nk, d_kg, h_kg, nkg, d_re, d_im);
    return xi_eval(ctx, precision, d_kk, h_kk, nk, d_kg, h_kg, nkg, d_re, d_im);
}

// ------------------------------------------------------------------ Lambda on a grid
// Separable Psi_1 GEMM stage: writes the (2nk x nkg) plane pair of TT into Gout.
template <typename TT>
sgl_status sep_gemms(sgl_ctx* ctx, int precision, const double* h_kg, const double* d_kg, int nk, int nkg,
                     void* Tt, void* Gout) {
    SepHost& S = ctx->sep;
    const cudaStream_t st = ctx->stream;
    const double Kg = nkg ? h_kg[nkg - 1] : 0.0;
    const int Nch = (S.n_cols_sep > 0 && Kg > 0) ? (int)(0.65 * S.max_sep_node * Kg + 50.0) : 0;
    const long long ld = 2LL * nk;
    // mixed path: at least 2 K-slices, combined in float-float.  The FP32 kernel's compensated
    // blocked accumulation already bounds the rounding of the long K sums (sep1 runs over ~6000
    // gamma nodes): on the reference's z_s = 1 cells the PDF tail error against the reference is
    // 2.1e-4 with 2 slices, where plain FP32 chains needed 64 slices to get below 5.4e-4.  The
    // slice count is now a throughput choice.
    const int msplit = precision == SGL_FP64 ? 1 : 2;
    const double* d_nodes = (const double*)ctx->arena.find("sep_nodes");
    if (S.n_cols_sep > 0) {
        if (nkg > 1 && Nch > 0 && Nch < 0.6 * nkg && h_kg[0] >= 0.0) {
            DBUF(d_t, double, "cheb_t", Nch);
            void* Bc = ctx->arena.get("cheb_B", (size_t)S.n_cols_sep * Nch * sizeof(TT));
            void* L = ctx->arena.get("cheb_L", (size_t)nkg * Nch * sizeof(TT));
            void* U = ctx->arena.get("cheb_U", (size_t)ld * Nch * sizeof(TT));
            if (!Bc || !L || !U) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (cheb)");
            // the basis tables depend on the plan and the k_gamma grid only: kept between PDFs
            std::vector<double> key{(double)precision, (double)S.version, Kg, (double)Nch,
                                    (double)ctx->arena.generation("cheb_t"), (double)ctx->arena.generation("cheb_L")};
            key.insert(key.end(), h_kg, h_kg + nkg);
            if (!table_current(ctx, "cheb_B", key)) {
                launch_cheb_points(Kg, Nch, d_t, st); CKLAUNCH();
                launch_j0m1_table(precision, d_nodes, S.n_cols_sep, d_t, Nch, Bc, st); CKLAUNCH();
                launch_cheb_matrix(precision, Kg, Nch, d_t, d_kg, nkg, L, st); CKLAUNCH();
                table_built(ctx, "cheb_B", key);
            }
            CKS(gemm_splitk<TT>(ctx, gd<TT>((int)ld, Nch, S.n_cols_sep, Tt, 1, ld, Bc, Nch, 1, U, Nch), "sep1", msplit));
            CKS(gemm_splitk<TT>(ctx, gd<TT>((int)ld, nkg, Nch, U, Nch, 1, L, 1, Nch, Gout, nkg), "sep2", msplit));
        } else {
            void* Bn = ctx->arena.get("sep_Bn", (size_t)S.n_cols_sep * nkg * sizeof(TT));
            if (!Bn) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (Bn)");
            std::vector<double> key{(double)precision, (double)S.version};
            key.insert(key.end(), h_kg, h_kg + nkg);
            if (!table_current(ctx, "sep_Bn", key)) {
                launch_j0m1_table(precision, d_nodes, S.n_cols_sep, d_kg, nkg, Bn, st); CKLAUNCH();
                table_built(ctx, "sep_Bn", key);
            }
            CKS(gemm_splitk<TT>(ctx, gd<TT>((int)ld, nkg, S.n_cols_sep, Tt, 1, ld, Bn, nkg, 1, Gout, nkg), "sep1", msplit));
        }
    } else {
        CK(cudaMemsetAsync(Gout, 0, (size_t)ld * nkg * sizeof(TT), st));
    }
    if (S.n_direct > 0) {
        void* Bd = ctx->arena.get("sep_Bd", (size_t)S.n_direct * nkg * sizeof(TT));
        if (!Bd) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (Bd)");
        std::vector<double> key{(double)precision, (double)S.version};
        key.insert(key.end(), h_kg, h_kg + nkg);
        if (!table_current(ctx, "sep_Bd", key)) {
            launch_j0m1_table(precision, d_nodes + S.n_cols_sep, S.n_direct, d_kg, nkg, Bd, st); CKLAUNCH();
            table_built(ctx, "sep_Bd", key);
        }
        const TT* Td = (const TT*)Tt + (long long)S.n_cols_sep * ld;
        CKS(gemm_splitk<TT>(ctx, gd<TT>((int)ld, nkg, S.n_direct, Td, 1, ld, Bd, nkg, 1, Gout, nkg, 1.0, 1.0), "sep3", msplit));
    }
    return SGL_OK;
}

// ln Phi on kk x kg into device planes (Lam._direct_call, sgl_full.py:3088-3131):
//   Psi_1: separable for >= 200000 points and nkg > 1, dense direct sums otherwise;
//   -1/2 k^2 V;
//   xi term: 101^2 coarse grid + not-a-knot bicubic spline when the grid has more than 101^2
//   points (and both axes > 1 point, both maxima > 0), exact otherwise.
// write_phi = 1 writes Phi = exp(ln Phi) in the precision's element type (inversion path).
sgl_status lambda_eval(sgl_ctx* ctx, int precision, const double* h_kk, int nk, const double* h_kg, int nkg,
                       int write_phi, void* out_re, void* out_im) {
    cudaStream_t st = ctx->stream;
    const long long npt = (long long)nk * nkg;
    DBUF(d_kk, double, "grid_kk", nk);
    DBUF(d_kg, double, "grid_kg", nkg);
    CKS(upload(ctx, d_kk, h_kk, nk));
    CKS(upload(ctx, d_kg, h_kg, nkg));
    const bool use_sep = npt >= kSepMinPoints && nkg > 1;
    const int n = ctx->vp_on ? ctx->vp_xi_coarse : kXiCoarse;                       // gamma nodes
    const int nkc = (ctx->vp_on && ctx->vp_xi_coarse_k > 0) ? ctx->vp_xi_coarse_k : n;  // kappa nodes
    const bool xi_active = ctx->xi.on || ctx->vp_on;
    const bool use_interp = xi_active && npt > (long long)n * n && nk > 1 && nkg > 1 && h_kk[nk - 1] > 0 &&
                            h_kg[nkg - 1] > 0;
    const bool exact_xi = xi_active && !use_interp;
    if (exact_xi && write_phi) return fail(ctx, SGL_ERR_UNSUPPORTED, "exact xi term on an inversion grid");

    // the xi term first, on the side stream when the separable part follows: its kernels run
    // while the host builds the separable plan (first call for a new kg_max) and concurrently
    // with the separable kernels, which have no data dependence on them.  Profiling keeps one
    // stream so that every kernel is timed alone.
    const double* Cre = nullptr; const double* Cim = nullptr;
    const float* Cf = nullptr;
    long long nq_f = 0;
    SplineAxis sk, sg;
    int ncg = 0;
    const bool fork = use_interp && use_sep && ctx->side && !ctx->profiling && !ctx->vp_on;
    if (fork) {
        CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
        CK(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
        swap_side(ctx);
        st = ctx->stream;
    }
    const sgl_status xi_status = [&]() -> sgl_status {
    if (use_interp) {
        SplineHost& Sg = ctx->splines[n];
        SplineHost& Sk = ctx->splines[nkc];
        if (!spline_setup(Sg, n) || !spline_setup(Sk, nkc)) return fail(ctx, SGL_ERR_VALUE, "singular spline collocation");
        const std::vector<double> s = linspace(0.0, 1.0, n), s_k = linspace(0.0, 1.0, nkc);
        std::vector<double> kkc(nkc), kgc(n);
        const double kkm = h_kk[nk - 1], kgm = h_kg[nkg - 1];
        for (int i = 0; i < nkc; ++i) kkc[i] = kkm * (s_k[i] * s_k[i]);
        for (int i = 0; i < n; ++i) kgc[i] = kgm * (s[i] * s[i]);
        DBUF(d_kkc, double, "xi_kkc", nkc);
        DBUF(d_kgc, double, "xi_kgc", n);
        CKS(upload(ctx, d_kkc, kkc.data(), nkc));
        CKS(upload(ctx, d_kgc, kgc.data(), n));
        const long long nq = (long long)nkc * n;
        DBUF(d_Q, double, "xi_Qc", 2 * nq);
        CKS(xi_any(ctx, precision, d_kkc, kkc.data(), nkc, d_kgc, kgc.data(), n, d_Q, d_Q + nq));
        // C = Mk Qc Mg^T for the real and imaginary parts (FP64)
        DBUF(d_Mk, double, "spl_mk", (long long)nkc * nkc);
        DBUF(d_Mg, double, "spl_mg", (long long)n * n);
        DBUF(d_knk, double, "spl_knots_k", nkc + 4);
        DBUF(d_kng, double, "spl_knots_g", n + 4);
        CKS(upload(ctx, d_Mk, Sk.minv.data(), (size_t)nkc * nkc));
        CKS(upload(ctx, d_Mg, Sg.minv.data(), (size_t)n * n));
        CKS(upload(ctx, d_knk, Sk.knots.data(), (size_t)nkc + 4));
        CKS(upload(ctx, d_kng, Sg.knots.data(), (size_t)n + 4));
        DBUF(d_tmp, double, "spl_tmp", 2 * nq);
        DBUF(d_C, double, "spl_C", 2 * nq);
        std::vector<GemmDesc<double>> a{gd<double>(nkc, n, nkc, d_Mk, nkc, 1, d_Q, n, 1, d_tmp, n),
                                        gd<double>(nkc, n, nkc, d_Mk, nkc, 1, d_Q + nq, n, 1, d_tmp + nq, n)};
        CKS(run_gemms(ctx, a, "spl_a"));
        std::vector<GemmDesc<double>> b{gd<double>(nkc, n, n, d_tmp, n, 1, d_Mg, 1, n, d_C, n),
                                        gd<double>(nkc, n, n, d_tmp + nq, n, 1, d_Mg, 1, n, d_C + nq, n)};
        CKS(run_gemms(ctx, b, "spl_b"));
        DBUF(d_lk, int, "spl_lk", nk);
        DBUF(d_bk, double, "spl_bk", 4 * nk);
        DBUF(d_lg, int, "spl_lg", nkg);
        DBUF(d_bg, double, "spl_bg", 4 * nkg);
        launch_spline_basis(d_kk, nk, kkm, d_knk, nkc, d_lk, d_bk, st); CKLAUNCH();
        launch_spline_basis(d_kg, nkg, kgm, d_kng, n, d_lg, d_bg, st); CKLAUNCH();
        sk.l = d_lk; sk.b = d_bk; sg.l = d_lg; sg.b = d_bg;
        Cre = d_C; Cim = d_C + nq; ncg = n;
        if (precision == SGL_MIXED && write_phi) {
            // FP32 copies for the mixed finalize's FP32 spline evaluation
            DBUF(d_Cf, float, "spl_Cf", 2 * nq);
            DBUF(d_bkf, float, "spl_bkf", 4 * nk);
            DBUF(d_bgf, float, "spl_bgf", 4 * nkg);
            launch_to_float(d_C, d_Cf, 2 * nq, st); CKLAUNCH();
            launch_to_float(d_bk, d_bkf, 4LL * nk, st); CKLAUNCH();
            launch_to_float(d_bg, d_bgf, 4LL * nkg, st); CKLAUNCH();
            sk.bf = d_bkf; sg.bf = d_bgf; Cf = d_Cf; nq_f = nq;
        }
    }
    return SGL_OK;
    }();
    if (fork) {
        // join point recorded even when the xi part failed, so the main stream never waits on
        // an event from an earlier call
        cudaEventRecord(ctx->ev_join, ctx->stream);
        swap_side(ctx);
        st = ctx->stream;
    }
    CKS(xi_status);
    const void* G = nullptr;
    const double2* A1 = nullptr;
    int fin_precision = precision;
    if (use_sep) {
        CKS(build_sep(ctx, h_kg[nkg - 1], nk));
        const size_t es = elem_size(precision);
        const long long ld = 2LL * nk;
        void* Tt = ctx->arena.get("sep_T", (size_t)ctx->sep.n_cols * ld * es);
        DBUF(d_Ap, double2, "sep_Apart", (long long)ctx->sepd.nchunks * nk);
        DBUF(d_A1, double2, "sep_A1", nk);
        void* Gout = ctx->arena.get("lam_G", (size_t)ld * nkg * es);
        if (!Tt || !Gout) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (lambda)");
        {
            Timed t(ctx, precision == SGL_FP64 ? "sep_sweep_f64" : "sep_sweep_mixed", (double)nk * ctx->sep.n_cells,
                    (double)ctx->sep.n_cols * ld * es);
            launch_sep_sweep(precision, d_kk, nk, ctx->sepd, Tt, d_Ap, d_A1, st);
        }
        CKLAUNCH();
        if (precision == SGL_FP64) CKS(sep_gemms<double>(ctx, precision, h_kg, d_kg, nk, nkg, Tt, Gout));
        else CKS(sep_gemms<float>(ctx, precision, h_kg, d_kg, nk, nkg, Tt, Gout));
        G = Gout; A1 = d_A1;
    } else {
        DBUF(d_dir, double, "lam_direct", 2 * npt);
        DBUF(d_zero, double2, "lam_zero", nk);
        const double* d_k0 = (const double*)ctx->arena.find("cells_k0");
        const double* d_g0 = (const double*)ctx->arena.find("cells_g0");
        const double* d_w0 = (const double*)ctx->arena.find("cells_w0");
        DBUF(d_dpart, double2, "direct_part", (long long)std::max(1, psi1_direct_chunks((int64_t)ctx->w0.size())) * npt);
        launch_psi1_direct(d_kk, nk, d_kg, nkg, d_k0, d_g0, d_w0, (int64_t)ctx->w0.size(), d_dir, d_dir + npt, d_dpart, st);
        CKLAUNCH();
        CK(cudaMemsetAsync(d_zero, 0, (size_t)nk * sizeof(double2), st));
        G = d_dir; A1 = d_zero; fin_precision = SGL_FP64;
    }

    if (fork) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    if (write_phi && fin_precision != precision) return fail(ctx, SGL_ERR_UNSUPPORTED, "inversion grid below 2e5 points");
    {
        Timed t(ctx, "finalize", 0.0, (double)npt * 2 * (elem_size(fin_precision) + (write_phi ? elem_size(precision) : 8)));
        launch_finalize(fin_precision, write_phi, G, nk, nkg, A1, d_kk, ctx->V, Cre, Cim, ncg, sk, sg, out_re, out_im,
                        nkg, st, Cf, nq_f);
    }
    CKLAUNCH();
    if (exact_xi) {
        DBUF(d_qr, double, "xi_full", 2 * npt);
        CKS(xi_any(ctx, precision, d_kk, h_kk, nk, d_kg, h_kg, nkg, d_qr, d_qr + npt));
        launch_sum_slices<double>(d_qr, 1, nk, nkg, (double*)out_re, nkg, 1.0, st); CKLAUNCH();
        launch_sum_slices<double>(d_qr + npt, 1, nk, nkg, (double*)out_im, nkg, 1.0, st); CKLAUNCH();
    }
    return SGL_OK;
}

// Direct evaluation on a small grid into HOST planes (Lam._direct_call for < 200000 points).
// precision SGL_MIXED: the Psi_1 sums from FP32 terms (k-reach probes of the mixed path); the xi
// term stays FP64.
sgl_status lambda_direct(sgl_ctx* ctx, const double* h_kk, int nk, const double* h_kg, int nkg, double* re,
                         double* im, int precision) {
    const cudaStream_t st = ctx->stream;
    const long long npt = (long long)nk * nkg;
    DBUF(d_kk, double, "dir_kk", nk);
    DBUF(d_kg, double, "dir_kg", nkg);
    DBUF(d_out, double, "dir_out", 4 * npt);
    CKS(upload(ctx, d_kk, h_kk, nk));
    CKS(upload(ctx, d_kg, h_kg, nkg));
    const double* d_k0 = (const double*)ctx->arena.find("cells_k0");
    const double* d_g0 = (const double*)ctx->arena.find("cells_g0");
    const double* d_w0 = (const double*)ctx->arena.find("cells_w0");
    DBUF(d_dpart, double2, "direct_part", (long long)std::max(1, psi1_direct_chunks((int64_t)ctx->w0.size())) * npt);
    launch_psi1_direct(d_kk, nk, d_kg, nkg, d_k0, d_g0, d_w0, (int64_t)ctx->w0.size(), d_out, d_out + npt, d_dpart, st,
                       precision);
    CKLAUNCH();
    bool xi = false;
    if (ctx->xi.on || ctx->vp_on) {
        // the vp closure's term follows the requested precision (its mixed ln R is within ~2e-8 of
        // FP64); the gauss term's exact line kernels are FP64
        CKS(xi_any(ctx, ctx->vp_on ? precision : SGL_FP64, d_kk, h_kk, nk, d_kg, h_kg, nkg, d_out + 2 * npt,
                   d_out + 3 * npt));
        xi = true;
    }
    std::vector<double> h((size_t)(4 * npt));
    CK(cudaMemcpyAsync(h.data(), d_out, (size_t)(xi ? 4 : 2) * npt * sizeof(double), cudaMemcpyDeviceToHost, st));
    CKS(sync_stream(ctx));
    for (long long e = 0; e < npt; ++e) {
        const int n = (int)(e / nkg);
        double r = h[(size_t)e] - 0.5 * (h_kk[n] * h_kk[n] * ctx->V);
        double i = h[(size_t)(npt + e)];
        if (xi) { r += h[(size_t)(2 * npt + e)]; i += h[(size_t)(3 * npt + e)]; }
        re[e] = r; im[e] = i;
    }
    return SGL_OK;
}

double trapz(const double* y, const double* x, int n) {
    double s = 0.0;
    for (int i = 0; i + 1 < n; ++i) s += (x[i + 1] - x[i]) * (y[i + 1] + y[i]) / 2.0;
    return s;
}
}  // namespace sglh

extern "C" {

sgl_status sgl_lam_set_cells(sgl_ctx* ctx, int64_t n_cells, const double* w0, const double* k0, const double* g0,
                             const int32_t* ig, const double* fe_g, int n_fe_g, double V) {
    if (!ctx) return SGL_ERR_VALUE;
    if (n_cells < 0 || (n_cells > 0 && (!w0 || !k0 || !g0 || !ig)) || !fe_g || n_fe_g < 2)
        return fail(ctx, SGL_ERR_VALUE, "invalid cell arrays");
    if (!std::isfinite(V)) return fail(ctx, SGL_ERR_VALUE, "V must be finite");
    for (int i = 0; i + 1 < n_fe_g; ++i)
        if (!(fe_g[i + 1] > fe_g[i]) || !std::isfinite(fe_g[i + 1]))
            return fail(ctx, SGL_ERR_VALUE, "gamma bin edges must be finite and increasing");
    for (int64_t c = 0; c < n_cells; ++c) {
        if (!std::isfinite(w0[c]) || !std::isfinite(k0[c]) || !std::isfinite(g0[c]))
            return fail(ctx, SGL_ERR_VALUE, "non-finite cell value");
        if (ig[c] < 0 || ig[c] + 1 >= n_fe_g) return fail(ctx, SGL_ERR_VALUE, "gamma bin index out of range");
    }
    CK(cudaSetDevice(ctx->device));
    ctx->w0.assign(w0, w0 + n_cells);
    ctx->k0.assign(k0, k0 + n_cells);
    ctx->g0.assign(g0, g0 + n_cells);
    ctx->ig.assign(ig, ig + n_cells);
    ctx->fe_g.assign(fe_g, fe_g + n_fe_g);
    ctx->V = V;
    DBUF(dk, double, "cells_k0", n_cells);
    DBUF(dg, double, "cells_g0", n_cells);
    DBUF(dw, double, "cells_w0", n_cells);
    CKS(upload(ctx, dk, k0, (size_t)n_cells));
    CKS(upload(ctx, dg, g0, (size_t)n_cells));
    CKS(upload(ctx, dw, w0, (size_t)n_cells));
    CK(cudaStreamSynchronize(ctx->stream));
    const long long sep_version = ctx->sep.version;
    ctx->sep = SepHost();
    ctx->sep.version = sep_version + 1;            // tables built for the old plan are stale
    ctx->sep_precision_ready = -1;
    ctx->has_cells = true;
    return SGL_OK;
}

sgl_status sgl_lam_set_xi(sgl_ctx* ctx, int n_groups, const int32_t* m, const int32_t* nrow, const int32_t* nidx,
                          const int32_t* idx, const double* rows, const double* ce_k, int n_ce_k, const double* ce_g,
                          int n_ce_g, double prune, double s0_override) {
    if (!ctx) return SGL_ERR_VALUE;
    if (n_groups < 0 || n_ce_k < 2 || n_ce_g < 2 || !ce_k || !ce_g) return fail(ctx, SGL_ERR_VALUE, "invalid xi arrays");
    CK(cudaSetDevice(ctx->device));
    // Psi_2 sums the squares of the rows independently (sign_m / 2 sum_r G_r^2), so a group of
    // more than kXiGroupRows rows is the same as its consecutive row ranges taken as groups of
    // their own over the same coarse cells.  Such groups are split here into near-equal ranges;
    // their rows stay where they are (a group's rows are row-major and contiguous), only the index
    // lists are repeated.  The fused mixed kernel then covers every group.
    std::vector<int32_t> sp_m, sp_nrow, sp_nidx, sp_idx;
    {
        bool any = false;
        for (int g = 0; g < n_groups; ++g) any |= nrow[g] > kXiGroupRows;
        if (any) {
            long long io = 0;
            for (int g = 0; g < n_groups; ++g) {
                if (nidx[g] < 1 || nrow[g] < 0) return fail(ctx, SGL_ERR_VALUE, "xi group with no rows or no coarse cells");
                const int parts = std::max(1, (nrow[g] + kXiGroupRows - 1) / kXiGroupRows);
                for (int p = 0; p < parts; ++p) {
                    const int r0 = (int)((long long)nrow[g] * p / parts), r1 = (int)((long long)nrow[g] * (p + 1) / parts);
                    sp_m.push_back(m[g]); sp_nrow.push_back(r1 - r0); sp_nidx.push_back(nidx[g]);
                    sp_idx.insert(sp_idx.end(), idx + io, idx + io + nidx[g]);
                }
                io += nidx[g];
            }
            n_groups = (int)sp_m.size();
            m = sp_m.data(); nrow = sp_nrow.data(); nidx = sp_nidx.data(); idx = sp_idx.data();
        }
    }
    XiHost X;
    X.n_kmc = n_ce_k - 1; X.n_gmc = n_ce_g - 1;
    const int ngc = X.n_gmc;
    // centres: signed-log kappa (sgl_full.py:466-468), geometric gamma
    for (int i = 0; i < X.n_kmc; ++i) {
        const double a = ce_k[i], b = ce_k[i + 1];
        X.kmc.push_back(a * b > 0 ? (b > 0 ? 1.0 : -1.0) * std::sqrt(std::fabs(a * b)) : 0.0);
    }
    for (int i = 0; i < X.n_gmc; ++i) X.gmc.push_back(std::sqrt(ce_g[i] * ce_g[i + 1]));
    // prune (sgl_full.py:2823-2830): rows with norm <= prune * (largest row norm of any group)
    std::vector<long long> idx_off(n_groups + 1, 0), row_off(n_groups + 1, 0);
    for (int g = 0; g < n_groups; ++g) {
        if (nrow[g] < 0 || nidx[g] < 1) return fail(ctx, SGL_ERR_VALUE, "xi group with no rows or no coarse cells");
        idx_off[g + 1] = idx_off[g] + nidx[g];
        row_off[g + 1] = row_off[g] + (long long)nrow[g] * (nidx[g] + 1);
    }
    // The host side runs in three passes, the data-heavy ones in parallel over groups (each
    // group writes disjoint, precomputed slices; the results do not depend on the thread count):
    //   1. row norms (prune threshold)        2. per-group index structure (serial, index-only)
    //   3. transposed kept rows, sums, 1-D reach stacks, U sums
    auto parallel_groups = [&](const std::function<void(int)>& fn) { HostPool::get().run(n_groups, fn); };
    HostTimer ht(ctx);
    // coherent access: the GPU reads the caller's rows in place (norms here, the data in pass 3)
    const bool coherent = ctx->coherent_host && !std::getenv("SGL_XI_HOST_PREP");
    std::vector<std::vector<double>> norms(n_groups);
    std::vector<double> hn;
    double* d_raw = nullptr;
    if (coherent) {
        std::vector<long long> rs;
        std::vector<int> rl;
        for (int g = 0; g < n_groups; ++g)
            for (int r = 0; r < nrow[g]; ++r) { rs.push_back(row_off[g] + (long long)r * (nidx[g] + 1)); rl.push_back(nidx[g] + 1); }
        const int nr = (int)rs.size();
        DBUF(d_rs, long long, "xi_prep_rs", std::max(1, nr));
        DBUF(d_rl, int, "xi_prep_rl", std::max(1, nr));
        CKS(upload(ctx, d_rs, rs.data(), rs.size()));
        CKS(upload(ctx, d_rl, rl.data(), rl.size()));
        // one read of the caller's rows over the link into device memory; everything after
        // reads the device copy
        d_raw = dbuf<double>(ctx, "xi_raw", (size_t)std::max<long long>(1, row_off[n_groups]));
        if (!d_raw) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (xi raw rows)");
        {
            Timed t(ctx, "xi_stage_rows", 0.0, 16.0 * (double)row_off[n_groups]);
            launch_xi_stage_rows(rows, row_off[n_groups], d_raw, ctx->stream);
        }
        CKLAUNCH();
        // the norms are written straight into host memory (coherent); the host reads them after
        // the per-group index work below, which overlaps these kernels
        hn.assign((size_t)std::max(1, nr), 0.0);
        launch_xi_row_norms(d_raw, d_rs, d_rl, nr, hn.data(), ctx->stream);
        CKLAUNCH();
    } else {
        parallel_groups([&](int g) {
            const int w = nidx[g] + 1;
            norms[g].resize(nrow[g]);
            for (int r = 0; r < nrow[g]; ++r) {
                double s = 0.0;
                const double* row = rows + row_off[g] + (long long)r * w;
                for (int e = 0; e < w; ++e) s += row[e] * row[e];
                norms[g][r] = std::sqrt(s);
            }
        });
    }
    for (int g = 0; g < n_groups; ++g)
        if (m[g] < 0 || m[g] > 2) return fail(ctx, SGL_ERR_UNSUPPORTED, "xi harmonic m must be 0, 1 or 2");
    // pass 2: entry order by p, unique p / q (index-only, before the norms are known), then the
    // keep lists and every output offset
    struct GPlan {
        std::vector<int> keep, order, pg, qg, qs, qpos, qord, qseg;
        int nP = 0, q0 = 0, qseg0 = 0, p0 = 0;
        long long ent0 = 0, rowel0 = 0, row0 = 0, u0 = 0, w0 = 0, um0 = 0;
    };
    std::vector<GPlan> plan(n_groups);
    std::vector<int> g_m, g_r, g_nP, idx_p, p_ptr{0}, ent_qg, g_nQ, idx_q;
    std::vector<long long> g_p_off, g_ent_off, g_row_off, p_prefix{0}, rowel_off, g_q_off, g_u_off;
    std::vector<int> kept;                      // groups with rows left after pruning
    long long ent_total = 0, row_total = 0, rowel_total = 0, u_total = 0, w0_total = 0, um_total[3] = {0, 0, 0};
    // per-group index work in parallel (entry order by p, unique q), then the keep lists from the
    // norms, then the serial offsets and the parallel concatenation in group order
    std::atomic<int> bad_index{0};
    parallel_groups([&](int g) {
        GPlan& P = plan[g];
        const int32_t* id = idx + idx_off[g];
        for (int e = 0; e < nidx[g]; ++e)
            if (id[e] < 0 || id[e] >= X.n_kmc * ngc) { bad_index = 1; return; }
        P.pg.resize(nidx[g]); P.qg.resize(nidx[g]);
        for (int e = 0; e < nidx[g]; ++e) { P.pg[e] = id[e] / ngc; P.qg[e] = id[e] % ngc; }
        // entries by kappa cell (stable counting sort), the number of distinct kappa cells and
        // the sorted unique gamma cells
        {
            std::vector<int> cnt(X.n_kmc + 1, 0);
            for (int e = 0; e < nidx[g]; ++e) ++cnt[P.pg[e] + 1];
            for (int i = 1; i <= X.n_kmc; ++i) P.nP += cnt[i] > 0;
            for (int i = 1; i <= X.n_kmc; ++i) cnt[i] += cnt[i - 1];
            P.order.resize(nidx[g]);
            for (int e = 0; e < nidx[g]; ++e) P.order[cnt[P.pg[e]]++] = e;
        }
        P.qpos.assign(X.n_gmc, -1);
        for (int e = 0; e < nidx[g]; ++e) P.qpos[P.qg[e]] = 0;
        P.qs.clear();
        for (int q = 0; q < X.n_gmc; ++q)
            if (P.qpos[q] == 0) { P.qpos[q] = (int)P.qs.size(); P.qs.push_back(q); }
        if (coherent) {
            const int ne = nidx[g];
            P.qseg.assign(P.qs.size() + 1, 0);
            for (int e = 0; e < ne; ++e) ++P.qseg[P.qpos[P.qg[e]] + 1];
            for (size_t i = 1; i < P.qseg.size(); ++i) P.qseg[i] += P.qseg[i - 1];
            std::vector<int> fill(P.qseg.begin(), P.qseg.end() - 1);
            P.qord.resize(ne);
            for (int e = 0; e < ne; ++e) P.qord[fill[P.qpos[P.qg[e]]]++] = e;     // stable by q
        }
    });
    if (coherent) {
        CKS(sync_stream(ctx));
        for (int g = 0, k = 0; g < n_groups; ++g) norms[g].assign(hn.begin() + k, hn.begin() + k + nrow[g]), k += nrow[g];
    }
    if (bad_index) return fail(ctx, SGL_ERR_VALUE, "coarse index out of range");
    double s0 = 0.0;
    for (int g = 0; g < n_groups; ++g)
        for (double v : norms[g]) s0 = std::max(s0, v);
    if (s0_override > 0) s0 = s0_override;
    for (int g = 0; g < n_groups; ++g)
        for (int r = 0; r < nrow[g]; ++r)
            if (!(prune > 0) || norms[g][(size_t)r] > prune * s0) plan[g].keep.push_back(r);
    ht.lap("xi_index");
    // every offset, serially in group order (O(groups))
    long long q_total = 0, qseg_total = 0;
    for (int g = 0; g < n_groups; ++g) {
        GPlan& P = plan[g];
        if (P.keep.empty()) continue;
        const int R = (int)P.keep.size(), mg = m[g];
        P.q0 = (int)q_total;
        P.qseg0 = (int)qseg_total;
        P.p0 = (int)p_prefix.back();
        g_q_off.push_back(q_total);
        g_u_off.push_back(u_total);
        g_nQ.push_back((int)P.qs.size());
        q_total += (long long)P.qs.size();
        if (coherent) qseg_total += (long long)P.qs.size() + 1;
        P.ent0 = ent_total; P.rowel0 = rowel_total; P.row0 = row_total; P.u0 = u_total;
        P.w0 = w0_total; P.um0 = um_total[mg];
        if (mg == 0) { w0_total += (long long)R * X.n_kmc; X.R0 += R; }
        um_total[mg] += (long long)R * X.n_gmc;
        X.Rm[mg] += R;
        u_total += (long long)R * P.qs.size();
        g_m.push_back(mg); g_r.push_back(R); g_nP.push_back(P.nP);
        g_p_off.push_back(p_prefix.back());
        g_ent_off.push_back(ent_total);
        g_row_off.push_back(row_total);
        rowel_off.push_back(rowel_total);
        p_prefix.push_back(p_prefix.back() + P.nP);
        ent_total += nidx[g];
        row_total += R;
        rowel_total += (long long)R * nidx[g];
        X.m.push_back(mg); X.r.push_back(R); X.nP.push_back(P.nP);
        kept.push_back(g);
    }
    // the concatenated index arrays, each group filling its own slices in parallel
    const long long total_p = p_prefix.back();
    idx_p.resize((size_t)total_p);
    p_ptr.assign((size_t)total_p + 1, 0);
    p_ptr[(size_t)total_p] = (int)ent_total;
    ent_qg.resize((size_t)ent_total);
    idx_q.resize((size_t)q_total);
    std::vector<int> qord_all, pord_all, qseg_all;
    if (coherent) {
        qord_all.resize((size_t)ent_total); pord_all.resize((size_t)ent_total);
        qseg_all.resize((size_t)qseg_total);
    }
    parallel_groups([&](int g) {
        const GPlan& P = plan[g];
        if (P.keep.empty()) return;
        const int ne = nidx[g];
        for (int i = 0, j = 0; i < ne; ++i) {
            const int e = P.order[i];
            if (i == 0 || P.pg[e] != P.pg[P.order[i - 1]]) {
                p_ptr[(size_t)P.p0 + j] = (int)(P.ent0 + i);
                idx_p[(size_t)P.p0 + j] = P.pg[e];
                ++j;
            }
            ent_qg[(size_t)(P.ent0 + i)] = P.qg[e];
        }
        std::copy(P.qs.begin(), P.qs.end(), idx_q.begin() + P.q0);
        if (coherent) {
            std::copy(P.qord.begin(), P.qord.end(), qord_all.begin() + P.ent0);
            std::copy(P.order.begin(), P.order.end(), pord_all.begin() + P.ent0);
            std::copy(P.qseg.begin(), P.qseg.end(), qseg_all.begin() + P.qseg0);
        }
    });
    ht.lap("xi_plan");
    // pass 3: data, in parallel over groups (host) or on the GPU from the caller's rows (coherent)
    std::vector<double> res((size_t)row_total), sum_rows((size_t)row_total);
    const long long ubase[3] = {0, um_total[0], um_total[0] + um_total[1]};
    bool dev_filled = false;                   // rows_t, sums, U, U0, W0 already on the device
    double* d_Uall_p = nullptr;
    std::vector<double> sig_v;                 // (rows . kc + res) per m = 0 row
    std::vector<double> U0, W0, res0, sum0;
    std::vector<double> U[3], resm[3], summ[3];
    double* rows_t_p = nullptr;
    float* rows_tf_p = nullptr;
    if (coherent && !kept.empty()) {
        std::vector<XiPrepRow> kr;
        std::vector<int2> tiles;                 // transpose tiles: (group's first row in kr, i0)
        int ne_max = 0, r_max = 0;
        for (int g : kept) {
            GPlan& P = plan[g];
            const int R = (int)P.keep.size(), ne = nidx[g], w = nidx[g] + 1;
            ne_max = std::max(ne_max, ne);
            r_max = std::max(r_max, R);
            for (int i0 = 0; i0 < ne; i0 += 64) tiles.push_back(make_int2((int)kr.size(), i0));
            for (int rr = 0; rr < R; ++rr) {
                XiPrepRow k{};
                k.src = row_off[g] + (long long)P.keep[rr] * w;
                k.dst = P.rowel0 + rr;
                k.ent0 = P.ent0;
                k.u_off = ubase[m[g]] + P.um0 + (long long)rr * X.n_gmc;
                k.u0_off = P.u0 + (long long)rr * P.qs.size();
                k.w0_off = P.w0 + (long long)rr * X.n_kmc;
                k.ne = ne; k.R = R; k.row = (int)(P.row0 + rr); k.m = m[g];
                k.nQ = (int)P.qs.size(); k.q0 = P.q0; k.qseg0 = P.qseg0;
                k.nP = P.nP; k.p0 = P.p0;
                kr.push_back(k);
            }
        }
        if (((size_t)ne_max + 1) * 8 <= 200 * 1024 && r_max <= 256) {
            DBUF(d_kr, XiPrepRow, "xi_prep_rows", kr.size());
            DBUF(d_tiles, int2, "xi_prep_tiles", std::max<size_t>(1, tiles.size()));
            DBUF(d_qord, int, "xi_prep_qord", std::max<long long>(1, ent_total));
            DBUF(d_pord, int, "xi_prep_pord", std::max<long long>(1, ent_total));
            DBUF(d_qseg, int, "xi_prep_qseg", std::max<size_t>(1, qseg_all.size()));
            DBUF(d_pptr0, int, "xi_pptr", p_ptr.size());
            DBUF(d_idxp0, int, "xi_idxp", idx_p.size());
            DBUF(d_idxq0, int, "xi_idxq", idx_q.size());
            DBUF(d_kmc0, double, "xi_kmc", X.n_kmc);
            DBUF(d_rows0, double, "xi_rows", rowel_total);
            DBUF(d_rowsf0, float, "xi_rows_f", rowel_total + kXiTailPad);
            DBUF(d_res0, double, "xi_res", row_total);
            DBUF(d_sum0, double, "xi_sum", row_total);
            DBUF(d_sig0, double, "xi_prep_sig", std::max<long long>(1, row_total));
            DBUF(d_U0x, double, "xi_Usum", std::max<long long>(1, u_total));
            DBUF(d_W0x, double, "xi_W0", std::max<long long>(1, w0_total));
            DBUF(d_Uall, double, "xi_Uall", std::max<long long>(1, ubase[2] + um_total[2]));
            // the device reads these host arrays directly (no staging memcpy on the host)
            static_assert(sizeof(XiPrepRow) % 4 == 0, "word copy");
            launch_copy_from_host(kr.data(), kr.size() * sizeof(XiPrepRow), d_kr, ctx->stream);
            launch_copy_from_host(tiles.data(), tiles.size() * sizeof(int2), d_tiles, ctx->stream);
            launch_copy_from_host(qord_all.data(), qord_all.size() * 4, d_qord, ctx->stream);
            launch_copy_from_host(pord_all.data(), pord_all.size() * 4, d_pord, ctx->stream);
            launch_copy_from_host(qseg_all.data(), qseg_all.size() * 4, d_qseg, ctx->stream);
            CKLAUNCH();
            CKS(upload(ctx, d_pptr0, p_ptr.data(), p_ptr.size()));
            CKS(upload(ctx, d_idxp0, idx_p.data(), idx_p.size()));
            CKS(upload(ctx, d_idxq0, idx_q.data(), idx_q.size()));
            CKS(upload(ctx, d_kmc0, X.kmc.data(), X.kmc.size()));
            CK(cudaMemsetAsync(d_U0x, 0, (size_t)std::max<long long>(1, u_total) * 8, ctx->stream));
            CK(cudaMemsetAsync(d_W0x, 0, (size_t)std::max<long long>(1, w0_total) * 8, ctx->stream));
            CK(cudaMemsetAsync(d_Uall, 0, (size_t)std::max<long long>(1, ubase[2] + um_total[2]) * 8, ctx->stream));
            XiPrepIdx ix{d_qord, d_qseg, d_pord, d_pptr0, d_idxp0, d_idxq0};
            XiPrepOut xo{d_rows0, d_rowsf0, d_res0, d_sum0, d_sig0, d_Uall, d_U0x, d_W0x};
            {
                Timed t(ctx, "xi_transpose", 0.0, 20.0 * (double)rowel_total);
                launch_xi_transpose(d_raw, d_kr, d_tiles, (int)tiles.size(), d_pord, d_rows0, d_rowsf0, ctx->stream);
            }
            {
                Timed t(ctx, "xi_rowprep", 0.0, 8.0 * (double)rowel_total);
                launch_xi_rowprep(d_raw, d_kr, (int)kr.size(), ne_max, ix, d_kmc0, xo, ctx->stream);
            }
            CKLAUNCH();
            sig_v.assign((size_t)row_total, 0.0);
            CK(cudaMemcpyAsync(res.data(), d_res0, (size_t)row_total * 8, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(sum_rows.data(), d_sum0, (size_t)row_total * 8, cudaMemcpyDeviceToHost, ctx->stream));
            CK(cudaMemcpyAsync(sig_v.data(), d_sig0, (size_t)row_total * 8, cudaMemcpyDeviceToHost, ctx->stream));
            CKS(sync_stream(ctx));
            ht.lap("xi_data_gpu");
            dev_filled = true;
            d_Uall_p = d_Uall;
        }
    }
    if (!dev_filled) {
    // the transposed rows (FP64 and FP32 copies) are written straight into pinned memory
    CKS(sync_stream(ctx));
    char* bp = big_pinned(ctx, (size_t)rowel_total * 12 + 256);
    if (!bp) return fail(ctx, SGL_ERR_CUDA, "pinned host allocation failed (xi rows)");
    rows_t_p = (double*)bp;
    rows_tf_p = (float*)(bp + ((size_t)rowel_total * 8 + 255) / 256 * 256);
    U0.assign((size_t)u_total, 0.0);
    W0.assign((size_t)w0_total, 0.0);
    for (int k = 0; k < 3; ++k) U[k].assign((size_t)um_total[k], 0.0);
    sig_v.assign((size_t)row_total, 0.0);
    parallel_groups([&](int g) {
        const GPlan& P = plan[g];
        if (P.keep.empty()) return;
        const int R = (int)P.keep.size(), mg = m[g], w = nidx[g] + 1, ne = nidx[g];
        double* rt = rows_t_p + P.rowel0;
        float* rtf = rows_tf_p + P.rowel0;
        // rows_t[i][rr] = row_rr[order[i]], in blocks of entries so the strided writes stay in cache
        for (int i0 = 0; i0 < ne; i0 += 128) {
            const int i1 = std::min(ne, i0 + 128);
            for (int rr = 0; rr < R; ++rr) {
                const double* row = rows + row_off[g] + (long long)P.keep[rr] * w;
                for (int i = i0; i < i1; ++i) {
                    const double v = row[P.order[i]];
                    rt[(long long)i * R + rr] = v;
                    rtf[(long long)i * R + rr] = (float)v;
                }
            }
        }
        // one pass per kept row for its sums and the 1-D reach / compensation stacks (the same
        // per-output summation order as separate passes)
        for (int rr = 0; rr < R; ++rr) {
            const double* row = rows + row_off[g] + (long long)P.keep[rr] * w;
            double* urow = U[mg].data() + P.um0 + (long long)rr * X.n_gmc;
            double sm = 0.0;
            if (mg == 0) {
                double* wrow = W0.data() + P.w0 + (long long)rr * X.n_kmc;
                double* u0 = U0.data() + P.u0 + (long long)rr * P.qs.size();
                double dot = 0.0;
                for (int e = 0; e < ne; ++e) {
                    const double v = row[e];
                    const int pe = P.pg[e], qe = P.qg[e];
                    sm += v;
                    wrow[pe] += v;
                    dot += v * X.kmc[pe];
                    u0[P.qpos[qe]] += v;
                    urow[qe] += v;
                }
                sig_v[(size_t)(P.row0 + rr)] = dot + row[ne];
            } else {
                for (int e = 0; e < ne; ++e) {
                    const double v = row[e];
                    sm += v;
                    urow[P.qg[e]] += v;
                }
            }
            res[(size_t)(P.row0 + rr)] = row[ne];
            sum_rows[(size_t)(P.row0 + rr)] = sm;
        }
    });
    ht.lap("xi_data");
    }
    double sigma_var = 0.0;
    for (int g : kept) {
        const GPlan& P = plan[g];
        const int R = (int)P.keep.size();
        for (int rr = 0; rr < R; ++rr) {
            if (m[g] == 0) {
                const double v = sig_v[(size_t)(P.row0 + rr)];
                sigma_var += v * v;
                res0.push_back(res[(size_t)(P.row0 + rr)]);
                sum0.push_back(sum_rows[(size_t)(P.row0 + rr)]);
            }
            resm[m[g]].push_back(res[(size_t)(P.row0 + rr)]);
            summ[m[g]].push_back(sum_rows[(size_t)(P.row0 + rr)]);
        }
    }
    X.n_groups = (int)g_m.size();
    X.total_p = (int)p_prefix.back();
    X.total_rows = (int)row_total;
    X.sigma_var = sigma_var;
    X.on = X.n_groups > 0;
    // upload
    XiDevice D;
    D.n_groups = X.n_groups; D.n_kmc = X.n_kmc; D.n_gmc = X.n_gmc;
    DBUF(d_kmc, double, "xi_kmc", X.n_kmc);
    DBUF(d_gmc, double, "xi_gmc", X.n_gmc);
    CKS(upload(ctx, d_kmc, X.kmc.data(), X.kmc.size()));
    CKS(upload(ctx, d_gmc, X.gmc.data(), X.gmc.size()));
    D.kmc = d_kmc; D.gmc = d_gmc;
    if (X.on) {
        DBUF(d_gm, int, "xi_gm", X.n_groups);
        DBUF(d_gr, int, "xi_gr", X.n_groups);
        DBUF(d_gnP, int, "xi_gnP", X.n_groups);
        DBUF(d_goff, long long, "xi_goff", 3 * X.n_groups);
        DBUF(d_pp, long long, "xi_pprefix", 2 * X.n_groups + 1);
        DBUF(d_idxp, int, "xi_idxp", idx_p.size());
        DBUF(d_pptr, int, "xi_pptr", p_ptr.size());
        DBUF(d_qg, int, "xi_entq", ent_qg.size() + kXiTailPad);
        DBUF(d_rows, double, "xi_rows", rowel_total);
        DBUF(d_res, double, "xi_res", res.size());
        DBUF(d_sum, double, "xi_sum", sum_rows.size());
        std::vector<long long> goff;
        goff.insert(goff.end(), g_p_off.begin(), g_p_off.end());
        goff.insert(goff.end(), g_ent_off.begin(), g_ent_off.end());
        goff.insert(goff.end(), g_row_off.begin(), g_row_off.end());
        std::vector<long long> pp = p_prefix;      // n_groups + 1
        pp.insert(pp.end(), rowel_off.begin(), rowel_off.end());
        CKS(upload(ctx, d_gm, g_m.data(), g_m.size()));
        CKS(upload(ctx, d_gr, g_r.data(), g_r.size()));
        CKS(upload(ctx, d_gnP, g_nP.data(), g_nP.size()));
        CKS(upload(ctx, d_goff, goff.data(), goff.size()));
        CKS(upload(ctx, d_pp, pp.data(), pp.size()));
        CKS(upload(ctx, d_idxp, idx_p.data(), idx_p.size()));
        CKS(upload(ctx, d_pptr, p_ptr.data(), p_ptr.size()));
        if (coherent) launch_copy_from_host(ent_qg.data(), ent_qg.size() * 4, d_qg, ctx->stream);
        else CKS(upload(ctx, d_qg, ent_qg.data(), ent_qg.size()));
        CKLAUNCH();
        if (!dev_filled) {
            if (rowel_total > 0)
                CK(cudaMemcpyAsync(d_rows, rows_t_p, (size_t)rowel_total * 8, cudaMemcpyHostToDevice, ctx->stream));
            CKS(upload(ctx, d_res, res.data(), res.size()));
            CKS(upload(ctx, d_sum, sum_rows.data(), sum_rows.size()));
        }
        D.g_m = d_gm; D.g_r = d_gr; D.g_nP = d_gnP;
        D.g_p_off = d_goff; D.g_ent_off = d_goff + X.n_groups; D.g_row_off = d_goff + 2 * X.n_groups;
        D.idx_p = d_idxp; D.p_ptr = d_pptr; D.ent_qg = d_qg; D.rows = d_rows; D.res = d_res; D.sum_rows = d_sum;
        {
            DBUF(d_rowsf, float, "xi_rows_f", rowel_total + kXiTailPad);
            if (rowel_total > 0 && !dev_filled)
                CK(cudaMemcpyAsync(d_rowsf, rows_tf_p, (size_t)rowel_total * 4, cudaMemcpyHostToDevice, ctx->stream));
            DBUF(d_gnQ, int, "xi_gnQ", g_nQ.size());
            DBUF(d_qoff, long long, "xi_qoff", g_q_off.size());
            DBUF(d_uoff, long long, "xi_uoff", g_u_off.size());
            DBUF(d_idxq, int, "xi_idxq", idx_q.size());
            DBUF(d_U0, double, "xi_Usum", std::max<long long>(1, u_total));
            CKS(upload(ctx, d_gnQ, g_nQ.data(), g_nQ.size()));
            CKS(upload(ctx, d_qoff, g_q_off.data(), g_q_off.size()));
            CKS(upload(ctx, d_uoff, g_u_off.data(), g_u_off.size()));
            CKS(upload(ctx, d_idxq, idx_q.data(), idx_q.size()));
            if (!dev_filled) CKS(upload(ctx, d_U0, U0.data(), U0.size()));
            CK(cudaStreamSynchronize(ctx->stream));   // host vectors are local
            ht.lap("xi_upload");
            D.rows_f = d_rowsf; D.g_nQ = d_gnQ; D.g_q_off = d_qoff; D.g_u_off = d_uoff; D.idx_q = d_idxq; D.U0 = d_U0;
            D.r_max = *std::max_element(g_r.begin(), g_r.end());
        }
        D.R0 = X.R0;
        if (X.R0 > 0) {
            DBUF(d_W0, double, "xi_W0", std::max<long long>(1, w0_total));
            DBUF(d_r0, double, "xi_res0", res0.size());
            DBUF(d_s0, double, "xi_sum0", sum0.size());
            if (!dev_filled) CKS(upload(ctx, d_W0, W0.data(), W0.size()));
            CKS(upload(ctx, d_r0, res0.data(), res0.size()));
            CKS(upload(ctx, d_s0, sum0.data(), sum0.size()));
            D.W0 = d_W0; D.res0 = d_r0; D.sum0 = d_s0;
        }
        for (int mm = 0; mm < 3; ++mm) {
            D.Rm[mm] = X.Rm[mm];
            if (X.Rm[mm] == 0) continue;
            const std::string sfx = std::to_string(mm);
            double* d_U = d_Uall_p ? d_Uall_p + ubase[mm] : dbuf<double>(ctx, "xi_U" + sfx, U[mm].size());
            if (!d_U) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (xi U)");
            DBUF(d_rm, double, "xi_resm" + sfx, resm[mm].size());
            DBUF(d_sm, double, "xi_summ" + sfx, summ[mm].size());
            if (!dev_filled) CKS(upload(ctx, d_U, U[mm].data(), U[mm].size()));
            CKS(upload(ctx, d_rm, resm[mm].data(), resm[mm].size()));
            CKS(upload(ctx, d_sm, summ[mm].data(), summ[mm].size()));
            D.U[mm] = d_U; D.resm[mm] = d_rm; D.summ[mm] = d_sm;
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->xi = X;
    ctx->xid = D;
    return SGL_OK;
}

sgl_status sgl_lam_sigma(sgl_ctx* ctx, double* sigma) {
    if (!ctx || !sigma) return SGL_ERR_VALUE;
    if (!ctx->has_cells) return fail(ctx, SGL_ERR_STATE, "cells not set");
    // sum w0 k0^2 in the reference's rounding (np.sum(w0 * k0**2)): the grid sizes are ceilings of
    // ratios of sigma that can sit within an ulp of an integer, so the same sigma bits matter
    std::vector<double> t(ctx->w0.size());
    for (size_t c = 0; c < t.size(); ++c) t[c] = ctx->w0[c] * (ctx->k0[c] * ctx->k0[c]);
    double v = pairwise_sum(t.data(), (long long)t.size());
    v += ctx->V;
    if (ctx->xi.on) v += ctx->xi.sigma_var;
    *sigma = std::sqrt(v);
    return SGL_OK;
}

sgl_status sgl_lnphi(sgl_ctx* ctx, const double* kk, int nkk, const double* kg, int nkg, int precision,
                     double* out_re, double* out_im) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->has_cells) return fail(ctx, SGL_ERR_STATE, "cells not set");
    if (nkk < 1 || nkg < 1 || !kk || !kg || !out_re || !out_im) return fail(ctx, SGL_ERR_VALUE, "empty grid");
    if (precision != SGL_FP64 && precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    for (int i = 0; i < nkk; ++i) if (!std::isfinite(kk[i])) return fail(ctx, SGL_ERR_VALUE, "non-finite kk");
    for (int i = 0; i < nkg; ++i) if (!std::isfinite(kg[i]) || kg[i] < 0) return fail(ctx, SGL_ERR_VALUE, "kg must be finite, >= 0");
    CK(cudaSetDevice(ctx->device));
    const long long npt = (long long)nkk * nkg;
    DBUF(d_re, double, "lnphi_re", npt);
    DBUF(d_im, double, "lnphi_im", npt);
    CKS(lambda_eval(ctx, precision, kk, nkk, kg, nkg, 0, d_re, d_im));
    CK(cudaMemcpyAsync(out_re, d_re, npt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(out_im, d_im, npt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CKS(sync_stream(ctx));
    CKS(check_dev_err(ctx));
    for (long long e = 0; e < npt; ++e)
        if (!std::isfinite(out_re[e]) || !std::isfinite(out_im[e])) return fail(ctx, SGL_ERR_NONFINITE, "non-finite ln Phi");
    return SGL_OK;
}

sgl_status sgl_xi_term(sgl_ctx* ctx, const double* kk, int nkk, const double* kg, int nkg, int precision,
                       double* out_re, double* out_im) {
    if (!ctx) return SGL_ERR_VALUE;
    if (!ctx->xi.on && !ctx->vp_on) return fail(ctx, SGL_ERR_STATE, "xi groups not set");
    if (nkk < 1 || nkg < 1 || !kk || !kg || !out_re || !out_im) return fail(ctx, SGL_ERR_VALUE, "empty grid");
    if (precision != SGL_FP64 && precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    for (int i = 0; i < nkk; ++i) if (!std::isfinite(kk[i])) return fail(ctx, SGL_ERR_VALUE, "non-finite kk");
    for (int i = 0; i < nkg; ++i) if (!std::isfinite(kg[i]) || kg[i] < 0) return fail(ctx, SGL_ERR_VALUE, "kg must be finite, >= 0");
    CK(cudaSetDevice(ctx->device));
    const long long npt = (long long)nkk * nkg;
    DBUF(d_kk, double, "xt_kk", nkk);
    DBUF(d_kg, double, "xt_kg", nkg);
    DBUF(d_o, double, "xt_out", 2 * npt);
    CKS(upload(ctx, d_kk, kk, nkk));
    CKS(upload(ctx, d_kg, kg, nkg));
    CKS(xi_any(ctx, precision, d_kk, kk, nkk, d_kg, kg, nkg, d_o, d_o + npt));
    CK(cudaMemcpyAsync(out_re, d_o, npt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(out_im, d_o + npt, npt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CKS(sync_stream(ctx));
    CKS(check_dev_err(ctx));
    return SGL_OK;
}

}  // extern "C"
