// Context entry points (create / destroy, errors, stream, statistics) and the small device
// building blocks of the surrogate MLP, the 1-D CF sweep and the FMA-rate probe.
#include "host.cuh"

thread_local std::string sglh::g_create_error;

std::string& sgl_noctx_error() { return sglh::g_create_error; }

extern "C" {

int sgl_abi_version(void) { return SGL_ABI_VERSION; }

sgl_status sgl_ctx_create(int device, sgl_ctx** out) {
    if (!out) { g_create_error = "out is NULL"; return SGL_ERR_VALUE; }
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        g_create_error = std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "count 0");
        return SGL_ERR_CUDA;
    }
    if (device < 0 || device >= n) { g_create_error = "device index out of range"; return SGL_ERR_VALUE; }
    e = cudaSetDevice(device);
    if (e != cudaSuccess) { g_create_error = cudaGetErrorString(e); return SGL_ERR_CUDA; }
    sgl_ctx* ctx = new sgl_ctx();
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        g_create_error = "stream creation failed"; delete ctx; return SGL_ERR_CUDA;
    }
    for (auto& ev : ctx->ev) cudaEventCreate(&ev);
    if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        ctx->side = nullptr;          // no second stream: the xi term runs in order on the first
        cudaGetLastError();
    }
    {
        int pa = 0, pt = 0;
        cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, device);
        cudaDeviceGetAttribute(&pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
        ctx->coherent_host = pa == 1 && pt == 1;
        cudaGetLastError();
    }
    ctx->pinned_cap = 16u << 20;
    if (cudaHostAlloc((void**)&ctx->pinned, ctx->pinned_cap, cudaHostAllocDefault) != cudaSuccess) {
        ctx->pinned = nullptr; ctx->pinned_cap = 0;
        cudaGetLastError();
    }
    if (ctx->side) {
        ctx->side_pinned_cap = 4u << 20;
        if (cudaHostAlloc((void**)&ctx->side_pinned, ctx->side_pinned_cap, cudaHostAllocDefault) != cudaSuccess) {
            ctx->side_pinned = nullptr; ctx->side_pinned_cap = 0;
            cudaGetLastError();
        }
    }
    *out = ctx;
    return SGL_OK;
}

void sgl_ctx_destroy(sgl_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    if (ctx->cfb) cfb_state_free(ctx->cfb);
    if (ctx->sur) sur_state_free(ctx->sur);
    if (ctx->cells) cells_state_free(ctx->cells);
    ctx->arena.release();
    for (auto& ev : ctx->ev) if (ev) cudaEventDestroy(ev);
    resolve_stats(ctx);
    for (auto& ev : ctx->ev_pool) cudaEventDestroy(ev);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->big_pinned) cudaFreeHost(ctx->big_pinned);
    if (ctx->side_pinned) cudaFreeHost(ctx->side_pinned);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int sgl_last_error(const sgl_ctx* ctx, char* buf, int buflen) {
    const std::string& m = ctx ? ctx->err : g_create_error;
    if (buf && buflen > 0) {
        const int n = std::min((int)m.size(), buflen - 1);
        std::memcpy(buf, m.data(), (size_t)n);
        buf[n] = 0;
    }
    return (int)m.size();
}

sgl_status sgl_ctx_stream(sgl_ctx* ctx, void** stream) {
    if (!ctx || !stream) return SGL_ERR_VALUE;
    *stream = (void*)ctx->stream;
    return SGL_OK;
}

sgl_status sgl_ctx_profile(sgl_ctx* ctx, int enable) {
    if (!ctx) return SGL_ERR_VALUE;
    resolve_stats(ctx);
    if (enable && !ctx->profiling) ctx->launches_at_enable = sgl::launch_counter();
    if (!enable && ctx->profiling) ctx->stats["_launches"].launches += sgl::launch_counter() - ctx->launches_at_enable;
    ctx->profiling = enable != 0;
    return SGL_OK;
}

int sgl_stats_json(sgl_ctx* ctx, char* buf, int buflen, int reset) {
    if (!ctx) return -1;
    resolve_stats(ctx);
    if (ctx->profiling) {
        ctx->stats["_launches"].launches += sgl::launch_counter() - ctx->launches_at_enable;
        ctx->launches_at_enable = sgl::launch_counter();
    }
    std::string js = "{";
    bool first = true;
    char tmp[512];
    for (auto& kv : ctx->stats) {
        std::snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f, \"flops\": %.6e, \"bytes\": %.6e}",
                      first ? "" : ", ", kv.first.c_str(), kv.second.launches, kv.second.ms, kv.second.flops,
                      kv.second.bytes);
        js += tmp;
        first = false;
    }
    js += "}";
    if (buf && buflen > 0) {
        const int n = std::min((int)js.size(), buflen - 1);
        std::memcpy(buf, js.data(), (size_t)n);
        buf[n] = 0;
    }
    if (reset) ctx->stats.clear();
    return (int)js.size();
}

// ------------------------------------------------------------------ surrogate MLP building blocks
sgl_status sgl_gemm_bf16(sgl_ctx* ctx, int M, int N, int K, const float* A, int64_t a_rs, int64_t a_cs, const float* B,
                         int64_t b_rs, int64_t b_cs, float* C, int64_t c_rs, int64_t c_cs, float alpha) {
    if (!ctx) return SGL_ERR_VALUE;
    if (M < 0 || N < 0 || K < 0 || (M > 0 && N > 0 && (!A || !B || !C))) return fail(ctx, SGL_ERR_VALUE, "invalid GEMM arguments");
    if (M == 0 || N == 0) return SGL_OK;
    CK(cudaSetDevice(ctx->device));
    std::vector<TcGemmDesc> v(1);
    TcGemmDesc& t = v[0];
    t = TcGemmDesc{};
    t.M = M; t.N = N; t.K = K;
    t.A = A; t.a_rs = a_rs; t.a_cs = a_cs;
    t.B = B; t.b_rs = b_rs; t.b_cs = b_cs;
    t.C = C; t.c_rs = c_rs; t.c_cs = c_cs;
    t.alpha = alpha;
    return run_tc_gemms(ctx, v, "bf16", 1);
}

sgl_status sgl_mlp_bias_act(sgl_ctx* ctx, int M, int N, const float* Z, const float* bias, float* Zb, float* A, int silu) {
    if (!ctx || M < 0 || N < 0) return SGL_ERR_VALUE;
    launch_bias_act(M, N, Z, bias, Zb, A, silu, ctx->stream);
    CKLAUNCH();
    return SGL_OK;
}

sgl_status sgl_mlp_act_grad(sgl_ctx* ctx, int M, int N, const float* dA, const float* Zb, float* dZ) {
    if (!ctx || M < 0 || N < 0) return SGL_ERR_VALUE;
    launch_act_grad(M, N, dA, Zb, dZ, ctx->stream);
    CKLAUNCH();
    return SGL_OK;
}

sgl_status sgl_mlp_col_sum(sgl_ctx* ctx, int M, int N, const float* X, float* out) {
    if (!ctx || M < 0 || N < 0) return SGL_ERR_VALUE;
    launch_col_sum(M, N, X, out, ctx->stream);
    CKLAUNCH();
    return SGL_OK;
}

sgl_status sgl_mlp_infer(sgl_ctx* ctx, int n, const float* X, int n_layers, const float* const* W, const float* const* b,
                         float* Y) {
    if (!ctx) return SGL_ERR_VALUE;
    if (n < 0 || !X || !W || !b || !Y) return fail(ctx, SGL_ERR_VALUE, "sgl_mlp_infer: invalid arguments");
    if (n_layers != 7) return fail(ctx, SGL_ERR_UNSUPPORTED, "sgl_mlp_infer: the fused kernel is 8 -> 6 x 256 SiLU -> 2");
    for (int l = 0; l < 7; ++l)
        if (!W[l] || !b[l]) return fail(ctx, SGL_ERR_VALUE, "sgl_mlp_infer: NULL weight or bias");
    if (n == 0) return SGL_OK;
    CK(cudaSetDevice(ctx->device));
    static thread_local int attr_device = -1;
    if (attr_device != ctx->device) {
        if (mlp_fused_attr() != SGL_OK) return fail(ctx, SGL_ERR_CUDA, "sgl_mlp_infer: shared-memory attribute");
        attr_device = ctx->device;
    }
    DBUF(Wp, unsigned char, "mlp_Wp", mlp_fused_wp_bytes());
    DBUF(small, float, "mlp_small", mlp_fused_small_floats());
    DBUF(ptrs, const float*, "mlp_ptrs", 11);
    const float* hp[11] = {W[1], W[2], W[3], W[4], W[5], b[0], b[1], b[2], b[3], b[4], b[5]};
    CKS(upload(ctx, ptrs, hp, 11));
    int* err = dev_err_flag(ctx);
    if (!err) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (error flag)");
    launch_mlp_fused(n, X, W, b, Wp, small, ptrs, Y, err, kNumSMs, ctx->stream);
    CKLAUNCH();
    return check_dev_err(ctx);
}

sgl_status sgl_mlp_mse(sgl_ctx* ctx, int64_t n, const float* pred, const float* target, float* dpred, double* loss) {
    if (!ctx || n < 1 || !pred || !target || !dpred || !loss) return SGL_ERR_VALUE;
    const int nb = mse_blocks(n);
    DBUF(part, double, "mse_part", nb);
    launch_mse(n, pred, target, dpred, part, ctx->stream);
    CKLAUNCH();
    std::vector<double> h((size_t)nb);
    CK(cudaMemcpyAsync(h.data(), part, nb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CKS(sync_stream(ctx));
    CKS(check_dev_err(ctx));
    double a = 0.0;
    for (double v : h) a += v;
    *loss = a / (double)n;
    return SGL_OK;
}

sgl_status sgl_mlp_adamw(sgl_ctx* ctx, int64_t n, float* w, const float* g, float* m, float* v, float lr, float b1,
                         float b2, float eps, float wd, int step) {
    if (!ctx || n < 0 || step < 1) return SGL_ERR_VALUE;
    const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
    launch_adamw(n, w, g, m, v, lr, b1, b2, eps, wd, c1, c2, ctx->stream);
    CKLAUNCH();
    return SGL_OK;
}

sgl_status sgl_sweep_set_cells(sgl_ctx* ctx, int64_t n_cells, const double* kap, const double* w) {
    if (!ctx) return SGL_ERR_VALUE;
    if (n_cells < 1 || !kap || !w) return fail(ctx, SGL_ERR_VALUE, "empty cell list");
    CK(cudaSetDevice(ctx->device));
    std::vector<float> kh((size_t)n_cells), kl((size_t)n_cells), wf((size_t)n_cells);
    for (int64_t c = 0; c < n_cells; ++c) {
        if (!std::isfinite(kap[c]) || !std::isfinite(w[c])) return fail(ctx, SGL_ERR_VALUE, "non-finite cell");
        const ff f = ff_from_double(kap[c]);
        kh[(size_t)c] = f.hi; kl[(size_t)c] = f.lo; wf[(size_t)c] = (float)w[c];
    }
    DBUF(d_k, double, "sw_kap", n_cells);
    DBUF(d_w, double, "sw_w", n_cells);
    DBUF(d_kh, float, "sw_kh", n_cells);
    DBUF(d_kl, float, "sw_kl", n_cells);
    DBUF(d_wf, float, "sw_wf", n_cells);
    CK(cudaMemcpyAsync(d_k, kap, (size_t)n_cells * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_w, w, (size_t)n_cells * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_kh, kh.data(), (size_t)n_cells * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_kl, kl.data(), (size_t)n_cells * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_wf, wf.data(), (size_t)n_cells * 4, cudaMemcpyHostToDevice, ctx->stream));
    CKS(sync_stream(ctx));
    ctx->sweep_n = n_cells;
    return SGL_OK;
}

sgl_status sgl_sweep_eval(sgl_ctx* ctx, const double* kk, int nk, int precision, double* out_re, double* out_im) {
    if (!ctx) return SGL_ERR_VALUE;
    if (ctx->sweep_n < 1) return fail(ctx, SGL_ERR_STATE, "sweep cells not set");
    if (nk < 1 || !kk || !out_re || !out_im) return fail(ctx, SGL_ERR_VALUE, "empty k grid");
    if (precision != SGL_FP64 && precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    for (int i = 0; i < nk; ++i) if (!std::isfinite(kk[i])) return fail(ctx, SGL_ERR_VALUE, "non-finite kk");
    CK(cudaSetDevice(ctx->device));
    const long long nc = ctx->sweep_n;
    const int nch = sweep1d_chunks(nk, nc);
    DBUF(d_kk, double, "sw_kk", nk);
    DBUF(d_part, double2, "sw_part", (long long)nch * nk);
    DBUF(d_out, double, "sw_out", 2LL * nk);
    CKS(upload(ctx, d_kk, kk, nk));
    {
        Timed t(ctx, precision == SGL_FP64 ? "sweep1d_f64" : "sweep1d_mixed", (double)nk * nc, (double)nk * 0 + nc * 16.0);
        launch_sweep1d(precision, d_kk, nk, (const double*)ctx->arena.find("sw_kap"), (const double*)ctx->arena.find("sw_w"),
                       (const float*)ctx->arena.find("sw_kh"), (const float*)ctx->arena.find("sw_kl"),
                       (const float*)ctx->arena.find("sw_wf"), nc, nch, d_part, d_out, d_out + nk, ctx->stream);
    }
    CKLAUNCH();
    CK(cudaMemcpyAsync(out_re, d_out, (size_t)nk * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(out_im, d_out + nk, (size_t)nk * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CKS(sync_stream(ctx));
    for (int i = 0; i < nk; ++i)
        if (!std::isfinite(out_re[i]) || !std::isfinite(out_im[i])) return fail(ctx, SGL_ERR_NONFINITE, "non-finite sweep");
    return SGL_OK;
}

sgl_status sgl_measure_peak(sgl_ctx* ctx, int fp64, double* tflops) {
    if (!ctx || !tflops) return SGL_ERR_VALUE;
    CK(cudaSetDevice(ctx->device));
    const int blocks = kNumSMs * 8, iters = fp64 ? 512 : 8192;
    DBUF(d_o, double, "peak_out", (long long)blocks * 256);
    launch_fma_probe(fp64, d_o, blocks, iters, ctx->stream);     // warm-up
    CKLAUNCH();
    cudaEvent_t a, b;
    cudaEventCreate(&a); cudaEventCreate(&b);
    cudaEventRecord(a, ctx->stream);
    for (int r = 0; r < 5; ++r) launch_fma_probe(fp64, d_o, blocks, iters, ctx->stream);
    cudaEventRecord(b, ctx->stream);
    CKS(sync_stream(ctx));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a); cudaEventDestroy(b);
    *tflops = 5.0 * (double)blocks * 256 * iters * 8 * 2 / (ms * 1e-3) / 1e12;
    return SGL_OK;
}

}  // extern "C"
