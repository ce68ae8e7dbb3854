// Host runtime and C ABI: context, device arena, per-population plans, and the per-PDF pipeline
// (grid plan -> reach probes -> ln Phi -> exp -> transforms -> path integral -> moments).
// Mirrors the control flow of the reference's Lam (sgl_full.py:2711-3452) and invert
// (sgl_full.py:159-375) for the default gauss chain.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <unistd.h>

#include "kernels.cuh"

using namespace sgl;

namespace {

// ------------------------------------------------------------------ constants (reference)
constexpr double kSepTheta = 0.5;          // sgl_full.py:3036
constexpr int kSepMg = 8;
constexpr int kSepSmax = 64;
constexpr long long kSepMinPoints = 200000;  // sgl_full.py:3038
constexpr int kXiCoarse = 101;             // Lam(xi_coarse=101)
constexpr int kXiGroupRows = 48;           // longest xi group the fused mixed Psi_2 kernel takes
// sgl.py:1176-1193 and sgl_full.py:33-60
constexpr double kSigReach = 12.0, kPppK = 18.0, kPppG = 96.0, kBoxReach = 6.0;
constexpr double kPtsPerSigKap = 72.0, kPtsPerSigGam = 36.0;
constexpr double kTailKapMax = 0.99, kTailGamMax = 0.8, kTailPppG = 12.0;
constexpr double kOutGridMax = 3.4e7;

thread_local std::string g_create_error;

struct Arena {                         // grow-only named device buffers
    std::unordered_map<std::string, std::pair<void*, size_t>> bufs;
    void* get(const std::string& name, size_t bytes) {
        auto it = bufs.find(name);
        if (bytes == 0) bytes = 16;
        if (it != bufs.end() && it->second.second >= bytes) return it->second.first;
        if (it != bufs.end()) { cudaFree(it->second.first); bufs.erase(it); }
        void* p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        bufs[name] = {p, bytes};
        return p;
    }
    void* find(const std::string& name) const {
        auto it = bufs.find(name);
        return it == bufs.end() ? nullptr : it->second.first;
    }
    void release() { for (auto& kv : bufs) cudaFree(kv.second.first); bufs.clear(); }
};

struct SepHost {
    double key = -1.0;
    int n_cells = 0, n_groups = 0, n_cols = 0, n_cols_sep = 0, n_direct = 0;
    std::vector<int> chunk_begin;
    double max_sep_node = 0.0;
};

struct XiHost {
    bool on = false;
    int n_groups = 0, n_kmc = 0, n_gmc = 0, total_p = 0, total_rows = 0;
    std::vector<int> m, r, nP;
    std::vector<long long> p_prefix_rowel;   // p_prefix (n_groups+1) then rowel_off (n_groups)
    std::vector<double> kmc, gmc;
    // sigma contribution: sum over m=0 rows of (rows . kc + res)^2
    double sigma_var = 0.0;
    int R0 = 0, Rm[3] = {0, 0, 0};
};

struct SplineHost {
    int n = 0;
    std::vector<double> knots, minv;
};

struct StatRow { long long launches = 0; double ms = 0, flops = 0, bytes = 0; };
struct Pending { std::string tag; cudaEvent_t a, b; double flops, bytes; };

}  // namespace

// host scratch of the separable plan, reused between plans (sizes follow the cell count)
struct SepScratch {
    std::vector<long long> keyv, order;
    std::vector<double> sl, sh, kap, w, wl;
    std::vector<char> direct;
    std::vector<float> kh, kl, wf, wlf;
    std::vector<int> grp;
};

struct sgl_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    Arena arena;
    // population (host copies)
    std::vector<double> w0, k0, g0, fe_g;
    std::vector<int> ig;
    double V = 0.0;
    bool has_cells = false;
    SepHost sep;
    SepDevice sepd;
    SepScratch sep_scratch;
    int sep_precision_ready = -1;
    XiHost xi;
    XiDevice xid;
    long long sweep_n = -1;          // cells of the 1-D sweep (sgl_sweep_set_cells)
    std::unordered_map<int, SplineHost> splines;   // not-a-knot collocation inverses by node count
    // positive (vp) Cox closure replacing the gauss xi term (sgl_vp_set)
    bool vp_on = false;
    VpDevice vpd;
    double vp_shear = 0.0;
    int vp_xi_coarse = 101, vp_xi_coarse_k = 0;   // coarse grid (gamma, kappa); grown by sgl_pdf's rule
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    int* dev_err = nullptr;          // raised by kernels whose bounded waits ran out
    bool coherent_host = false;      // the GPU reads pageable host memory through the host page tables
    // pinned staging ring for small uploads (pageable copies would serialise host and device);
    // reset whenever the stream has been synchronised
    char* pinned = nullptr;
    size_t pinned_cap = 0, pinned_off = 0;
    // second stream for the xi term, which runs concurrently with the separable part of ln Phi
    // (fork / join by events); it has its own pinned staging ring.  swap_side() exchanges the two
    // so that every helper keeps using ctx->stream / ctx->pinned.
    cudaStream_t side = nullptr;
    char* side_pinned = nullptr;
    size_t side_pinned_cap = 0, side_pinned_off = 0;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // pinned host buffer for the large per-population arrays built on the host (grow-only)
    char* big_pinned = nullptr;
    size_t big_cap = 0;
    // per-kernel statistics (sgl_ctx_profile)
    bool profiling = false;
    long long launches_at_enable = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<Pending> pending;
    std::unordered_map<std::string, StatRow> stats;
};

namespace {

// ------------------------------------------------------------------ error helpers
sgl_status fail(sgl_ctx* c, sgl_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(ctx, SGL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define CKLAUNCH()                                                                            \
    do {                                                                                      \
        cudaError_t e_ = cudaGetLastError();                                                  \
        if (e_ != cudaSuccess)                                                                \
            return fail(ctx, SGL_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_));   \
    } while (0)

#define CKS(expr)                                                                             \
    do {                                                                                      \
        sgl_status s_ = (expr);                                                               \
        if (s_ != SGL_OK) return s_;                                                          \
    } while (0)

template <typename T>
T* dbuf(sgl_ctx* ctx, const std::string& name, size_t count) {
    return (T*)ctx->arena.get(name, count * sizeof(T));
}

#define DBUF(var, T, name, count)                                                             \
    T* var = dbuf<T>(ctx, name, (size_t)(count));                                             \
    if (!var) return fail(ctx, SGL_ERR_CUDA, std::string("device allocation failed: ") + name)

sgl_status sync_stream(sgl_ctx* ctx) {
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->pinned_off = 0;
    // the other stream's staging ring is reused only once that stream is idle too
    if (ctx->side && cudaStreamQuery(ctx->side) == cudaSuccess) ctx->side_pinned_off = 0;
    cudaGetLastError();        // a not-ready query is not an error
    return SGL_OK;
}

template <typename T>
sgl_status upload(sgl_ctx* ctx, T* dst, const T* src, size_t n) {
    if (n == 0) return SGL_OK;
    const size_t bytes = n * sizeof(T);
    if (ctx->pinned && ctx->pinned_off + bytes <= ctx->pinned_cap) {
        char* stage = ctx->pinned + ctx->pinned_off;
        std::memcpy(stage, src, bytes);
        ctx->pinned_off += (bytes + 255) & ~(size_t)255;
        CK(cudaMemcpyAsync(dst, stage, bytes, cudaMemcpyHostToDevice, ctx->stream));
        return SGL_OK;
    }
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return SGL_OK;
}

// host-side phase timing, recorded in the context's statistics as "host_<tag>" while profiling
struct HostTimer {
    sgl_ctx* c; std::chrono::steady_clock::time_point t0;
    explicit HostTimer(sgl_ctx* c_) : c(c_), t0(std::chrono::steady_clock::now()) {}
    void lap(const char* tag) {
        const auto t1 = std::chrono::steady_clock::now();
        if (c->profiling) {
            StatRow& r = c->stats[std::string("host_") + tag];
            r.launches += 1;
            r.ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        }
        t0 = t1;
    }
};

// exchanges the context's stream (and its pinned staging ring) with the side stream
void swap_side(sgl_ctx* c) {
    std::swap(c->stream, c->side);
    std::swap(c->pinned, c->side_pinned);
    std::swap(c->pinned_cap, c->side_pinned_cap);
    std::swap(c->pinned_off, c->side_pinned_off);
}

// Persistent host worker pool for the population preparation: spawning threads costs ~0.3 ms per
// batch of 16 on the Grace host, more than most of the parallel passes themselves.  run() hands
// out task indices [0, ntasks) through an atomic counter; the calling thread works too.  One job
// at a time: a caller that finds the pool busy (another context on another host thread), or a
// process forked after the pool started, runs its tasks inline.  Every task writes disjoint
// outputs, so results never depend on the scheduling.
class HostPool {
  public:
    static HostPool& get() {
        static HostPool pool;
        return pool;
    }
    void run(int ntasks, const std::function<void(int)>& fn) {
        std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
        if (!busy.owns_lock() || workers_.empty() || getpid() != pid_ || ntasks <= 1) {
            for (int t = 0; t < ntasks; ++t) fn(t);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = &fn;
            ntasks_ = ntasks;
            next_ = 0;
            pending_ = (int)workers_.size();
            ++gen_;
        }
        cv_.notify_all();
        for (int t; (t = next_.fetch_add(1)) < ntasks;) fn(t);
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [&] { return pending_ == 0; });
        job_ = nullptr;
    }
    int size() const { return (int)workers_.size() + 1; }

  private:
    HostPool() : pid_(getpid()) {
        const int n = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), 16)) - 1;
        for (int i = 0; i < n; ++i) workers_.emplace_back([this] { loop(); });
    }
    ~HostPool() {
        if (getpid() != pid_) {                  // forked child: the workers are the parent's
            for (auto& w : workers_) w.detach();
            return;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& w : workers_) if (w.joinable()) w.join();
    }
    void loop() {
        long long seen = 0;
        for (;;) {
            const std::function<void(int)>* job;
            int nt;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
                job = job_;
                nt = ntasks_;
            }
            for (int t; (t = next_.fetch_add(1)) < nt;) (*job)(t);
            std::lock_guard<std::mutex> lk(mu_);
            if (--pending_ == 0) done_cv_.notify_one();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(int)>* job_ = nullptr;
    int ntasks_ = 0, pending_ = 0;
    std::atomic<int> next_{0};
    long long gen_ = 0;
    bool stop_ = false;
    pid_t pid_;
};

// fn(lo, hi) over [0, n) in contiguous blocks on the pool (every index written by one block)
void parallel_for(long long n, const std::function<void(long long, long long)>& fn) {
    const int nblk = (int)std::max(1LL, std::min<long long>(4LL * HostPool::get().size(), (n + 2047) / 2048));
    if (nblk == 1) { fn(0, n); return; }
    const long long blk = (n + nblk - 1) / nblk;
    HostPool::get().run(nblk, [&](int b) {
        const long long lo = (long long)b * blk, hi = std::min(n, lo + blk);
        if (lo < hi) fn(lo, hi);
    });
}

// pinned host buffer of at least `bytes` (grow-only; the stream is synchronised before it grows)
char* big_pinned(sgl_ctx* ctx, size_t bytes) {
    if (bytes <= ctx->big_cap) return ctx->big_pinned;
    cudaStreamSynchronize(ctx->stream);
    if (ctx->big_pinned) cudaFreeHost(ctx->big_pinned);
    ctx->big_pinned = nullptr; ctx->big_cap = 0;
    const size_t cap = std::max(bytes, (size_t)64 << 20);
    if (cudaHostAlloc((void**)&ctx->big_pinned, cap, cudaHostAllocDefault) != cudaSuccess) {
        ctx->big_pinned = nullptr;
        return nullptr;
    }
    ctx->big_cap = cap;
    return ctx->big_pinned;
}

// numpy.linspace: a + i * step (separately rounded), last point = b exactly
std::vector<double> linspace(double a, double b, long long n) {
    std::vector<double> v((size_t)n);
    if (n == 1) { v[0] = a; return v; }
    const double step = (b - a) / (double)(n - 1);
    for (long long i = 0; i < n; ++i) { volatile double t = (double)i * step; v[(size_t)i] = t + a; }
    v[(size_t)n - 1] = b;
    return v;
}

size_t elem_size(int precision) { return precision == SGL_FP64 ? sizeof(double) : sizeof(float); }

// Scoped device timer of one tagged launch (only when profiling is on).
struct Timed {
    sgl_ctx* c; std::string tag; double flops, bytes; cudaEvent_t a = nullptr, b = nullptr;
    Timed(sgl_ctx* c_, std::string t, double f, double by) : c(c_), tag(std::move(t)), flops(f), bytes(by) {
        if (!c->profiling) return;
        a = take(); b = take();
        cudaEventRecord(a, c->stream);
    }
    cudaEvent_t take() {
        if (c->ev_pool.empty()) { cudaEvent_t e; cudaEventCreate(&e); return e; }
        cudaEvent_t e = c->ev_pool.back(); c->ev_pool.pop_back(); return e;
    }
    ~Timed() {
        if (!c->profiling) return;
        cudaEventRecord(b, c->stream);
        c->pending.push_back(Pending{tag, a, b, flops, bytes});
    }
};

void resolve_stats(sgl_ctx* c) {
    if (c->pending.empty()) return;
    cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    for (auto& p : c->pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        StatRow& r = c->stats[p.tag];
        r.launches += 1; r.ms += ms; r.flops += p.flops; r.bytes += p.bytes;
        c->ev_pool.push_back(p.a); c->ev_pool.push_back(p.b);
    }
    c->pending.clear();
}

// ------------------------------------------------------------------ GEMM dispatch
template <typename T>
sgl_status run_gemms(sgl_ctx* ctx, std::vector<GemmDesc<T>>& d, const std::string& tag) {
    if (d.empty()) return SGL_OK;
    int tiles = gemm_plan(d.data(), (int)d.size());
    // FP64 problems too small for one wave of 64 x 64 tiles run on 16 x 16 tiles
    const bool small = sizeof(T) == 8 && tiles < kNumSMs;
    if (small) tiles = gemm_plan(d.data(), (int)d.size(), 16, 16);
    DBUF(dd, GemmDesc<T>, "gemm_desc_" + tag, d.size());
    CKS(upload(ctx, dd, d.data(), d.size()));
    double fl = 0.0;
    for (auto& g : d) fl += 2.0 * g.M * (double)g.N * g.K;
    {
        Timed t(ctx, std::string(sizeof(T) == 8 ? "gemm_f64_" : "gemm_f32_") + tag, fl, 0.0);
        int layout = (d[0].a_cs == 1 ? 1 : 0) | (d[0].b_cs == 1 ? 2 : 0);
        for (auto& g : d)
            if (((g.a_cs == 1 ? 1 : 0) | (g.b_cs == 1 ? 2 : 0)) != layout) layout = -1;
        if (small) layout = kSmallTiles;
        launch_grouped_gemm<T>(dd, (int)d.size(), tiles, layout, ctx->stream);
    }
    CKLAUNCH();
    return SGL_OK;
}

// device error flag of this context (zeroed on first use)
int* dev_err_flag(sgl_ctx* ctx) {
    if (!ctx->dev_err) {
        ctx->dev_err = (int*)ctx->arena.get("dev_err", sizeof(int));
        if (ctx->dev_err) cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream);
    }
    return ctx->dev_err;
}

// reads (and clears) the flag; call after the stream has work queued that may raise it
sgl_status check_dev_err(sgl_ctx* ctx) {
    if (!ctx->dev_err) return SGL_OK;
    int h = 0;
    CK(cudaMemcpyAsync(&h, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CKS(sync_stream(ctx));
    if (h) {
        CK(cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream));
        return fail(ctx, SGL_ERR_CUDA, "tensor-core GEMM: a bounded mbarrier wait ran out");
    }
    return SGL_OK;
}

// parts = 2: operands to ~22 bits (3 MMAs per K-step); parts = 3: FP32 operands exactly (6 MMAs)
sgl_status run_tc_gemms(sgl_ctx* ctx, std::vector<TcGemmDesc>& d, const std::string& tag, int parts) {
    if (d.empty()) return SGL_OK;
    std::vector<TcPackDesc> pk(2 * d.size());
    int tiles = 0;
    long long quads = 0;
    const long long pfl = tc_gemm_plan(d.data(), (int)d.size(), parts, pk.data(), &tiles, &quads);
    DBUF(dd, TcGemmDesc, "tc_desc_" + tag, d.size());
    DBUF(dp, TcPackDesc, "tc_pack_" + tag, pk.size());
    DBUF(packed, float, "tc_packed", std::max<long long>(pfl, 1));
    CKS(upload(ctx, dd, d.data(), d.size()));
    CKS(upload(ctx, dp, pk.data(), pk.size()));
    int* err = dev_err_flag(ctx);
    if (!err) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (error flag)");
    double fl = 0.0;
    for (auto& g : d) fl += 2.0 * g.M * (double)g.N * g.K;
    {
        Timed t(ctx, "gemm_tc_" + tag, fl, (double)pfl * 4.0);
        launch_tc_gemm(parts, dd, (int)d.size(), tiles, dp, quads, packed, err, ctx->stream);
    }
    CKLAUNCH();
    return SGL_OK;
}

template <typename T>
GemmDesc<T> gd(int M, int N, int K, const void* A, long long ars, long long acs, const void* B, long long brs,
               long long bcs, void* C, long long ldc, double alpha = 1.0, double beta = 0.0) {
    GemmDesc<T> g{};
    g.M = M; g.N = N; g.K = K;
    g.A = (const T*)A; g.a_rs = ars; g.a_cs = acs;
    g.B = (const T*)B; g.b_rs = brs; g.b_cs = bcs;
    g.C = (T*)C; g.ldc = ldc;
    g.alpha = (T)alpha; g.beta = (T)beta;
    return g;
}

// One GEMM with split-K when it would under-fill the GPU: K slices write workspace slices,
// then a fixed-order sum (deterministic).  SIMT kernels (FP64, and FP32 where chosen below).
template <typename T>
sgl_status gemm_splitk_simt(sgl_ctx* ctx, GemmDesc<T> g, const std::string& tag, int min_split = 1) {
    GemmDesc<T> tmp = g;
    const int tiles = gemm_plan(&tmp, 1);
    int split = 1;
    if (tiles < 2 * kNumSMs) split = std::min(ceil_div(2 * kNumSMs, tiles), std::max(1, g.K / 512));
    // min_split > 1 (mixed path): at least min_split slices of at least 32 terms; FP32 slices
    // are combined in float-float
    split = std::max(split, std::min(min_split, std::max(1, g.K / 32)));
    if (split <= 1) { std::vector<GemmDesc<T>> v{g}; return run_gemms(ctx, v, tag); }
    const long long slice = (long long)g.M * g.N;
    DBUF(ws, T, "splitk_ws_" + tag, slice * split);
    std::vector<GemmDesc<T>> v;
    const int kc = ceil_div(g.K, split);
    for (int s = 0; s < split; ++s) {
        const int k0 = s * kc, k1 = std::min(g.K, k0 + kc);
        if (k1 <= k0) continue;
        GemmDesc<T> p = g;
        p.K = k1 - k0;
        p.A = g.A + (long long)k0 * g.a_cs;
        p.B = g.B + (long long)k0 * g.b_rs;
        p.C = ws + (long long)v.size() * slice;
        p.ldc = g.N;
        p.beta = T(0);
        v.push_back(p);
    }
    CKS(run_gemms(ctx, v, tag));
    launch_sum_slices<T>(ws, (int)v.size(), g.M, g.N, g.C, g.ldc, g.beta, ctx->stream);
    CKLAUNCH();
    return SGL_OK;
}

// FP32 on the tensor cores.  K split into >= min_split slices (FP32 accumulation in TMEM within a
// slice), slices combined in FP64 by the fixed-order sum.
sgl_status gemm_splitk_tc(sgl_ctx* ctx, GemmDesc<float> g, const std::string& tag, int min_split, int parts = 3) {
    int split = std::max(1, std::min(min_split, std::max(1, g.K / 32)));
    const long long slice = (long long)g.M * g.N;
    const bool direct = split == 1 && g.beta == 0.f;
    float* ws = nullptr;
    if (!direct) {
        ws = dbuf<float>(ctx, "splitk_ws_" + tag, (size_t)(slice * split));
        if (!ws) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (split-K workspace)");
    }
    std::vector<TcGemmDesc> v;
    const int kc = ceil_div(g.K, split);
    for (int s = 0; s < split; ++s) {
        const int k0 = s * kc, k1 = std::min(g.K, k0 + kc);
        if (k1 <= k0) continue;
        TcGemmDesc t{};
        t.M = g.M; t.N = g.N; t.K = k1 - k0;
        t.A = g.A + (long long)k0 * g.a_cs; t.a_rs = g.a_rs; t.a_cs = g.a_cs;
        t.B = g.B + (long long)k0 * g.b_rs; t.b_rs = g.b_rs; t.b_cs = g.b_cs;
        if (direct) { t.C = g.C; t.c_rs = g.ldc; t.c_cs = 1; }
        else { t.C = ws + (long long)v.size() * slice; t.c_rs = g.N; t.c_cs = 1; }
        t.alpha = g.alpha;
        v.push_back(t);
    }
    CKS(run_tc_gemms(ctx, v, tag, parts));
    if (!direct) {
        launch_sum_slices<float>(ws, (int)v.size(), g.M, g.N, g.C, g.ldc, g.beta, ctx->stream);
        CKLAUNCH();
    }
    return SGL_OK;
}

// Mixed-path GEMMs that run on the tensor cores with TF32-split operands: none of the separable
// Psi_1 or transform GEMMs.  The tail relative error of the mixed PDF (bar 1e-3) was measured with
// each moved to tcgen05.  On the bench workload: all on SIMT 3.6e-4; sep2 + sep3 3.5e-4; kappa
// 6.4e-4; the Hankel pair 5.0e-4; sep1 2.0e-3; more K-slices do not help (3x: 1.2e-3, 6x: 1.8e-3
// with all six moved).  On the reference's own z_s = 1 population against its stored PDF:
// sep2 + sep3 on tcgen05 1.30e-3, on SIMT 8.5e-4.  The tensor core's FP32 accumulation has a
// per-instruction bias that the Fourier sums do not cancel, where SIMT FMAs round to nearest.
// (The Hankel correction term, of relative size 2^-24, does run on BF16 tensor cores.)
bool tc_for(const std::string& /*tag*/) {
    return false;
}

template <typename T>
sgl_status gemm_splitk(sgl_ctx* ctx, GemmDesc<T> g, const std::string& tag, int min_split = 1) {
    if constexpr (sizeof(T) == 4) {
        if (tc_for(tag)) return gemm_splitk_tc(ctx, g, tag, min_split);
    }
    return gemm_splitk_simt<T>(ctx, g, tag, min_split);
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
    S.key = key; S.n_cells = (int)N; S.n_groups = n_groups; S.n_cols_sep = n_cols_sep;
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
            launch_cheb_points(Kg, Nch, d_t, st); CKLAUNCH();
            void* Bc = ctx->arena.get("cheb_B", (size_t)S.n_cols_sep * Nch * sizeof(TT));
            void* L = ctx->arena.get("cheb_L", (size_t)nkg * Nch * sizeof(TT));
            void* U = ctx->arena.get("cheb_U", (size_t)ld * Nch * sizeof(TT));
            if (!Bc || !L || !U) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (cheb)");
            launch_j0m1_table(precision, d_nodes, S.n_cols_sep, d_t, Nch, Bc, st); CKLAUNCH();
            launch_cheb_matrix(precision, Kg, Nch, d_t, d_kg, nkg, L, st); CKLAUNCH();
            CKS(gemm_splitk<TT>(ctx, gd<TT>((int)ld, Nch, S.n_cols_sep, Tt, 1, ld, Bc, Nch, 1, U, Nch), "sep1", msplit));
            CKS(gemm_splitk<TT>(ctx, gd<TT>((int)ld, nkg, Nch, U, Nch, 1, L, 1, Nch, Gout, nkg), "sep2", msplit));
        } else {
            void* Bn = ctx->arena.get("sep_Bn", (size_t)S.n_cols_sep * nkg * sizeof(TT));
            if (!Bn) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (Bn)");
            launch_j0m1_table(precision, d_nodes, S.n_cols_sep, d_kg, nkg, Bn, st); CKLAUNCH();
            CKS(gemm_splitk<TT>(ctx, gd<TT>((int)ld, nkg, S.n_cols_sep, Tt, 1, ld, Bn, nkg, 1, Gout, nkg), "sep1", msplit));
        }
    } else {
        CK(cudaMemsetAsync(Gout, 0, (size_t)ld * nkg * sizeof(TT), st));
    }
    if (S.n_direct > 0) {
        void* Bd = ctx->arena.get("sep_Bd", (size_t)S.n_direct * nkg * sizeof(TT));
        if (!Bd) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (Bd)");
        launch_j0m1_table(precision, d_nodes + S.n_cols_sep, S.n_direct, d_kg, nkg, Bd, st); CKLAUNCH();
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
                         double* im, int precision = SGL_FP64) {
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

}  // namespace

// Message of the last failed call that has no context (sgl_ctx_create, sgl_cf_kappa_noalloc).
std::string& sgl_noctx_error() { return g_create_error; }

// ================================================================== C ABI
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
    ctx->sep = SepHost();
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
    double v = 0.0;
    for (size_t c = 0; c < ctx->w0.size(); ++c) v += ctx->w0[c] * ctx->k0[c] * ctx->k0[c];
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
    if (n_xi < 0 || (n_xi > 0 && (!xi_out || !P_out))) return fail(ctx, SGL_ERR_VALUE, "invalid output grid");
    sgl_invert_opts o;
    sgl_invert_opts_default(&o);
    if (opts) o = *opts;
    if (o.precision != SGL_FP64 && o.precision != SGL_MIXED) return fail(ctx, SGL_ERR_VALUE, "unknown precision");
    if (o.n_xi_wide < 2 || o.n_k_int < 2 || !(o.phi_tol > 0) || !(o.xi_reach > 0) || o.window < 0 || o.window > 2)
        return fail(ctx, SGL_ERR_VALUE, "invalid inversion options");
    for (int i = 0; i < n_xi; ++i) if (!std::isfinite(xi_out[i])) return fail(ctx, SGL_ERR_VALUE, "non-finite xi_out");
    CK(cudaSetDevice(ctx->device));
    CKS(sync_stream(ctx));
    const cudaStream_t st = ctx->stream;
    double sigma;
    CKS(sgl_lam_sigma(ctx, &sigma));
    if (!(sigma > 0) || !std::isfinite(sigma)) return fail(ctx, SGL_ERR_VALUE, "sigma_kappa must be positive");
    // ---- vector_grid (sgl.py:1229-1258)
    const double sig_xi = 2.0 * sigma;
    const double xi_max = o.xi_reach * sig_xi, xi_min = -kBoxReach * sig_xi;
    double kap_max = 1.0 - std::exp(-0.5 * xi_max);
    const double kap_min = -kBoxReach * sigma;
    double gam_max = kBoxReach * sigma;
    const double g0 = gam_max;
    double k_k_max = kSigReach / sigma, k_g_max = kSigReach / sigma;
    long long n_kap = (long long)std::ceil((kap_max - kap_min) / (sigma / kPtsPerSigKap)) + 1;
    long long n_gam = (long long)std::ceil(gam_max / (sigma / kPtsPerSigGam)) + 1;
    // ---- invert grid logic (sgl_full.py:191-262)
    double kap_max_new = kap_max, gam_max_new = gam_max;
    if (o.tail_box) { kap_max_new = std::max(kap_max, kTailKapMax); gam_max_new = std::max(g0, kTailGamMax); }
    double dk_k = 2.0 * M_PI / (kPppK * std::max(std::fabs(kap_min), kap_max));
    double dk_g = 2.0 * M_PI / (kPppG * gam_max);
    if (o.tail_box && kTailPppG > 0) dk_g = std::min(dk_g, 2.0 * M_PI / (kTailPppG * gam_max_new));
    if (kap_max_new != kap_max || gam_max_new != gam_max) {
        kap_max = kap_max_new; gam_max = gam_max_new;
        n_kap = (long long)std::ceil((kap_max - kap_min) / (sigma / kPtsPerSigKap)) + 1;
        n_gam = (long long)std::ceil(gam_max / (sigma / kPtsPerSigGam)) + 1;
    }
    // ---- measured reach (_reach, sgl_full.py:38-47): 20 probes k0 * 1.25^j per axis
    const int nprobe = (int)std::ceil(std::log(64.0) / std::log(1.25)) + 1;
    double reach[2], phic[2];
    for (int ax = 0; ax < 2; ++ax) {
        const double k0v = ax == 0 ? k_k_max : k_g_max;
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
        phic[ax] = std::exp(re[i]);
    }
    k_k_max = reach[0]; k_g_max = reach[1];
    const long long nk_k = (long long)std::ceil(k_k_max / dk_k) + 1;
    const long long nk_g = (long long)std::ceil(k_g_max / dk_g) + 1;
    if (ctx->vp_on) {
        // the positive closure's coarse grid follows ln R as the box grows, per axis
        // (sgl_full.py:226-238); persistent, like the reference's Lam attributes
        const double kks = k_k_max * sigma, kgs = k_g_max * sigma;
        ctx->vp_xi_coarse = (int)std::min(401.0, std::max((double)ctx->vp_xi_coarse, 1.0 + std::ceil(12.65 * std::sqrt(kgs))));
        ctx->vp_xi_coarse_k = (int)std::min(4001.0, std::max({(double)ctx->vp_xi_coarse_k, (double)ctx->vp_xi_coarse,
                                                              1.0 + std::ceil(66.7 * std::sqrt(kks))}));
    }
    if ((double)n_kap * (double)n_gam > kOutGridMax)
        return fail(ctx, SGL_ERR_UNSUPPORTED, "geometric output grid (n_kap * n_gam > OUT_GRID_MAX) not implemented");
    // Above 2e7 k-points the reference accumulates Phi, the Hankel product and the kappa transform
    // over k_kappa row blocks to bound host memory (_invert_blocked, sgl_full.py:97-157; "same sums,
    // partial-sum order -> roundoff").  The whole grid fits in HBM here, so the same sums run
    // unblocked; allocation failure is reported as such.  The Phi rows are one grid dimension of
    // the composition kernel, hence the axis limit.
    if (nk_k > 65535) return fail(ctx, SGL_ERR_UNSUPPORTED, "k_kappa axis longer than 65535 points");
    if (nk_k < 2 || nk_g < 2) return fail(ctx, SGL_ERR_VALUE, "degenerate k grid");
    const std::vector<double> kk = linspace(0.0, k_k_max, nk_k);
    const std::vector<double> kg = linspace(0.0, k_g_max, nk_g);
    const std::vector<double> kap = linspace(kap_min, kap_max, n_kap);
    const std::vector<double> gam = linspace(0.0, gam_max, n_gam);
    const int nk = (int)nk_k, nkg = (int)nk_g, nkap = (int)n_kap, ngam = (int)n_gam;
    const int P = o.precision;
    const size_t es = elem_size(P);

    cudaEventRecord(ctx->ev[0], st);
    // ---- Phi = exp(ln Phi) on the full grid
    void* Phi = ctx->arena.get("phi", 2ULL * nk * nkg * es);
    if (!Phi) return fail(ctx, SGL_ERR_CUDA, "device allocation failed (phi)");
    CKS(lambda_eval(ctx, P, kk.data(), nk, kg.data(), nkg, 1, Phi, (char*)Phi + (size_t)nk * nkg * es));
    // window (sgl_full.py:254-258): 1 always, 2 ("auto") only when the reach did not converge
    const bool use_win = o.window == 1 || (o.window == 2 && std::max(phic[0], phic[1]) > o.phi_tol);
    if (use_win) {
        std::vector<double> wk(nk), wg(nkg);
        for (int i = 0; i < nk; ++i) {
            const double x = std::fabs(kk[i]) * 2.0 / k_k_max;
            const double v = x < 1 ? 2.0 / 3.0 - x * x + x * x * x / 2 : (x < 2 ? (2 - x) * (2 - x) * (2 - x) / 6 : 0.0);
            wk[i] = v / (2.0 / 3.0);
        }
        for (int j = 0; j < nkg; ++j) {
            const double r = std::min(1.0, std::max(0.0, std::fabs(kg[j]) / k_g_max));
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
    launch_hankel_matrix(P, d_kg, nkg, dkg, d_gam, ngam, ldF, M, st); CKLAUNCH();
    launch_kappa_matrix(P, d_kk, nk, dkk, d_kap, nkap, CS, st); CKLAUNCH();
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
    const std::vector<double> xw = linspace(xi_min, xi_max, nw);
    std::vector<double> xall(xw);
    xall.insert(xall.end(), xi_out, xi_out + n_xi);
    DBUF(d_x, double, "path_x", xall.size());
    DBUF(d_pi, double, "path_out", xall.size());
    CKS(upload(ctx, d_x, xall.data(), xall.size()));
    const double g_def = std::min(g0, gam_max);
    {
        Timed t(ctx, "path_integral", 0.0, (double)xall.size() * o.n_k_int * 2 * 4 * 8);
        launch_path_integral(d_P3, d_P3f, nkap, ngam, kap.front(), kap.back(), gam.back(), d_x, (int)xall.size(),
                             gam_max, g_def, o.n_k_int, d_pi, st);
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
        meta->nk_k = nk_k; meta->nk_g = nk_g; meta->n_kap = n_kap; meta->n_gam = n_gam;
        meta->k_k_max = k_k_max; meta->k_g_max = k_g_max; meta->kap_min = kap_min; meta->kap_max = kap_max;
        meta->gam_max = gam_max; meta->xi_min = xi_min; meta->xi_max = xi_max; meta->sigma = sigma;
        meta->phi_at_k_cut = phic[0]; meta->phi_at_g_cut = phic[1];
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

}  // extern "C"
