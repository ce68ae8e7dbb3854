// Host runtime shared by the engine's C ABI translation units: the context (streams, device
// arena, pinned staging, host worker pool, statistics), error helpers and the GEMM dispatch.
// The stages live in host_lam.cu (population plans, ln Phi), host_vp.cu (positive closure),
// host_invert.cu (grid plan, transforms, path integral) and host_ctx.cu (context entry points).
#pragma once
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

namespace sglh {

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

extern thread_local std::string g_create_error;   // message of the last failed call without a context

struct Arena {                         // grow-only named device buffers
    std::unordered_map<std::string, std::pair<void*, size_t>> bufs;
    std::unordered_map<std::string, long long> gen;     // per name: which allocation it is
    long long next_gen = 0;
    void* get(const std::string& name, size_t bytes) {
        auto it = bufs.find(name);
        if (bytes == 0) bytes = 16;
        if (it != bufs.end() && it->second.second >= bytes) return it->second.first;
        if (it != bufs.end()) { cudaFree(it->second.first); bufs.erase(it); }
        void* p = nullptr;
        gen[name] = ++next_gen;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        bufs[name] = {p, bytes};
        return p;
    }
    long long generation(const std::string& name) const {
        auto it = gen.find(name);
        return it == gen.end() ? 0 : it->second;
    }
    void* find(const std::string& name) const {
        auto it = bufs.find(name);
        return it == bufs.end() ? nullptr : it->second.first;
    }
    void release() { for (auto& kv : bufs) cudaFree(kv.second.first); bufs.clear(); }
};

struct SepHost {
    double key = -1.0;
    long long version = 0;                // bumped by every new plan (nodes, columns)
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

}  // namespace sglh

using namespace sglh;

// host scratch of the separable plan, reused between plans (sizes follow the cell count)
struct SepScratch {
    std::vector<long long> keyv, order;
    std::vector<double> sl, sh, kap, w, wl;
    std::vector<char> direct;
    std::vector<float> kh, kl, wf, wlf;
    std::vector<int> grp;
};

struct CfbState;                         // batched CF solver state (host_cfbatch.cu)
void cfb_state_free(CfbState* s);
int cfb_n_inst(const CfbState* s);
void cfb_inst_grid(const CfbState* s, int i, long long* k_off, int* nk, double* dk, double* k0);
struct SurState;                         // surrogate + judge assembly state (host_sur.cu)
void sur_state_free(SurState* s);
struct CellsState;                       // binned-cell deposit state (host_cells.cu)
void cells_state_free(CellsState* s);

struct sgl_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    CfbState* cfb = nullptr;
    SurState* sur = nullptr;
    CellsState* cells = nullptr;
    // batched solver launch shapes found by the autotuner, per precision and batch shape class
    std::unordered_map<long long, std::pair<int, int>> cfb_shapes;
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
    // device tables that depend only on a grid or plan (Hankel / kappa matrices, the separable basis):
    // the key they were built for, with the generation of the arena buffer that holds them
    std::unordered_map<std::string, std::vector<double>> table_keys;
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

namespace sglh {

// ------------------------------------------------------------------ error helpers
inline sgl_status fail(sgl_ctx* c, sgl_status s, const std::string& msg) {
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

// A device table named `name` built for `key` is current when neither the key nor its buffer's
// allocation changed since table_built(); the caller rebuilds it otherwise.
inline bool table_current(sgl_ctx* ctx, const std::string& name, std::vector<double> key) {
    key.push_back((double)ctx->arena.generation(name));
    auto it = ctx->table_keys.find(name);
    return it != ctx->table_keys.end() && it->second == key;
}
inline void table_built(sgl_ctx* ctx, const std::string& name, std::vector<double> key) {
    key.push_back((double)ctx->arena.generation(name));
    ctx->table_keys[name] = std::move(key);
}

inline sgl_status sync_stream(sgl_ctx* ctx) {
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->pinned_off = 0;
    // the other stream's staging ring is reused only once that stream is idle too
    if (ctx->side && cudaStreamQuery(ctx->side) == cudaSuccess) ctx->side_pinned_off = 0;
    cudaGetLastError();        // a not-ready query is not an error
    return SGL_OK;
}

template <typename T>
inline sgl_status upload(sgl_ctx* ctx, T* dst, const T* src, size_t n) {
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
inline void swap_side(sgl_ctx* c) {
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
inline void parallel_for(long long n, const std::function<void(long long, long long)>& fn) {
    const int nblk = (int)std::max(1LL, std::min<long long>(4LL * HostPool::get().size(), (n + 2047) / 2048));
    if (nblk == 1) { fn(0, n); return; }
    const long long blk = (n + nblk - 1) / nblk;
    HostPool::get().run(nblk, [&](int b) {
        const long long lo = (long long)b * blk, hi = std::min(n, lo + blk);
        if (lo < hi) fn(lo, hi);
    });
}

// pinned host buffer of at least `bytes` (grow-only; the stream is synchronised before it grows)
inline char* big_pinned(sgl_ctx* ctx, size_t bytes) {
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
inline std::vector<double> linspace(double a, double b, long long n) {
    std::vector<double> v((size_t)n);
    if (n == 1) { v[0] = a; return v; }
    const double step = (b - a) / (double)(n - 1);
    for (long long i = 0; i < n; ++i) { volatile double t = (double)i * step; v[(size_t)i] = t + a; }
    v[(size_t)n - 1] = b;
    return v;
}

inline size_t elem_size(int precision) { return precision == SGL_FP64 ? sizeof(double) : sizeof(float); }

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

inline void resolve_stats(sgl_ctx* c) {
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
inline sgl_status run_gemms(sgl_ctx* ctx, std::vector<GemmDesc<T>>& d, const std::string& tag) {
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
inline int* dev_err_flag(sgl_ctx* ctx) {
    if (!ctx->dev_err) {
        ctx->dev_err = (int*)ctx->arena.get("dev_err", sizeof(int));
        if (ctx->dev_err) cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream);
    }
    return ctx->dev_err;
}

// reads (and clears) the flag; call after the stream has work queued that may raise it
inline sgl_status check_dev_err(sgl_ctx* ctx) {
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
// drain = true: the drained-accumulation kernel (TMEM sums folded into TwoSum running sums every
// 64 products), tiles of at most tc_drain_bn() columns
inline sgl_status run_tc_gemms(sgl_ctx* ctx, std::vector<TcGemmDesc>& d, const std::string& tag, int parts,
                               bool drain = false) {
    if (d.empty()) return SGL_OK;
    std::vector<TcPackDesc> pk(2 * d.size());
    int tiles = 0;
    long long quads = 0;
    const long long pfl = tc_gemm_plan(d.data(), (int)d.size(), parts, pk.data(), &tiles, &quads, true,
                                       drain ? tc_drain_bn() : 256);     // 256: the TMEM columns of one tile
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
        if (drain) launch_tc_gemm_drain(parts, dd, (int)d.size(), tiles, dp, quads, packed, err, ctx->stream);
        else launch_tc_gemm(parts, dd, (int)d.size(), tiles, dp, quads, packed, err, ctx->stream);
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
inline sgl_status gemm_splitk_simt(sgl_ctx* ctx, GemmDesc<T> g, const std::string& tag, int min_split = 1) {
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
inline sgl_status gemm_splitk_tc(sgl_ctx* ctx, GemmDesc<float> g, const std::string& tag, int min_split, int parts = 3,
                                 bool drain = false) {
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
    CKS(run_tc_gemms(ctx, v, tag, parts, drain));
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
// Mixed-path GEMMs on the drained tcgen05 kernel (TF32 parts of FP32 operands, TMEM sums drained into
// TwoSum running sums every 64 products).  Measured against the reference's PDFs (tail relative error,
// bar 1e-3; all-SIMT: 2.1e-4 on its z_s = 1 cells with 3 groups, 6.5e-4 on the full z_s = 1
// population, 1.7e-3 on the 300-cell blocked case): sep1 on tcgen05 gives 3.7e-4 / 5.3e-4 / 1.2e-3
// and is 8% faster than on SIMT; the Hankel and kappa transforms on tcgen05 give 1.9e-3 on the z_s = 1
// cells whether the sums are drained every 64 or every 16 products, and sep2 / sep3 are slower there.
constexpr const char* kTcDrainTags[] = {"sep1"};
constexpr int kTcDrainParts = 3;                // TF32 parts of its operands (3: FP32 operands exactly)
inline bool tc_for(const std::string& tag) {
    for (const char* t : kTcDrainTags)
        if (tag == t) return true;
    return false;
}

template <typename T>
inline sgl_status gemm_splitk(sgl_ctx* ctx, GemmDesc<T> g, const std::string& tag, int min_split = 1) {
    if constexpr (sizeof(T) == 4) {
        if (tc_for(tag)) return gemm_splitk_tc(ctx, g, tag, min_split, kTcDrainParts, true);
    }
    return gemm_splitk_simt<T>(ctx, g, tag, min_split);
}

// ------------------------------------------------------------------ across translation units
// host_vp.cu
sgl_status vp_qxi(sgl_ctx* ctx, int precision, const double* d_kk, int nk, const double* d_kg, const double* h_kg,
                  int nkg, double* d_re, double* d_im);
// host_lam.cu
sgl_status lambda_eval(sgl_ctx* ctx, int precision, const double* h_kk, int nk, const double* h_kg, int nkg,
                       int write_phi, void* out_re, void* out_im);
sgl_status lambda_direct(sgl_ctx* ctx, const double* h_kk, int nk, const double* h_kg, int nkg, double* re,
                         double* im, int precision = SGL_FP64);
double trapz(const double* y, const double* x, int n);
}  // namespace sglh

// Message of the last failed call that has no context (sgl_ctx_create, sgl_cf_kappa_noalloc).
std::string& sgl_noctx_error();
