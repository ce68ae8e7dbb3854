// Batched plain solver: one handle owning several contexts (slots) on one device, each holding a
// resident population, and a native scheduler that runs many PDFs across them.
//
// A PDF is independent of every other PDF, so the slots exchange nothing.  sgl_batch_pdf gives
// every slot that has jobs its own host thread; the thread runs its slot's jobs in the order given,
// each through sgl_pdf on the slot's streams, so the device overlaps the slots' kernels and the
// host-side steps of one slot's inversion (grid plan, moments) with the kernels of the others.
// The threads are the batch's own and persist between calls: a call hands each its job list and
// waits for all of them.
#include <thread>

#include "host.cuh"

struct sgl_batch {
    int device = 0;
    std::vector<sgl_ctx*> slots;
    // persistent workers, one per slot
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv, done_cv;
    long long gen = 0;
    int pending = 0;
    bool stop = false;
    std::function<void(int)> job;
};

namespace {

void batch_worker(sgl_batch* b, int slot) {
    long long seen = 0;
    for (;;) {
        std::function<void(int)> fn;
        {
            std::unique_lock<std::mutex> lk(b->mu);
            b->cv.wait(lk, [&] { return b->gen != seen || b->stop; });
            if (b->stop) return;
            seen = b->gen;
            fn = b->job;
        }
        fn(slot);
        std::lock_guard<std::mutex> lk(b->mu);
        if (--b->pending == 0) b->done_cv.notify_all();
    }
}

}  // namespace

extern "C" {

sgl_status sgl_batch_create(int device, int slots, sgl_batch** out) {
    if (!out) return SGL_ERR_VALUE;
    *out = nullptr;
    if (slots < 1 || slots > 64) {
        sgl_noctx_error() = "sgl_batch_create: slots must be in [1, 64]";
        return SGL_ERR_VALUE;
    }
    auto* b = new sgl_batch();
    b->device = device;
    for (int s = 0; s < slots; ++s) {
        sgl_ctx* c = nullptr;
        const sgl_status st = sgl_ctx_create(device, &c);
        if (st != SGL_OK) {
            for (sgl_ctx* x : b->slots) sgl_ctx_destroy(x);
            delete b;
            return st;                       // sgl_ctx_create left its message
        }
        b->slots.push_back(c);
    }
    for (int s = 0; s < slots; ++s) b->workers.emplace_back(batch_worker, b, s);
    *out = b;
    return SGL_OK;
}

void sgl_batch_destroy(sgl_batch* b) {
    if (!b) return;
    {
        std::lock_guard<std::mutex> lk(b->mu);
        b->stop = true;
    }
    b->cv.notify_all();
    for (auto& w : b->workers) if (w.joinable()) w.join();
    for (sgl_ctx* c : b->slots) sgl_ctx_destroy(c);
    delete b;
}

int sgl_batch_slots(const sgl_batch* b) { return b ? (int)b->slots.size() : 0; }

sgl_ctx* sgl_batch_slot(sgl_batch* b, int slot) {
    if (!b || slot < 0 || slot >= (int)b->slots.size()) return nullptr;
    return b->slots[(size_t)slot];
}

sgl_status sgl_batch_pdf(sgl_batch* b, int n_jobs, const int32_t* job_slot, const double* xi_out, int n_xi,
                         const sgl_invert_opts* opts, double* P_out, sgl_invert_meta* meta, int32_t* job_status) {
    if (!b) return SGL_ERR_VALUE;
    const int ns = (int)b->slots.size();
    if (n_jobs < 0 || (n_jobs > 0 && (!job_slot || !P_out)) || n_xi < 0 || (n_xi > 0 && !xi_out)) {
        sgl_noctx_error() = "sgl_batch_pdf: invalid job or output arrays";
        return SGL_ERR_VALUE;
    }
    std::vector<std::vector<int>> per_slot((size_t)ns);
    for (int j = 0; j < n_jobs; ++j) {
        if (job_slot[j] < 0 || job_slot[j] >= ns) {
            sgl_noctx_error() = "sgl_batch_pdf: job " + std::to_string(j) + " names slot " +
                                std::to_string(job_slot[j]) + " of " + std::to_string(ns);
            return SGL_ERR_VALUE;
        }
        per_slot[(size_t)job_slot[j]].push_back(j);
    }
    std::vector<sgl_status> st((size_t)std::max(n_jobs, 1), SGL_OK);
    auto fn = [&](int s) {
        sgl_ctx* c = b->slots[(size_t)s];
        for (int j : per_slot[(size_t)s]) {
            st[(size_t)j] = sgl_pdf(c, xi_out, n_xi, opts, P_out + (size_t)j * n_xi, meta ? meta + j : nullptr);
            if (st[(size_t)j] != SGL_OK) break;      // the slot's later jobs keep SGL_ERR_STATE below
        }
    };
    {
        std::unique_lock<std::mutex> lk(b->mu);
        b->job = fn;
        b->pending = ns;
        ++b->gen;
    }
    b->cv.notify_all();
    {
        std::unique_lock<std::mutex> lk(b->mu);
        b->done_cv.wait(lk, [&] { return b->pending == 0; });
        b->job = nullptr;
    }
    sgl_status first = SGL_OK;
    int first_job = -1;
    for (int s = 0; s < ns; ++s) {
        bool failed = false;
        for (int j : per_slot[(size_t)s]) {
            if (failed) st[(size_t)j] = SGL_ERR_STATE;     // not run: an earlier job of its slot failed
            else if (st[(size_t)j] != SGL_OK) failed = true;
        }
    }
    for (int j = 0; j < n_jobs; ++j) {
        if (job_status) job_status[j] = (int32_t)st[(size_t)j];
        if (st[(size_t)j] != SGL_OK && first == SGL_OK) { first = st[(size_t)j]; first_job = j; }
    }
    if (first != SGL_OK) {
        char buf[512];
        sgl_last_error(b->slots[(size_t)job_slot[first_job]], buf, (int)sizeof(buf));
        sgl_noctx_error() = "sgl_batch_pdf: job " + std::to_string(first_job) + ": " + buf;
    }
    return first;
}

}  // extern "C"
