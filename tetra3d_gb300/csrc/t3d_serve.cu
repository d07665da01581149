// t3d_serve.cu -- render-request serving with continuous batching.
//
// Requests (scene id + camera + light subset) queue in arrival order. The
// server owns `streams` launch slots; each slot is a private frame context (its
// own stream, tables, scratch and output buffers) over the parent context's
// resident scenes, driven by its own host thread. A free slot admits queued
// requests in FIFO order while the batch has room (max_batch) and the device
// bytes of everything in flight stay within the HBM budget, builds the batch's
// launch tables, launches all admitted jobs in one persistent-kernel launch,
// waits for it and posts the completions. Slots run concurrently -- their table
// builds overlap each other and the GPU work of the other slots -- so requests
// arriving while others are on the GPU are admitted as soon as a slot and
// memory free up. Each request's output is written only by its own job's
// segments, so its result does not depend on what it was batched with. A slot's
// buffers grow in stream order from the server's memory pool, so a batch larger
// than any before does not stall the other slots.
// Scenes must not be uploaded or released while a server runs.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <iterator>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "t3d_runtime.h"

using namespace t3d;
using Clock = std::chrono::steady_clock;

namespace {

struct Pending {
    t3d_request req;
    double arrival_abs;  // seconds since server start
    double admit_abs = 0;
    uint64_t bytes = 0;
    uint32_t pairs = 0;  // render pairs of its scene (model parts), the size of its host table build
};

struct Slot {
    t3d_ctx* ctx = nullptr;
    cudaEvent_t ev = nullptr;
    std::thread worker;
    std::vector<Pending> batch;
    uint64_t bytes = 0;
    uint64_t pairs = 0;
    double launch_abs = 0;  // the batch's tables built and its kernels queued
};

// FNV-1a over the raw bytes of a request's emitted stream, in emit order.
uint64_t fnv(const void* p, size_t n, uint64_t h) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

}  // namespace

struct t3d_server {
    t3d_ctx* owner = nullptr;
    cudaMemPool_t pool = nullptr;  // the slots' scratch and outputs grow in this pool, in stream order
    uint64_t budget = 0;
    uint32_t max_batch = 1;
    uint32_t max_pairs = 4096;  // render pairs per batch (0: no bound)
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Pending> queue;
    std::vector<t3d_completion> done;
    std::atomic<bool> stop{false};
    uint64_t inflight = 0;
    // the slot that completed a batch last, and the slots with a batch in flight. While none is
    // in flight only the last one watches the clock for the next replayed arrival, so at low load
    // the slot whose host caches are warm takes the next request; otherwise every idle slot does.
    const Slot* last_done = nullptr;
    uint32_t nbusy = 0;
    Clock::time_point t0;
    bool verify = true;
    std::string err;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    uint64_t request_bytes(const t3d_request& r) {
        auto it = owner->scenes.find(r.job.scene);
        if (it == owner->scenes.end()) return 0;
        const Scene* sc = it->second.get();
        // outputs (108 B per slot), per-vertex scratch (48 B), visible lists and tables
        return 116ull * sc->ntris + 48ull * sc->nverts + 1024ull * (sc->models.size() + 4);
    }

    // render pairs of a request's scene (counted once per scene: scenes do not change while
    // the server runs); called without the lock held
    std::mutex pairs_mu;
    std::map<uint32_t, uint32_t> scene_pairs;
    uint32_t request_pairs(const t3d_request& r) {
        std::lock_guard<std::mutex> g(pairs_mu);
        auto c = scene_pairs.find(r.job.scene);
        if (c != scene_pairs.end()) return c->second;
        auto it = owner->scenes.find(r.job.scene);
        if (it == owner->scenes.end()) return 0;
        uint64_t n = 0;
        for (const auto& m : it->second->models) n += it->second->meshes[m.d.mesh].parts.size();
        const uint32_t v = (uint32_t)std::min<uint64_t>(n, 0xFFFFFFFFull);
        scene_pairs[r.job.scene] = v;
        return v;
    }

    // Completions of the slot's finished launch (called without the lock held).
    void finish(Slot& s, int rc) {
        t3d_stats st;
        if (rc == T3D_OK) rc = t3d_frame_sync(s.ctx, &st);
        const double t = now();
        std::vector<uint64_t> vis(s.batch.size(), 0), sum(s.batch.size(), 1469598103934665603ull);
        // per-job algorithmic bytes, read back with the counts by t3d_frame_sync
        std::vector<unsigned long long> jb(s.batch.size(), 0ull);
        if (rc == T3D_OK)
            for (size_t k = 0; k < jb.size() && k < s.ctx->job_bytes_host.size(); k++) jb[k] = s.ctx->job_bytes_host[k];
        if (rc == T3D_OK) {
            const auto& info = s.ctx->tables.seg_info;
            for (const auto& si : info)
                if (si.job < s.batch.size()) vis[si.job] += si.count;
            if (verify && !info.empty()) {
                // one copy of each output stream for the whole batch, then the hashes of
                // every pair's written slots in emit order
                uint64_t slots = 0;
                for (const auto& si : info) slots = std::max<uint64_t>(slots, (uint64_t)si.base + si.capacity);
                std::vector<float> xy(12 * slots), rg(12 * slots), dp(3 * slots);
                if (slots && (cudaMemcpy(xy.data(), s.ctx->out_xyuv.ptr, 48 * slots, cudaMemcpyDeviceToHost) != cudaSuccess ||
                              cudaMemcpy(rg.data(), s.ctx->out_rgba.ptr, 48 * slots, cudaMemcpyDeviceToHost) != cudaSuccess ||
                              cudaMemcpy(dp.data(), s.ctx->out_depth.ptr, 12 * slots, cudaMemcpyDeviceToHost) != cudaSuccess))
                    rc = T3D_E_CUDA;
                for (const auto& si : info) {
                    if (rc != T3D_OK || si.job >= s.batch.size() || !si.count) continue;
                    sum[si.job] = fnv(xy.data() + 12ull * si.base, 48ull * si.count, sum[si.job]);
                    sum[si.job] = fnv(rg.data() + 12ull * si.base, 48ull * si.count, sum[si.job]);
                    sum[si.job] = fnv(dp.data() + 3ull * si.base, 12ull * si.count, sum[si.job]);
                }
            }
        }
        std::lock_guard<std::mutex> g(mu);
        nbusy--;
        last_done = &s;
        if (rc != T3D_OK && err.empty()) err = s.ctx->err;
        for (size_t k = 0; k < s.batch.size(); k++) {
            t3d_completion c;
            memset(&c, 0, sizeof c);
            c.id = s.batch[k].req.id;
            c.status = rc;
            c.visible_tris = rc == T3D_OK ? vis[k] : 0;
            c.arrival_s = s.batch[k].arrival_abs;
            c.admit_s = s.batch[k].admit_abs;
            c.launch_s = s.launch_abs;
            c.batch = (uint32_t)s.batch.size();
            c.done_s = t;
            c.checksum = (verify && rc == T3D_OK) ? sum[k] : 0;
            c.model_bytes = rc == T3D_OK ? jb[k] : 0;
            done.push_back(c);
        }
        inflight -= s.bytes;
        s.bytes = 0;
        s.pairs = 0;
        s.batch.clear();
    }

    // Admits queued requests into the slot's batch (called with mu held).
    bool admit(Slot& s) {
        double t = now();
        while (!queue.empty() && s.batch.size() < max_batch) {
            Pending& p = queue.front();
            if (p.arrival_abs > t) break;  // replay: not arrived yet
            if (p.bytes > budget) {         // can never fit
                t3d_completion c;
                memset(&c, 0, sizeof c);
                c.id = p.req.id;
                c.status = T3D_E_ADMIT;
                c.arrival_s = p.arrival_abs;
                c.done_s = t;
                done.push_back(c);
                queue.pop_front();
                continue;
            }
            if (inflight + s.bytes + p.bytes > budget) break;  // wait for memory
            if (max_pairs && !s.batch.empty() && s.pairs + p.pairs > max_pairs) break;  // the next batch takes it
            p.admit_abs = t;
            s.bytes += p.bytes;
            s.pairs += p.pairs;
            s.batch.push_back(p);
            queue.pop_front();
        }
        return !s.batch.empty();
    }

    // One slot's worker: admit, build + launch, wait, complete.
    void slot_loop(Slot& s) {
        cudaSetDevice(owner->device);
        std::vector<t3d_job_desc> jobs;
        while (true) {
            {
                std::unique_lock<std::mutex> g(mu);
                while (!admit(s)) {
                    if (stop.load() && queue.empty()) return;
                    // a replayed arrival due within 100 us is waited for by polling the clock (a timed
                    // sleep overshoots by tens of microseconds); otherwise sleep until a submit, a
                    // completion or shortly before the next arrival
                    const double due = queue.empty() ? 1.0 : queue.front().arrival_abs - now();
                    const bool may_poll = nbusy > 0 || last_done == nullptr || last_done == &s;
                    if (due < 100e-6 && may_poll) {
                        g.unlock();
                        const double until = now() + std::max(0.0, due);
                        while (now() < until) std::this_thread::yield();
                        g.lock();
                        continue;
                    }
                    cv.wait_for(g, std::chrono::duration<double>(std::max(50e-6, std::min(200e-6, due - 60e-6))));
                }
                nbusy++;
                inflight += s.bytes;
            }
            jobs.resize(s.batch.size());
            for (size_t k = 0; k < s.batch.size(); k++) jobs[k] = s.batch[k].req.job;
            int rc = t3d_render_jobs(s.ctx, jobs.data(), (uint32_t)jobs.size(), T3D_MODE_BATCHED, 0, nullptr);
            s.launch_abs = now();
            finish(s, rc);  // its read-back waits for the launch
            cv.notify_all();  // memory and the slot are free again
        }
    }
};

extern "C" {

int t3d_server_create(t3d_ctx* ctx, uint64_t hbm_budget_bytes, uint32_t max_batch, uint32_t streams, t3d_server** out) {
    if (!ctx || !out || max_batch == 0 || streams == 0 || streams > 16 || hbm_budget_bytes == 0) return T3D_E_INVAL;
    *out = nullptr;
    t3d_server* s = new (std::nothrow) t3d_server();
    if (!s) return T3D_E_OOM;
    s->owner = ctx;
    s->budget = hbm_budget_bytes;
    s->max_batch = max_batch;
    s->t0 = Clock::now();
    s->slots.resize(streams);
    // A batch larger than any before grows its slot's buffers. Grown with cudaMalloc / cudaFree
    // that would wait for every slot's work on the device (a latency spike for all requests in
    // flight); grown from this pool in the slot's stream order it waits for nothing. The pool
    // keeps freed memory for reuse.
    {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = ctx->device;
        cudaSetDevice(ctx->device);
        if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) {
            delete s;
            return T3D_E_CUDA;
        }
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    for (uint32_t i = 0; i < streams; i++) {
        Slot& sl = s->slots[i];
        int rc = t3d_create(ctx->device, &sl.ctx);
        if (rc != T3D_OK) {
            for (uint32_t k = 0; k < i; k++) { cudaEventDestroy(s->slots[k].ev); t3d_destroy(s->slots[k].ctx); }
            cudaMemPoolDestroy(s->pool);
            delete s;
            return rc;
        }
        sl.ctx->pool = s->pool;
        // pinned staging of launch tables and read-backs, sized once (a pinned allocation
        // during serving would also synchronize the device)
        sl.ctx->table_host.ensure(32ull << 20);
        sl.ctx->readback.ensure(4ull << 20);
        sl.ctx->scene_owner = ctx;
        sl.ctx->tile_tris = ctx->tile_tris;
        sl.ctx->vchunk = ctx->vchunk;
        sl.ctx->block_threads = ctx->block_threads;
        sl.ctx->use_meshlets = ctx->use_meshlets;
        sl.ctx->split_phases = ctx->split_phases;
        sl.ctx->spin_limit = ctx->spin_limit;
        sl.ctx->want_job_bytes = true;
        // With one launch per phase no block waits on another, so every slot launches full
        // grids and the device interleaves the slots' blocks (a lone request gets every SM).
        // A frame as one cooperative launch needs all its blocks resident at once: each slot
        // then takes 1/streams of the co-resident blocks, so the slots' grids fit side by side.
        sl.ctx->grid_share = ctx->split_phases ? 1u : streams;
        configure(sl.ctx);
        cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming);
    }
    // Back the pool with memory now (1 GB per slot, within the budget): a slot's first large
    // batch then draws on it instead of mapping new memory while requests wait.
    {
        const size_t per = (size_t)std::min<uint64_t>(1ull << 30, hbm_budget_bytes / streams);
        std::vector<void*> warm(streams, nullptr);
        cudaStream_t st = s->slots[0].ctx->stream;
        for (uint32_t i = 0; i < streams; i++)
            if (cudaMallocFromPoolAsync(&warm[i], per, s->pool, st) != cudaSuccess) warm[i] = nullptr;
        for (void* p : warm)
            if (p) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        cudaGetLastError();
    }
    for (auto& sl : s->slots) sl.worker = std::thread([s, &sl] { s->slot_loop(sl); });
    *out = s;
    return T3D_OK;
}

int t3d_server_destroy(t3d_server* s) {
    if (!s) return T3D_E_INVAL;
    s->stop = true;
    s->cv.notify_all();
    for (auto& x : s->slots)
        if (x.worker.joinable()) x.worker.join();
    for (auto& x : s->slots) {
        cudaEventDestroy(x.ev);
        t3d_destroy(x.ctx);
    }
    cudaMemPoolDestroy(s->pool);
    delete s;
    return T3D_OK;
}

int t3d_server_set_verify(t3d_server* s, int verify) {
    if (!s) return T3D_E_INVAL;
    std::lock_guard<std::mutex> g(s->mu);
    s->verify = verify != 0;
    return T3D_OK;
}

int t3d_server_submit(t3d_server* s, const t3d_request* req) {
    if (!s || !req) return T3D_E_INVAL;
    if (s->owner->scenes.find(req->job.scene) == s->owner->scenes.end()) return T3D_E_NOTFOUND;
    if (req->job.camera.width <= 0 || req->job.camera.height <= 0) return T3D_E_INVAL;
    Pending p;
    p.req = *req;
    p.bytes = s->request_bytes(*req);
    p.pairs = s->request_pairs(*req);
    if (p.bytes > s->budget) return T3D_E_ADMIT;
    {
        std::lock_guard<std::mutex> g(s->mu);
        p.arrival_abs = s->now();
        s->queue.push_back(p);
    }
    s->cv.notify_all();
    return T3D_OK;
}

int t3d_server_set_batch_pairs(t3d_server* s, uint32_t max_pairs) {
    if (!s) return T3D_E_INVAL;
    std::lock_guard<std::mutex> g(s->mu);
    s->max_pairs = max_pairs;
    return T3D_OK;
}

int t3d_server_poll(t3d_server* s, t3d_completion* out, uint32_t max, uint32_t* n_out) {
    if (!s || !n_out || (max && !out)) return T3D_E_INVAL;
    std::lock_guard<std::mutex> g(s->mu);
    uint32_t n = (uint32_t)std::min<size_t>(max, s->done.size());
    if (n) memcpy(out, s->done.data(), sizeof(t3d_completion) * n);
    s->done.erase(s->done.begin(), s->done.begin() + n);
    *n_out = n;
    return T3D_OK;
}

int t3d_server_replay(t3d_server* s, const t3d_request* reqs, uint32_t n, t3d_completion* out) {
    if (!s || (n && (!reqs || !out))) return T3D_E_INVAL;
    for (uint32_t i = 0; i < n; i++) {
        if (s->owner->scenes.find(reqs[i].job.scene) == s->owner->scenes.end()) return T3D_E_NOTFOUND;
        if (reqs[i].job.camera.width <= 0 || reqs[i].job.camera.height <= 0) return T3D_E_INVAL;
    }
    // Enqueue everything with future arrival times; the scheduler admits each
    // request only once its arrival time has passed. The requests are prepared
    // before the lock is taken, so the slots keep admitting meanwhile.
    std::vector<Pending> add(n);
    for (uint32_t i = 0; i < n; i++) {
        add[i].req = reqs[i];
        add[i].arrival_abs = reqs[i].arrival_s;
        add[i].bytes = s->request_bytes(reqs[i]);
        add[i].pairs = s->request_pairs(reqs[i]);
    }
    std::stable_sort(add.begin(), add.end(), [](const Pending& a, const Pending& b) { return a.arrival_abs < b.arrival_abs; });
    {
        std::lock_guard<std::mutex> g(s->mu);
        const double base = s->now() + 0.002;
        for (auto& p : add) p.arrival_abs += base;
        std::deque<Pending> merged;
        std::merge(s->queue.begin(), s->queue.end(), add.begin(), add.end(), std::back_inserter(merged),
                   [](const Pending& a, const Pending& b) { return a.arrival_abs < b.arrival_abs; });
        s->queue.swap(merged);
    }
    s->cv.notify_all();
    std::vector<t3d_completion> got;
    got.reserve(n);
    while (got.size() < n) {
        std::vector<t3d_completion> tmp(256);
        uint32_t k = 0;
        t3d_server_poll(s, tmp.data(), (uint32_t)tmp.size(), &k);
        got.insert(got.end(), tmp.begin(), tmp.begin() + k);
        if (k == 0) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    std::map<uint64_t, size_t> pos;
    for (uint32_t i = 0; i < n; i++) pos[reqs[i].id] = i;
    for (auto& c : got) {
        auto it = pos.find(c.id);
        if (it != pos.end()) out[it->second] = c;
    }
    return T3D_OK;
}

}  // extern "C"
