// r2p_server.cu -- the served path: a continuous-batching request server
// over pooled device and pinned host memory (part of the C ABI of
// include/r2p.h; no counterpart in the reference).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "r2p_engine_impl.h"

using namespace r2p;

// ===========================================================================
// Serving: continuous batching over pooled device memory
// ===========================================================================
namespace r2p {

// First-fit allocator over [0, cap) in 256-byte units with coalescing frees.
class RangeAllocator {
public:
    void init(size_t cap)
    {
        free_.clear();
        cap_ = cap;
        used_ = 0;
        if (cap) free_[0] = cap;
    }
    bool alloc(size_t n, size_t& off)
    {
        n = align_up(n ? n : 1, 256);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            off = it->first;
            const size_t rest = it->second - n, o2 = it->first + n;
            free_.erase(it);
            if (rest) free_[o2] = rest;
            used_ += n;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(size_t off, size_t n)
    {
        n = align_up(n ? n : 1, 256);
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }
    size_t peak() const { return peak_; }
    size_t cap() const { return cap_; }

private:
    std::map<size_t, size_t> free_;
    size_t cap_ = 0, used_ = 0, peak_ = 0;
};

using Clock = std::chrono::steady_clock;

enum ReqState { RQ_PENDING, RQ_RUNNING, RQ_DONE, RQ_FAILED, RQ_CANCELED };

struct Request {
    uint64_t ticket = 0;
    r2p_image img{};
    ImgPlan plan;
    size_t raw_bytes = 0, bound = 0, est_scratch = 0;
    // host side: pixels then PNG, in the pinned pool or (when full) in `heap`
    size_t h_off = 0, h_bytes = 0;
    bool h_pinned = false;
    std::vector<uint8_t> heap;
    uint8_t* h_px = nullptr;
    uint8_t* h_png = nullptr;
    // device side: pixels then PNG
    size_t d_off = 0, d_bytes = 0;
    int state = RQ_PENDING;
    int status = R2P_OK;
    size_t png_len = 0;
    Clock::time_point t_submit, t_dispatch, t_done;
};

struct Slot {
    cudaStream_t s = nullptr;
    bool active = false;
    int phase = 0;                 // 1: kernels + lengths queued, 2: PNG copies queued
    // set by the stream's host functions, which never take the server mutex
    std::atomic<bool> lens_ready{false}, pngs_ready{false};
    std::vector<Request*> reqs;
    std::vector<ImgPlan> plans;
    Prepared P;
    size_t scratch_off = 0, scratch_bytes = 0;
    // descriptor + length staging: a range of the pinned pool, else `heap`
    size_t stage_off = 0, stage_bytes = 0;
    bool stage_pinned = false;
    std::vector<uint8_t> heap;
    uint8_t* h_desc = nullptr;
    uint64_t* h_lens = nullptr;
    void* srv = nullptr;           // the owning r2p_server
};

}  // namespace r2p

// Locking: `mu` guards the queues, the pools, request states and statistics.
// The dispatcher makes its CUDA calls without `mu` where it can, and the
// stream host functions take only `wake_mu` (never held across a CUDA call),
// so a CUDA call that waits for the device can never wait on a host function
// that waits on a lock.
struct r2p_server {
    r2p_engine* eng = nullptr;
    r2p_server_config cfg{};
    uint8_t* dmem = nullptr;
    uint8_t* hmem = nullptr;
    r2p::RangeAllocator dpool, hpool;
    std::mutex mu;
    std::condition_variable cv_done;
    std::mutex wake_mu;
    std::condition_variable cv_wake;
    uint64_t wake_seq = 0;
    std::deque<r2p::Request*> pending;
    std::unordered_map<uint64_t, r2p::Request*> reqs;
    std::vector<std::unique_ptr<r2p::Slot>> slots;
    std::thread dispatcher;
    bool stop = false;
    uint64_t next_ticket = 1;
    // statistics
    std::vector<double> lat_ms;
    uint64_t completed = 0, failed = 0, canceled = 0, batches = 0, batched_images = 0;
    int dispatch_error = R2P_OK;
};

namespace r2p {

static void wake_dispatcher(r2p_server* sv)
{
    {
        std::lock_guard<std::mutex> lk(sv->wake_mu);
        sv->wake_seq++;
    }
    sv->cv_wake.notify_one();
}

static uint64_t wake_snapshot(r2p_server* sv)
{
    std::lock_guard<std::mutex> lk(sv->wake_mu);
    return sv->wake_seq;
}

static void CUDART_CB host_lens_ready(void* p)
{
    Slot* sl = static_cast<Slot*>(p);
    sl->lens_ready.store(true, std::memory_order_release);
    wake_dispatcher(reinterpret_cast<r2p_server*>(sl->srv));
}

static void CUDART_CB host_pngs_ready(void* p)
{
    Slot* sl = static_cast<Slot*>(p);
    sl->pngs_ready.store(true, std::memory_order_release);
    wake_dispatcher(reinterpret_cast<r2p_server*>(sl->srv));
}

static double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Finish a request (mu held): free its device memory and count it.
static void finish_request(r2p_server* sv, Request* r, int state, int status)
{
    if (r->d_bytes) sv->dpool.release(r->d_off, r->d_bytes);
    r->d_bytes = 0;
    r->state = state;
    r->status = status;
    r->t_done = Clock::now();
    if (state == RQ_DONE) {
        sv->completed++;
        sv->lat_ms.push_back(ms_between(r->t_submit, r->t_done));
    } else if (state == RQ_FAILED) {
        sv->failed++;
    } else {
        sv->canceled++;
    }
}

// Release a slot's scratch and staging (mu held).
static void release_slot_memory(r2p_server* sv, Slot& sl)
{
    if (sl.scratch_bytes) sv->dpool.release(sl.scratch_off, sl.scratch_bytes);
    if (sl.stage_pinned) sv->hpool.release(sl.stage_off, sl.stage_bytes);
    sl.scratch_bytes = sl.stage_bytes = 0;
    sl.stage_pinned = false;
}

// Phase 1 -> 2 (no lock: a running slot and its requests belong to the
// dispatcher): the lengths are on the host, queue the exact PNG bytes back.
static void queue_png_copies(r2p_server* sv, Slot& sl)
{
    for (size_t i = 0; i < sl.reqs.size(); i++) {
        Request* r = sl.reqs[i];
        const uint64_t len = sl.h_lens[i];
        if (len >> 63) {
            r->status = (int)(len & 0xFF);
            r->png_len = 0;
            continue;
        }
        r->png_len = (size_t)len;
        if (cudaMemcpyAsync(r->h_png, sv->dmem + r->d_off + align_up(r->raw_bytes, 256), len, cudaMemcpyDeviceToHost,
                            sl.s) != cudaSuccess) {
            r->status = cuda_err(cudaGetLastError(), "server png readback");
            r->png_len = 0;
        }
    }
    sl.phase = 2;
    if (cudaLaunchHostFunc(sl.s, host_pngs_ready, &sl) != cudaSuccess) {
        cudaStreamSynchronize(sl.s);
        sl.pngs_ready.store(true, std::memory_order_release);
    }
}

// Phase 2 done (mu held): hand the results over and free the slot.
static void retire_slot(r2p_server* sv, Slot& sl)
{
    for (Request* r : sl.reqs) {
        if (r->status == R2P_OK) finish_request(sv, r, RQ_DONE, R2P_OK);
        else finish_request(sv, r, RQ_FAILED, r->status);
    }
    release_slot_memory(sv, sl);
    sl.reqs.clear();
    sl.plans.clear();
    sl.active = false;
    sl.phase = 0;
    sv->cv_done.notify_all();
}

// Form one batch for an idle slot from the pending queue and launch it.
// Returns whether a batch was formed.
static bool launch_batch(r2p_server* sv, Slot& sl)
{
    r2p_engine* e = sv->eng;
    std::vector<Request*> take;
    CallBuffers cb;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        size_t est = 0, raw_total = 0;
        while (!sv->pending.empty() && (int)take.size() < sv->cfg.max_batch_images) {
            Request* r = sv->pending.front();
            if (!take.empty() && raw_total + r->raw_bytes > sv->cfg.max_batch_bytes) break;
            // admission: its pixels + PNG now, and room for its scratch later
            if (!sv->dpool.alloc(r->d_bytes, r->d_off)) break;
            if (sv->dpool.cap() - sv->dpool.used() < est + r->est_scratch) {
                sv->dpool.release(r->d_off, r->d_bytes);
                break;
            }
            est += r->est_scratch;
            raw_total += r->raw_bytes;
            sv->pending.pop_front();
            take.push_back(r);
        }
        if (take.empty()) return false;
        // plan; if the batch's scratch does not fit, hand back requests from the tail
        for (;;) {
            sl.plans.clear();
            cb = CallBuffers();
            for (Request* r : take) {
                sl.plans.push_back(r->plan);
                cb.raw.push_back(sv->dmem + r->d_off);
                cb.filt.push_back(nullptr);
                cb.prior.push_back(nullptr);
                cb.out.push_back(sv->dmem + r->d_off + align_up(r->raw_bytes, 256));
                cb.out_cap.push_back(r->bound);
                cb.out_len.push_back(nullptr);
            }
            sl.P = Prepared();
            plan_work(e, sl.plans, cb, 8 * take.size(), sl.P);
            if (sv->dpool.alloc(sl.P.total, sl.scratch_off)) {
                sl.scratch_bytes = sl.P.total;
                break;
            }
            Request* r = take.back();
            take.pop_back();
            sv->dpool.release(r->d_off, r->d_bytes);
            sv->pending.push_front(r);
            if (take.empty()) return false;
        }
        // descriptor + length staging from the pinned pool (no allocation call)
        sl.stage_bytes = align_up(sl.P.desc_bytes, 256) + 8 * take.size();
        sl.stage_pinned = sv->hpool.alloc(sl.stage_bytes, sl.stage_off);
        uint8_t* hs;
        if (sl.stage_pinned) {
            hs = sv->hmem + sl.stage_off;
        } else {
            sl.heap.resize(sl.stage_bytes);
            hs = sl.heap.data();
        }
        sl.h_desc = hs;
        sl.h_lens = reinterpret_cast<uint64_t*>(hs + align_up(sl.P.desc_bytes, 256));
        const Clock::time_point now = Clock::now();
        for (Request* r : take) {
            r->state = RQ_RUNNING;
            r->t_dispatch = now;
        }
        sv->batches++;
        sv->batched_images += take.size();
    }
    // enqueue without the lock
    const size_t n = take.size();
    uint8_t* base = sv->dmem + sl.scratch_off;
    for (size_t i = 0; i < n; i++) cb.out_len[i] = reinterpret_cast<uint64_t*>(base + sl.P.o_extra) + i;
    fill_pointers(sl.plans, cb, sl.P, base);
    sl.reqs = take;
    sl.active = true;
    sl.phase = 1;
    sl.lens_ready.store(false, std::memory_order_relaxed);
    sl.pngs_ready.store(false, std::memory_order_relaxed);
    cudaError_t ce = cudaSuccess;
    for (size_t i = 0; i < n && ce == cudaSuccess; i++) {
        Request* r = take[i];
        ce = cudaMemcpyAsync(sv->dmem + r->d_off, r->h_px, r->raw_bytes, cudaMemcpyHostToDevice, sl.s);
    }
    if (ce == cudaSuccess) {
        write_descriptors(sl.h_desc, sl.plans, sl.P);
        ce = cudaMemcpyAsync(base, sl.h_desc, sl.P.desc_bytes, cudaMemcpyHostToDevice, sl.s);
    }
    int rc = (ce == cudaSuccess) ? launch_stages(e, (int)n, sl.P, base, ST_ALL, sl.s, nullptr, nullptr)
                                 : cuda_err(ce, "server batch upload");
    if (rc == R2P_OK) {
        ce = cudaMemcpyAsync(sl.h_lens, base + sl.P.o_extra, 8 * n, cudaMemcpyDeviceToHost, sl.s);
        if (ce == cudaSuccess) ce = cudaLaunchHostFunc(sl.s, host_lens_ready, &sl);
        if (ce != cudaSuccess) rc = cuda_err(ce, "server batch readback");
    }
    if (rc != R2P_OK) {
        // nothing of this batch will report back: let queued work drain, then
        // fail its requests
        cudaStreamSynchronize(sl.s);
        std::lock_guard<std::mutex> lk(sv->mu);
        for (Request* r : take) finish_request(sv, r, RQ_FAILED, rc);
        release_slot_memory(sv, sl);
        sl.reqs.clear();
        sl.plans.clear();
        sl.active = false;
        sl.phase = 0;
        sv->dispatch_error = rc;
        sv->cv_done.notify_all();
    }
    return true;
}

static void dispatcher_main(r2p_server* sv)
{
    cudaSetDevice(sv->eng->device);
    for (;;) {
        // taken before looking at any state, so no wake-up in between is lost
        const uint64_t seen = wake_snapshot(sv);
        bool progressed = false;
        for (auto& slp : sv->slots) {
            Slot& sl = *slp;
            if (!sl.active) continue;
            if (sl.phase == 1 && sl.lens_ready.load(std::memory_order_acquire)) {
                queue_png_copies(sv, sl);
                progressed = true;
            }
            if (sl.phase == 2 && sl.pngs_ready.load(std::memory_order_acquire)) {
                std::lock_guard<std::mutex> lk(sv->mu);
                retire_slot(sv, sl);
                progressed = true;
            }
        }
        for (auto& slp : sv->slots)
            if (!slp->active && launch_batch(sv, *slp)) progressed = true;
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            bool any_active = false;
            for (auto& slp : sv->slots) any_active |= slp->active;
            if (sv->stop && sv->pending.empty() && !any_active) break;
        }
        if (progressed) continue;
        std::unique_lock<std::mutex> wl(sv->wake_mu);
        sv->cv_wake.wait_for(wl, std::chrono::milliseconds(50), [&] { return sv->wake_seq != seen; });
    }
}

}  // namespace r2p

extern "C" {

int r2p_server_create(int device, const r2p_server_config* cfg, r2p_server** out)
{
    if (!out) return set_err(R2P_EINVAL, "out is NULL");
    *out = nullptr;
    r2p_server_config c{};
    if (cfg) c = *cfg;
    if (c.hbm_budget == 0) c.hbm_budget = (size_t)40 << 30;
    if (c.host_pool_bytes == 0) c.host_pool_bytes = (size_t)4 << 30;
    if (c.max_inflight_batches <= 0) c.max_inflight_batches = 8;
    if (c.max_batch_images <= 0) c.max_batch_images = 512;
    if (c.max_batch_bytes == 0) c.max_batch_bytes = (size_t)96 << 20;
    r2p_engine* e = nullptr;
    int rc = r2p_engine_create(device, 0, &e);
    if (rc) return rc;
    r2p_server* sv = new r2p_server();
    sv->eng = e;
    sv->cfg = c;
    cudaError_t ce = cudaMalloc(&sv->dmem, c.hbm_budget);
    if (ce == cudaSuccess) ce = cudaMallocHost(&sv->hmem, c.host_pool_bytes);
    for (int i = 0; i < c.max_inflight_batches; i++) {
        sv->slots.emplace_back(new r2p::Slot());
        sv->slots.back()->srv = sv;
        if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&sv->slots.back()->s, cudaStreamNonBlocking);
    }
    if (ce != cudaSuccess) {
        for (auto& sl : sv->slots)
            if (sl->s) cudaStreamDestroy(sl->s);
        if (sv->dmem) cudaFree(sv->dmem);
        if (sv->hmem) cudaFreeHost(sv->hmem);
        r2p_engine_destroy(e);
        delete sv;
        return cuda_err(ce, "r2p_server_create");
    }
    sv->dpool.init(c.hbm_budget);
    sv->hpool.init(c.host_pool_bytes);
    sv->dispatcher = std::thread(dispatcher_main, sv);
    *out = sv;
    return R2P_OK;
}

int r2p_server_set_tuning(r2p_server* sv, int n, const r2p_tuning* classes)
{
    if (!sv) return set_err(R2P_EINVAL, "NULL server");
    return r2p_engine_set_tuning(sv->eng, n, classes);
}

int r2p_server_submit(r2p_server* sv, const r2p_image* img, const void* h_pixels, uint64_t* ticket)
{
    return r2p_server_submit_ex(sv, img, h_pixels, 0u, ticket);
}

int r2p_server_submit_ex(r2p_server* sv, const r2p_image* img, const void* h_pixels, uint32_t flags,
                         uint64_t* ticket)
{
    if (!sv || !img || !h_pixels || !ticket) return set_err(R2P_EINVAL, "NULL argument");
    if (flags & ~(uint32_t)R2P_SUBMIT_BORROW) return set_err(R2P_EINVAL, "unknown submit flags");
    const bool borrow = (flags & R2P_SUBMIT_BORROW) != 0;
    Request* r = new Request();
    r->img = *img;
    int rc = plan_image(*img, 0, r->plan, sv->eng->tuning);
    if (rc) { delete r; return rc; }
    r->raw_bytes = (size_t)r->plan.raw_bytes;
    r->bound = (size_t)r->plan.png_bound;
    r->d_bytes = align_up(r->raw_bytes, 256) + align_up(r->bound, 256);
    const DevImage& d = r->plan.di;
    r->est_scratch = sizeof(DevImage) + 4096 + (size_t)d.nblocks * (sizeof(BlockOut) + lz77_slot_bytes(d.block_size)) +
                     align_up(d.filt_bytes + 64, 256) + (size_t)r->plan.lut_cap + 4 * 256;
    if (r->d_bytes + r->est_scratch > sv->cfg.hbm_budget) {
        delete r;
        return set_err(R2P_EBUDGET, "request larger than the server's HBM budget");
    }
    // host space: the PNG (and a copy of the pixels unless they are borrowed)
    const size_t px_room = borrow ? 0 : align_up(r->raw_bytes, 256);
    r->h_bytes = px_room + r->bound;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        r->h_pinned = sv->hpool.alloc(r->h_bytes, r->h_off);
    }
    uint8_t* hb;
    if (r->h_pinned) {
        hb = sv->hmem + r->h_off;
    } else {
        r->heap.resize(r->h_bytes);
        hb = r->heap.data();
    }
    r->h_png = hb + px_room;
    if (borrow) {
        r->h_px = static_cast<uint8_t*>(const_cast<void*>(h_pixels));
    } else {
        r->h_px = hb;
        memcpy(r->h_px, h_pixels, r->raw_bytes);
    }
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stop) {
            if (r->h_pinned) sv->hpool.release(r->h_off, r->h_bytes);
            delete r;
            return set_err(R2P_ECANCELED, "server is shutting down");
        }
        r->ticket = sv->next_ticket++;
        sv->reqs[r->ticket] = r;
        sv->pending.push_back(r);
        *ticket = r->ticket;
    }
    wake_dispatcher(sv);
    return R2P_OK;
}

int r2p_server_wait(r2p_server* sv, uint64_t ticket, int timeout_ms, r2p_result* res)
{
    if (!sv || !res) return set_err(R2P_EINVAL, "NULL argument");
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return set_err(R2P_ENOTFOUND, "unknown ticket");
    Request* r = it->second;
    auto finished = [&] { return r->state == RQ_DONE || r->state == RQ_FAILED || r->state == RQ_CANCELED; };
    if (timeout_ms < 0) sv->cv_done.wait(lk, finished);
    else if (!sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished))
        return set_err(R2P_ETIMEOUT, "request still running");
    res->status = r->status;
    res->png = r->state == RQ_DONE ? r->h_png : nullptr;
    res->png_len = r->state == RQ_DONE ? r->png_len : 0;
    res->latency_ms = ms_between(r->t_submit, r->t_done);
    res->queue_ms = r->state == RQ_CANCELED ? res->latency_ms : ms_between(r->t_submit, r->t_dispatch);
    return r->status == R2P_OK ? R2P_OK : set_err(r->status, r->state == RQ_CANCELED ? "request cancelled"
                                                                                   : "request failed");
}

int r2p_server_cancel(r2p_server* sv, uint64_t ticket)
{
    if (!sv) return set_err(R2P_EINVAL, "NULL server");
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return set_err(R2P_ENOTFOUND, "unknown ticket");
    Request* r = it->second;
    if (r->state != RQ_PENDING) return set_err(R2P_EINVAL, "request already dispatched or finished");
    for (auto q = sv->pending.begin(); q != sv->pending.end(); ++q)
        if (*q == r) { sv->pending.erase(q); break; }
    r->d_bytes = 0;
    finish_request(sv, r, RQ_CANCELED, R2P_ECANCELED);
    sv->cv_done.notify_all();
    return R2P_OK;
}

int r2p_server_release(r2p_server* sv, uint64_t ticket)
{
    if (!sv) return set_err(R2P_EINVAL, "NULL server");
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return set_err(R2P_ENOTFOUND, "unknown ticket");
    Request* r = it->second;
    if (r->state == RQ_PENDING || r->state == RQ_RUNNING) return set_err(R2P_EINVAL, "request still in flight");
    if (r->h_pinned) sv->hpool.release(r->h_off, r->h_bytes);
    sv->reqs.erase(it);
    delete r;
    return R2P_OK;
}

int r2p_server_get_stats(r2p_server* sv, r2p_server_stats* st)
{
    if (!sv || !st) return set_err(R2P_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    memset(st, 0, sizeof(*st));
    st->completed = sv->completed;
    st->failed = sv->failed;
    st->canceled = sv->canceled;
    st->batches = sv->batches;
    st->mean_batch_images = sv->batches ? (double)sv->batched_images / (double)sv->batches : 0.0;
    st->pending = sv->pending.size();
    st->device_bytes_in_use = sv->dpool.used();
    st->device_bytes_peak = sv->dpool.peak();
    if (!sv->lat_ms.empty()) {
        std::vector<double> v = sv->lat_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) { return v[std::min(v.size() - 1, (size_t)(q * (double)(v.size() - 1) + 0.5))]; };
        st->p50_ms = pct(0.50);
        st->p99_ms = pct(0.99);
        st->max_ms = v.back();
    }
    return R2P_OK;
}

int r2p_server_reset_stats(r2p_server* sv)
{
    if (!sv) return set_err(R2P_EINVAL, "NULL server");
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->lat_ms.clear();
    sv->completed = sv->failed = sv->canceled = sv->batches = sv->batched_images = 0;
    return R2P_OK;
}

void r2p_server_destroy(r2p_server* sv)
{
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    r2p::wake_dispatcher(sv);
    if (sv->dispatcher.joinable()) sv->dispatcher.join();
    cudaSetDevice(sv->eng->device);
    for (auto& kv : sv->reqs) delete kv.second;
    for (auto& sl : sv->slots)
        if (sl->s) cudaStreamDestroy(sl->s);
    if (sv->dmem) cudaFree(sv->dmem);
    if (sv->hmem) cudaFreeHost(sv->hmem);
    r2p_engine_destroy(sv->eng);
    delete sv;
}

}  // extern "C"
