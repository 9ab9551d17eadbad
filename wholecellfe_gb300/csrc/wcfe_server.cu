// wcfe_server.cu — continuous batching of whole cell simulations on one engine.
//
// Requests (a mesh, its start positions, parameters and a step count) are admitted as
// device memory frees up and advance together, so that many cells of different sizes and
// stiffness laws share every launch.  The loop keeps the GPU busy and the host off its
// critical path:
//
//  - preparation: worker threads build each request's connectivity, patches and start
//    state in the engine's layout (serving_prepare: host arithmetic only), in arrival
//    order, ahead of admission;
//  - admission: in arrival order while the HBM budget has room; the cell's blocks come
//    from a stream-ordered memory pool and are uploaded on an admission stream, which
//    the engine stream waits for with an event; the host waits for those uploads only,
//    never for the steps in flight;
//  - stepping: one iteration enqueues K steps of every resident cell (K chosen so that an
//    iteration takes about `iter_ms` of GPU time).  Each cell carries its remaining step
//    count on the device (ctl[3]); the last patch CTA of a step counts it down and the
//    kernels skip a cell whose count ran out, so a cell runs exactly its requested
//    number of steps whatever K is;
//  - retirement: a cell that finishes within an iteration has its positions copied into
//    a pinned ring right after that iteration's steps and its blocks freed behind the
//    copy, both in stream order; the host decodes the result once the iteration's event
//    has completed;
//  - at most two iterations are in flight: the host waits for the one before the last
//    while the GPU runs the last.
//
// A cell's arithmetic does not depend on which other cells share its launches, so each
// result is the same alone and in the mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/wcfe.h"
#include "wcfe_serving.h"

namespace {
using clk = std::chrono::steady_clock;

struct Req {
    int64_t id = 0;
    int32_t nv = 0, nt = 0, steps = 0;
    std::vector<int32_t> tri, sub_tri;
    std::vector<double> x, sub_X, x_final;
    int32_t sub_nv = 0, sub_nt = 0;
    wcfe_params prm{};
    // preparation (worker threads)
    std::atomic<int> prep{0};          // 0 queued, 1 ready, 2 failed
    std::string prep_err;
    wcfe::PreparedCell pc;
    // on the device
    int32_t cell = -1;
    int32_t left = 0;                  // steps not yet enqueued
    int32_t done_steps = 0;            // steps enqueued so far (the parity of its positions)
    // retirement
    size_t ring_off = 0, ring_bytes = 0;
    int status = 0;                    // WCFE_OK, or the error that ended it
    bool finished = false;
    clk::time_point t_submit, t_done;
};

struct Iter {
    cudaEvent_t t0 = nullptr, t1 = nullptr;   // timing events around the iteration's steps
    int k = 0;
    std::vector<Req*> retired;                 // results copied in this iteration
};
}  // namespace

struct wcfe_server {
    wcfe_engine* eng = nullptr;
    double dt = 0;
    int64_t next_id = 0;
    double iter_ms = 8.0;          // GPU time one iteration aims at
    int kmax = 64;
    double step_ms_est = 0.0;      // last measured device time per step
    // requests
    std::map<int64_t, std::unique_ptr<Req>> all;
    std::deque<Req*> queue;        // arrival order, not yet admitted
    std::vector<Req*> active;
    // preparation workers
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Req*> to_prepare;
    std::vector<std::thread> workers;
    bool stop = false;
    // device
    cudaStream_t adm = nullptr;
    cudaMemPool_t pool = nullptr;
    cudaEvent_t adm_ev = nullptr;
    std::deque<Iter> inflight;
    std::vector<cudaEvent_t> free_events;
    // pinned result ring (FIFO: results are decoded in the order they were copied)
    uint8_t* ring = nullptr;
    size_t ring_cap = 0, ring_head = 0, ring_used = 0;
    std::deque<std::pair<size_t, size_t>> ring_live;   // (offset, bytes) in copy order
    // statistics
    std::vector<double> step_times;   // seconds per step (device time of an iteration / its steps)
    uint64_t cell_steps = 0;
};

namespace {

int fail_srv(const char* msg, int code) { return wcfe::set_error(msg, code); }

void worker_loop(wcfe_server* s) {
    for (;;) {
        Req* r = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, [&] { return s->stop || !s->to_prepare.empty(); });
            if (s->stop) return;
            r = s->to_prepare.front();
            s->to_prepare.pop_front();
        }
        std::string err = wcfe::serving_prepare(s->eng, r->pc, r->nv, r->nt, r->tri.data(), r->x.data(), r->prm,
                                                r->steps);
        r->prep_err = err;
        r->prep.store(err.empty() ? 1 : 2, std::memory_order_release);
    }
}

cudaEvent_t get_event(wcfe_server* s) {
    if (!s->free_events.empty()) {
        cudaEvent_t e = s->free_events.back();
        s->free_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// a chunk of the pinned ring; false if it has no room now
bool ring_alloc(wcfe_server* s, size_t bytes, size_t* off) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes > s->ring_cap) return false;
    size_t start = s->ring_head;
    if (start + bytes > s->ring_cap) {   // wrap: the tail end of the ring is skipped
        const size_t skip = s->ring_cap - start;
        if (s->ring_used + skip + bytes > s->ring_cap) return false;
        s->ring_live.push_back({start, skip});
        s->ring_used += skip;
        start = 0;
    }
    if (s->ring_used + bytes > s->ring_cap) return false;
    s->ring_live.push_back({start, bytes});
    s->ring_used += bytes;
    s->ring_head = start + bytes;
    *off = start;
    return true;
}
// release ring chunks from the front while they are no longer live
void ring_release_front(wcfe_server* s, size_t off) {
    while (!s->ring_live.empty()) {
        const auto f = s->ring_live.front();
        s->ring_live.pop_front();
        s->ring_used -= f.second;
        if (f.first == off) break;
    }
    if (s->ring_live.empty()) s->ring_head = 0;
}

// the oldest iteration in flight has completed: timings and its retired results
void finish_iter(wcfe_server* s) {
    Iter it = s->inflight.front();
    s->inflight.pop_front();
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, it.t0, it.t1) == cudaSuccess && it.k > 0) {
        const double per = ms / it.k;
        s->step_ms_est = per;
        for (int i = 0; i < it.k; ++i) s->step_times.push_back(per * 1e-3);
    } else {
        cudaGetLastError();
    }
    const auto now = clk::now();
    for (Req* r : it.retired) {
        r->x_final.assign(3 * (size_t)r->nv, 0.0);
        wcfe::serving_decode_positions(s->eng, s->ring + r->ring_off, r->nv, r->x_final.data());
        ring_release_front(s, r->ring_off);
        r->finished = true;
        r->t_done = now;
    }
    s->free_events.push_back(it.t0);
    s->free_events.push_back(it.t1);
}

int wait_oldest(wcfe_server* s) {
    if (s->inflight.empty()) return WCFE_OK;
    if (cudaEventSynchronize(s->inflight.front().t1) != cudaSuccess) {
        cudaGetLastError();
        return fail_srv("serving iteration failed on the device", WCFE_ERR_CUDA);
    }
    finish_iter(s);
    return WCFE_OK;
}

// admit prepared requests from the head of the queue while the budget has room
int admit(wcfe_server* s, int* admitted) {
    wcfe_engine* e = s->eng;
    const uint64_t budget = wcfe::engine_budget(e);
    *admitted = 0;
    while (!s->queue.empty()) {
        Req* r = s->queue.front();
        const int st = r->prep.load(std::memory_order_acquire);
        if (st == 0) break;   // still being prepared: keep arrival order
        if (st == 2) {
            r->status = WCFE_ERR_TOPOLOGY;
            r->finished = true;
            r->t_done = clk::now();
            s->queue.pop_front();
            continue;
        }
        const uint64_t need = r->pc.state_bytes + r->pc.patch_bytes;
        if (budget && wcfe::engine_used(e) + need > budget) {
            if (s->active.empty() && s->inflight.empty()) {   // can never fit
                r->status = WCFE_ERR_BUDGET;
                r->finished = true;
                r->t_done = clk::now();
                s->queue.pop_front();
                continue;
            }
            break;
        }
        int32_t id = -1;
        int rc = wcfe::serving_admit(e, r->pc, s->adm, s->pool, &id);
        if (rc) return rc;
        if (cudaStreamSynchronize(s->adm) != cudaSuccess) {   // the uploads have read the host arrays
            cudaGetLastError();
            return fail_srv("admission upload failed", WCFE_ERR_CUDA);
        }
        r->pc = wcfe::PreparedCell();
        r->cell = id;
        r->left = r->steps;
        r->done_steps = 0;
        s->active.push_back(r);
        s->queue.pop_front();
        ++*admitted;
    }
    if (*admitted) {
        if (cudaEventRecord(s->adm_ev, s->adm) != cudaSuccess ||
            cudaStreamWaitEvent(wcfe::engine_stream(e), s->adm_ev, 0) != cudaSuccess) {
            cudaGetLastError();
            return fail_srv("admission event failed", WCFE_ERR_CUDA);
        }
    }
    return WCFE_OK;
}

// requests with a substrate mesh take the engine's synchronous path (rare in serving)
int admit_with_substrate(wcfe_server* s, Req* r) {
    int32_t id = -1;
    int rc = wcfe_cell_create(s->eng, r->nv, r->nt, r->tri.data(), nullptr, nullptr, nullptr, &r->prm, &id);
    if (rc) return rc;
    rc = wcfe_cell_set_state(s->eng, id, r->x.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (!rc) rc = wcfe_cell_set_substrate(s->eng, id, r->sub_nv, r->sub_nt, r->sub_tri.data(), r->sub_X.data(), nullptr);
    if (!rc) rc = wcfe_cell_set_step_budget(s->eng, id, r->steps);
    if (rc) {
        wcfe_cell_destroy(s->eng, id);
        return rc;
    }
    r->cell = id;
    r->left = r->steps;
    s->active.push_back(r);
    return WCFE_OK;
}

}  // namespace

extern "C" {

int wcfe_server_create(wcfe_engine* eng, double dt, wcfe_server** out) {
    if (!eng || !out || !(dt > 0)) return fail_srv("bad argument", WCFE_ERR_ARG);
    std::unique_ptr<wcfe_server> s(new wcfe_server());
    s->eng = eng;
    s->dt = dt;
    if (cudaSetDevice(wcfe::engine_device(eng)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->adm, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->adm_ev, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return fail_srv("serving streams", WCFE_ERR_CUDA);
    }
    cudaMemPoolProps pp{};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = wcfe::engine_device(eng);
    if (cudaMemPoolCreate(&s->pool, &pp) != cudaSuccess) {
        cudaGetLastError();
        return fail_srv("cudaMemPoolCreate", WCFE_ERR_CUDA);
    }
    uint64_t keep = ~0ull;   // the pool keeps freed blocks for later admissions
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    s->ring_cap = size_t(256) << 20;
    if (cudaMallocHost(&s->ring, s->ring_cap) != cudaSuccess) {
        cudaGetLastError();
        return fail_srv("pinned result ring", WCFE_ERR_NOMEM);
    }
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nw = (int)std::min(4u, std::max(1u, hw / 2));
    for (int i = 0; i < nw; ++i) s->workers.emplace_back(worker_loop, s.get());
    *out = s.release();
    return WCFE_OK;
}

int wcfe_server_destroy(wcfe_server* s) {
    if (!s) return WCFE_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    for (auto& t : s->workers) t.join();
    cudaSetDevice(wcfe::engine_device(s->eng));
    while (!s->inflight.empty()) wait_oldest(s);
    for (Req* r : s->active)
        if (r->cell >= 0) wcfe_cell_destroy(s->eng, r->cell);
    cudaStreamSynchronize(wcfe::engine_stream(s->eng));
    cudaStreamSynchronize(s->adm);
    for (cudaEvent_t e : s->free_events) cudaEventDestroy(e);
    if (s->adm_ev) cudaEventDestroy(s->adm_ev);
    if (s->adm) cudaStreamDestroy(s->adm);
    if (s->ring) cudaFreeHost(s->ring);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return WCFE_OK;
}

int wcfe_server_submit(wcfe_server* s, const wcfe_request* q, int64_t* id) {
    if (!s || !q || !q->tri || !q->x || !q->params || q->n_vert <= 0 || q->n_tri <= 0 || q->n_steps <= 0)
        return fail_srv("bad argument", WCFE_ERR_ARG);
    std::unique_ptr<Req> r(new Req());
    r->id = s->next_id++;
    r->nv = q->n_vert;
    r->nt = q->n_tri;
    r->steps = q->n_steps;
    r->tri.assign(q->tri, q->tri + 3 * (size_t)q->n_tri);
    r->x.assign(q->x, q->x + 3 * (size_t)q->n_vert);
    r->prm = *q->params;
    if (q->sub_tri && q->sub_X && q->sub_n_tri > 0) {
        r->sub_nv = q->sub_n_vert;
        r->sub_nt = q->sub_n_tri;
        r->sub_tri.assign(q->sub_tri, q->sub_tri + 3 * (size_t)q->sub_n_tri);
        r->sub_X.assign(q->sub_X, q->sub_X + 3 * (size_t)q->sub_n_vert);
        r->prep.store(1);   // admitted through the engine's own cell creation
    }
    r->t_submit = clk::now();
    if (id) *id = r->id;
    Req* p = r.get();
    s->all[r->id] = std::move(r);
    s->queue.push_back(p);
    if (p->sub_nt == 0) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->to_prepare.push_back(p);
        }
        s->cv.notify_one();
    }
    return WCFE_OK;
}

int wcfe_server_iterate(wcfe_server* s, int32_t* n_active, int32_t* n_queued) {
    if (!s) return fail_srv("bad argument", WCFE_ERR_ARG);
    if (cudaSetDevice(wcfe::engine_device(s->eng)) != cudaSuccess) {
        cudaGetLastError();
        return fail_srv("cudaSetDevice", WCFE_ERR_CUDA);
    }
    // iterations that have completed meanwhile
    while (!s->inflight.empty() && cudaEventQuery(s->inflight.front().t1) == cudaSuccess) finish_iter(s);
    cudaGetLastError();   // cudaErrorNotReady from the query
    // admission: requests with a substrate through the engine's synchronous path
    while (!s->queue.empty() && s->queue.front()->sub_nt > 0) {
        Req* r = s->queue.front();
        const uint64_t budget = wcfe::engine_budget(s->eng);
        if (budget && wcfe_engine_free_bytes(s->eng) < wcfe_cell_bytes(r->nv, r->nt) && !s->active.empty()) break;
        while (!s->inflight.empty()) {
            int rc = wait_oldest(s);
            if (rc) return rc;
        }
        int rc = admit_with_substrate(s, r);
        if (rc) return rc;
        s->queue.pop_front();
    }
    // with nothing on the device, wait for the head of the queue to be prepared
    if (s->active.empty() && s->inflight.empty())
        while (!s->queue.empty() && s->queue.front()->prep.load(std::memory_order_acquire) == 0)
            std::this_thread::sleep_for(std::chrono::microseconds(50));
    int admitted = 0;
    int rc = admit(s, &admitted);
    if (rc) return rc;
    if (!s->active.empty()) {
        // K steps: about iter_ms of GPU time at the last measured step time
        int k = s->step_ms_est > 0 ? (int)(s->iter_ms / s->step_ms_est) : 1;
        k = std::max(1, std::min(k, s->kmax));
        Iter it;
        it.t0 = get_event(s);
        it.t1 = get_event(s);
        if (!it.t0 || !it.t1) return fail_srv("cudaEventCreate", WCFE_ERR_CUDA);
        it.k = k;
        cudaStream_t st = wcfe::engine_stream(s->eng);
        if (cudaEventRecord(it.t0, st) != cudaSuccess) return fail_srv("cudaEventRecord", WCFE_ERR_CUDA);
        rc = wcfe::serving_step(s->eng, k, s->dt);
        if (rc) return rc;
        // cells whose last step is among these k: results into the ring, blocks freed behind the copy
        std::vector<Req*> keep;
        for (Req* r : s->active) {
            const int adv = std::min(r->left, k);
            r->left -= adv;
            r->done_steps += adv;
            s->cell_steps += (uint64_t)adv;
            if (r->left > 0) {
                keep.push_back(r);
                continue;
            }
            const size_t nb = wcfe::serving_raw_bytes(r->nv);
            size_t off = 0;
            while (!ring_alloc(s, nb, &off)) {
                if (s->inflight.empty()) return fail_srv("result ring too small for one cell", WCFE_ERR_LIMIT);
                if ((rc = wait_oldest(s))) return rc;
            }
            size_t got = 0;
            rc = wcfe::serving_retire(s->eng, r->cell, r->done_steps & 1, s->ring + off, nb, &got);
            if (rc) return rc;
            r->cell = -1;
            r->ring_off = off;
            r->ring_bytes = got;
            it.retired.push_back(r);
        }
        s->active.swap(keep);
        if (cudaEventRecord(it.t1, st) != cudaSuccess) return fail_srv("cudaEventRecord", WCFE_ERR_CUDA);
        s->inflight.push_back(it);
        // at most two iterations in flight: wait for the one before this
        while (s->inflight.size() > 2)
            if ((rc = wait_oldest(s))) return rc;
    } else {
        // nothing resident: drain what is in flight so that results become visible
        while (!s->inflight.empty())
            if ((rc = wait_oldest(s))) return rc;
    }
    if (s->active.empty() && s->queue.empty())
        while (!s->inflight.empty())
            if ((rc = wait_oldest(s))) return rc;
    if (n_active) *n_active = (int32_t)s->active.size();
    if (n_queued) *n_queued = (int32_t)(s->queue.size() + s->inflight.size());
    return WCFE_OK;
}

int wcfe_server_result(wcfe_server* s, int64_t id, double* x_out, double* seconds) {
    if (!s) return fail_srv("bad argument", WCFE_ERR_ARG);
    auto it = s->all.find(id);
    if (it == s->all.end() || !it->second->finished) return fail_srv("request unknown or still running", WCFE_ERR_ARG);
    Req* r = it->second.get();
    if (r->status) return r->status;
    if (x_out) std::memcpy(x_out, r->x_final.data(), sizeof(double) * r->x_final.size());
    if (seconds) *seconds = std::chrono::duration<double>(r->t_done - r->t_submit).count();
    return WCFE_OK;
}

int64_t wcfe_server_step_times(wcfe_server* s, double* out, int64_t cap) {
    if (!s) return -1;
    int64_t n = (int64_t)s->step_times.size();
    if (out)
        for (int64_t i = 0; i < n && i < cap; ++i) out[i] = s->step_times[i];
    return n;
}

int wcfe_server_set_iteration_ms(wcfe_server* s, double ms) {
    if (!s || !(ms > 0)) return fail_srv("bad argument", WCFE_ERR_ARG);
    s->iter_ms = ms;
    return WCFE_OK;
}

uint64_t wcfe_server_cell_steps(const wcfe_server* s) { return s ? s->cell_steps : 0; }

}  // extern "C"
