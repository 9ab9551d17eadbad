// wcfe_server.cu — continuous batching of whole cell simulations on one engine.
//
// Requests (a mesh, its initial positions, parameters and a step count) queue
// on the host.  Each iteration admits queued requests in arrival order while
// the engine's HBM budget has room for them, advances every resident cell by
// one explicit step in one batched launch per phase, and retires the cells
// whose step count is reached (final positions copied back, memory freed for
// the next admissions).  A cell's arithmetic does not depend on which other
// cells share its launches, so each result is the same alone and in the mix.
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "../../include/wcfe.h"

namespace {
using clk = std::chrono::steady_clock;

struct Req {
    int64_t id = 0;
    int32_t nv = 0, nt = 0, steps = 0, done_steps = 0;
    std::vector<int32_t> tri, sub_tri;
    std::vector<double> x, sub_X, x_final;
    int32_t sub_nv = 0, sub_nt = 0;
    wcfe_params prm{};
    int32_t cell = -1;
    bool finished = false;
    clk::time_point t_submit, t_done;
};
}  // namespace

struct wcfe_server {
    wcfe_engine* eng = nullptr;
    double dt = 0;
    int64_t next_id = 0;
    std::deque<Req*> queue;
    std::vector<Req*> active;
    std::map<int64_t, std::unique_ptr<Req>> all;
    std::vector<double> step_times;
};

extern "C" {

int wcfe_server_create(wcfe_engine* eng, double dt, wcfe_server** out) {
    if (!eng || !out || !(dt > 0)) return WCFE_ERR_ARG;
    wcfe_server* s = new wcfe_server();
    s->eng = eng;
    s->dt = dt;
    *out = s;
    return WCFE_OK;
}

int wcfe_server_destroy(wcfe_server* s) {
    if (!s) return WCFE_ERR_ARG;
    for (Req* r : s->active)
        if (r->cell >= 0) wcfe_cell_destroy(s->eng, r->cell);
    delete s;
    return WCFE_OK;
}

int wcfe_server_submit(wcfe_server* s, const wcfe_request* q, int64_t* id) {
    if (!s || !q || !q->tri || !q->x || !q->params || q->n_vert <= 0 || q->n_tri <= 0 || q->n_steps <= 0)
        return WCFE_ERR_ARG;
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
    }
    r->t_submit = clk::now();
    if (id) *id = r->id;
    s->queue.push_back(r.get());
    s->all[r->id] = std::move(r);
    return WCFE_OK;
}

int wcfe_server_iterate(wcfe_server* s, int32_t* n_active, int32_t* n_queued) {
    if (!s) return WCFE_ERR_ARG;
    const auto t0 = clk::now();
    // admission, in arrival order, while the budget has room
    while (!s->queue.empty()) {
        Req* r = s->queue.front();
        uint64_t free = wcfe_engine_free_bytes(s->eng);
        uint64_t need = wcfe_cell_bytes(r->nv, r->nt);
        if (free && need > free && !s->active.empty()) break;
        int32_t id = -1;
        int rc = wcfe_cell_create(s->eng, r->nv, r->nt, r->tri.data(), nullptr, nullptr, nullptr, &r->prm, &id);
        if (rc == WCFE_ERR_BUDGET || rc == WCFE_ERR_NOMEM) {
            if (s->active.empty()) return rc;  // cannot ever fit
            break;
        }
        if (rc) return rc;
        rc = wcfe_cell_set_state(s->eng, id, r->x.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
        if (!rc && r->sub_nt > 0)
            rc = wcfe_cell_set_substrate(s->eng, id, r->sub_nv, r->sub_nt, r->sub_tri.data(), r->sub_X.data(), nullptr);
        if (rc) {
            wcfe_cell_destroy(s->eng, id);
            return rc;
        }
        r->cell = id;
        s->active.push_back(r);
        s->queue.pop_front();
    }
    // one step of every resident cell
    if (!s->active.empty()) {
        int rc = wcfe_engine_step(s->eng, 1, s->dt);
        if (rc) return rc;
    }
    // retire finished cells
    std::vector<Req*> keep;
    for (Req* r : s->active) {
        r->done_steps++;
        if (r->done_steps >= r->steps) {
            r->x_final.assign(3 * (size_t)r->nv, 0.0);
            int rc = wcfe_cell_get_state(s->eng, r->cell, r->x_final.data(), nullptr, nullptr, nullptr, nullptr, nullptr,
                                         nullptr);
            if (rc) return rc;
            wcfe_cell_destroy(s->eng, r->cell);
            r->cell = -1;
            r->finished = true;
            r->t_done = clk::now();
            r->tri.clear();
            r->tri.shrink_to_fit();
            r->x.clear();
            r->x.shrink_to_fit();
        } else {
            keep.push_back(r);
        }
    }
    s->active.swap(keep);
    int rc = wcfe_engine_sync(s->eng);
    if (rc) return rc;
    s->step_times.push_back(std::chrono::duration<double>(clk::now() - t0).count());
    if (n_active) *n_active = (int32_t)s->active.size();
    if (n_queued) *n_queued = (int32_t)s->queue.size();
    return WCFE_OK;
}

int wcfe_server_result(wcfe_server* s, int64_t id, double* x_out, double* seconds) {
    if (!s) return WCFE_ERR_ARG;
    auto it = s->all.find(id);
    if (it == s->all.end() || !it->second->finished) return WCFE_ERR_ARG;
    Req* r = it->second.get();
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

}  // extern "C"
