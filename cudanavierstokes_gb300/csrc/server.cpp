// server.cpp -- request loop for "advance N steps" solves with continuous batching.
//
// Clients submit (parameters, initial fields, N) from any thread. One worker thread owns
// the GPU batch: between steps it admits queued requests in arrival order while the HBM
// budget allows (cns_batch_add fails with CNS_ERR_OOM otherwise and the request waits),
// advances every resident simulation by one step (the batch's concurrent mode: each
// member's step graph on one of the batch's streams, so their kernels overlap), and
// retires the ones that reached their N: their fields are copied to host
// memory, their device memory is released and their latency (submit -> result ready) is
// recorded. State stays on the device for the whole life of a request.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cns.h"
#include "solver_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    cns_params p{};
    int nsteps = 0;
    std::vector<double> in[5];
    std::vector<double> out[5];
    int state = CNS_REQ_QUEUED;
    int err = CNS_OK;
    std::string msg;
    int member = -1;
    Clock::time_point t_submit, t_admit, t_done;
};

}  // namespace

struct cns_server {
    cns_batch* batch = nullptr;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::map<int64_t, std::shared_ptr<Request>> all;
    std::vector<std::shared_ptr<Request>> running;
    int64_t next_id = 1;
    bool stop = false;
    std::thread worker;
    // statistics
    int64_t point_steps = 0, steps_done = 0, completed = 0;
    Clock::time_point t_first{}, t_last{};
    bool any = false;
    std::vector<double> latencies;
    int max_batch = CNS_BATCH_MAX;

    void loop();
};

namespace {

void finish(cns_server* s, const std::shared_ptr<Request>& r) {
    const size_t N = (size_t)r->p.mx * r->p.my * r->p.mz;
    for (int f = 0; f < 5; f++) r->out[f].resize(N);
    int rc = cns_batch_get_fields(s->batch, r->member, r->out[0].data(), r->out[1].data(), r->out[2].data(),
                                  r->out[3].data(), r->out[4].data());
    cns_batch_remove(s->batch, r->member);
    std::lock_guard<std::mutex> lk(s->mu);
    r->t_done = Clock::now();
    r->state = rc ? CNS_REQ_FAILED : CNS_REQ_DONE;
    r->err = rc;
    if (rc) r->msg = cns_last_error();
    if (!rc) {
        s->completed++;
        s->latencies.push_back(std::chrono::duration<double>(r->t_done - r->t_submit).count());
    }
    s->t_last = r->t_done;
    for (int f = 0; f < 5; f++) { r->in[f].clear(); r->in[f].shrink_to_fit(); }
}

}  // namespace

void cns_server::loop() {
    cudaSetDevice(device);
    for (;;) {
        // ---- admission at the step boundary ----
        std::vector<std::shared_ptr<Request>> admit;
        {
            std::unique_lock<std::mutex> lk(mu);
            if (running.empty())
                cv_work.wait(lk, [&] { return stop || !queue.empty(); });
            if (stop) break;
            while (!queue.empty() && (int)(running.size() + admit.size()) < max_batch) {
                admit.push_back(queue.front());
                queue.pop_front();
            }
        }
        std::vector<std::shared_ptr<Request>> deferred;
        for (auto& r : admit) {
            int id = -1;
            int rc = cns_batch_add(batch, &r->p, r->in[0].data(), r->in[1].data(), r->in[2].data(),
                                   r->in[3].data(), r->in[4].data(), r->nsteps + 1, &id);
            std::lock_guard<std::mutex> lk(mu);
            if (rc == CNS_ERR_OOM && !running.empty()) {
                deferred.push_back(r);          // no room yet: wait for a retirement
            } else if (rc) {
                r->state = CNS_REQ_FAILED;
                r->err = rc;
                r->msg = cns_last_error();
                r->t_done = Clock::now();
            } else {
                r->member = id;
                r->state = CNS_REQ_RUNNING;
                r->t_admit = Clock::now();
                if (!any) { t_first = r->t_admit; any = true; }
                running.push_back(r);
            }
        }
        if (!deferred.empty()) {
            std::lock_guard<std::mutex> lk(mu);
            for (auto it = deferred.rbegin(); it != deferred.rend(); ++it) queue.push_front(*it);
        }
        cv_done.notify_all();
        if (running.empty()) continue;
        // ---- one step for every resident simulation ----
        int rc = cns_batch_step(batch, 1);
        if (rc) {
            std::lock_guard<std::mutex> lk(mu);
            for (auto& r : running) {
                r->state = CNS_REQ_FAILED;
                r->err = rc;
                r->msg = cns_last_error();
                r->t_done = Clock::now();
                cns_batch_remove(batch, r->member);
            }
            running.clear();
            cv_done.notify_all();
            continue;
        }
        int64_t pts = 0;
        for (auto& r : running) pts += (int64_t)r->p.mx * r->p.my * r->p.mz;
        {
            std::lock_guard<std::mutex> lk(mu);
            point_steps += pts;
            steps_done++;
        }
        // ---- retire the finished ones ----
        std::vector<std::shared_ptr<Request>> still;
        for (auto& r : running) {
            int64_t st = 0;
            cns_batch_member_steps(batch, r->member, &st);
            if (st >= r->nsteps) finish(this, r);
            else still.push_back(r);
        }
        {
            // every change of `running` holds the lock: cns_server_stats reads its size
            std::lock_guard<std::mutex> lk(mu);
            running.swap(still);
        }
        cv_done.notify_all();
    }
}

extern "C" {

int cns_server_create(int device, int precision, int stencil_size, int stencil_visc, int64_t hbm_budget_bytes,
                      int max_batch, cns_server** out) {
    if (!out) return cns::set_error(CNS_ERR_INVALID, "out is NULL");
    *out = nullptr;
    cns_batch* b = nullptr;
    int rc = cns_batch_create(device, precision, stencil_size, stencil_visc, hbm_budget_bytes, &b);
    if (rc) return rc;
    cns_batch_set_mode(b, CNS_BATCH_CONCURRENT);
    cns_server* s = new cns_server();
    s->batch = b;
    s->device = device;
    if (max_batch > 0 && max_batch < CNS_BATCH_MAX) s->max_batch = max_batch;
    s->worker = std::thread([s] { s->loop(); });
    *out = s;
    return CNS_OK;
}

int cns_server_destroy(cns_server* s) {
    if (!s) return CNS_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cns_batch_destroy(s->batch);
    delete s;
    return CNS_OK;
}

int cns_server_submit(cns_server* s, const cns_params* p, const double* r, const double* u, const double* v,
                      const double* w, const double* e, int nsteps, int64_t* req_id) {
    if (!s || !p || !r || !u || !v || !w || !e || !req_id) return cns::set_error(CNS_ERR_INVALID, "NULL argument");
    if (nsteps < 1) return cns::set_error(CNS_ERR_INVALID, "nsteps must be >= 1");
    int rc = cns_check_params(p);
    if (rc) return rc;
    auto q = std::make_shared<Request>();
    q->p = *p;
    q->nsteps = nsteps;
    const size_t N = (size_t)p->mx * p->my * p->mz;
    const double* src[5] = {r, u, v, w, e};
    for (int f = 0; f < 5; f++) q->in[f].assign(src[f], src[f] + N);
    q->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        q->id = s->next_id++;
        s->all[q->id] = q;
        s->queue.push_back(q);
        *req_id = q->id;
    }
    s->cv_work.notify_all();
    return CNS_OK;
}

int cns_server_poll(cns_server* s, int64_t req_id, int* state, double* latency_s) {
    if (!s) return cns::set_error(CNS_ERR_INVALID, "server is NULL");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(req_id);
    if (it == s->all.end()) return cns::set_error(CNS_ERR_INVALID, "unknown request id");
    if (state) *state = it->second->state;
    if (latency_s)
        *latency_s = it->second->state == CNS_REQ_DONE
                         ? std::chrono::duration<double>(it->second->t_done - it->second->t_submit).count()
                         : -1.0;
    return CNS_OK;
}

int cns_server_wait(cns_server* s, int64_t req_id, double timeout_s, double* r, double* u, double* v, double* w,
                    double* e) {
    if (!s) return cns::set_error(CNS_ERR_INVALID, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(req_id);
    if (it == s->all.end()) return cns::set_error(CNS_ERR_INVALID, "unknown request id");
    auto q = it->second;
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
        return q->state == CNS_REQ_DONE || q->state == CNS_REQ_FAILED;
    });
    if (!ok) return cns::set_error(CNS_ERR_TIMEOUT, "request not finished within the timeout");
    if (q->state == CNS_REQ_FAILED) return cns::set_error(q->err ? q->err : CNS_ERR_STATE, q->msg.c_str());
    double* dst[5] = {r, u, v, w, e};
    for (int f = 0; f < 5; f++)
        if (dst[f]) std::memcpy(dst[f], q->out[f].data(), q->out[f].size() * sizeof(double));
    s->all.erase(it);
    return CNS_OK;
}

int cns_server_stats(cns_server* s, cns_server_stats_t* st) {
    if (!s || !st) return cns::set_error(CNS_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(st, 0, sizeof *st);
    st->completed = s->completed;
    st->queued = (int64_t)s->queue.size();
    st->running = (int64_t)s->running.size();
    st->batch_steps = s->steps_done;
    st->point_steps = s->point_steps;
    st->busy_seconds = s->any ? std::chrono::duration<double>(s->t_last - s->t_first).count() : 0.0;
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
        if (l.empty()) return 0.0;
        size_t idx = (size_t)std::ceil(q * l.size()) - 1;
        if (idx >= l.size()) idx = l.size() - 1;
        return l[idx];
    };
    st->p50_s = pct(0.50);
    st->p99_s = pct(0.99);
    st->max_s = l.empty() ? 0.0 : l.back();
    return CNS_OK;
}

}  // extern "C"
