// dgx_server.cpp -- continuous batching of solve requests on one GPU.
//
// New, no counterpart in the reference (which runs one solve per process).
// Clients submit solve requests (mesh spec, order, equation, initial
// condition, end time) at any time.  A worker thread admits queued requests
// while the device-memory budget and the slot limit allow.  It creates their
// solvers, whose state then stays resident on the device, and repacks the
// active set into a batch (per-class work lists + a CUDA-graph step) whenever
// solves join or finish.  It then advances the batch a few steps at a time,
// gathers every solve's time in one copy, and retires the solves that reached
// their end time, recording time-to-solution.  Requests that arrive while
// others run join at the next repack, so their work overlaps on the device.
// Each solve's result is the same alone and in the mix (the batched kernels are
// bitwise equal to the plain path).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <vector>

#include "dgx_internal.h"

namespace dgx {
namespace {

using Clock = std::chrono::steady_clock;

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2, kFailed = 3, kCancelled = 4 };

struct Request {
    long long id = 0;
    dgx_request r{};
    int state = kQueued;
    int status = DGX_OK;
    Clock::time_point submitted, started, finished;
    size_t bytes = 0;
    dgx_mesh *mesh = nullptr;
    dgx_solver *solver = nullptr;
    std::vector<double> result;      // final state (keep_state), reference layout
    double totals[4] = {0, 0, 0, 0};
    double t_final = 0.0;
    long long steps = 0, dofs = 0;
    bool cancel = false;
};

using MeshKey = std::tuple<int, double, double, double, unsigned long long>;

size_t estimate_bytes(const dgx_request &r, bool mesh_cached) {
    const size_t E = 2 * static_cast<size_t>(r.n) * r.n, S = 3 * static_cast<size_t>(r.n) * r.n;
    const size_t np = static_cast<size_t>(num_modes(r.order)), nv = r.equation == DGX_EULER ? 4 : 1;
    const size_t vb = r.precision == DGX_FP64 ? 8 : 4;
    size_t mesh = E * (6 * 8 + 3 * 4 + 6 * 8 + 3 * 4 + 5 * 4 + 9 * 4 + 5 * 8 + 9 * 8 + 4) + S * (4 * 4 + 3 * 8);
    return (mesh_cached ? 0 : mesh) + 4 * nv * np * E * vb + 4096;
}

}  // namespace
}  // namespace dgx

using namespace dgx;

struct dgx_server {
    size_t budget = 0, in_use = 0;
    int max_active = 0;
    int device = 0;
    std::mutex mu;
    std::condition_variable cv, idle_cv;
    std::deque<Request *> queue;
    std::map<long long, Request *> all;
    std::vector<Request *> active;
    int in_transit = 0;   // admitted, out of the queue, not yet active or finished
    std::map<MeshKey, dgx_mesh *> meshes;     // shared meshes (refcounted by their solvers)
    std::vector<double> latencies;
    long long next_id = 1, submitted = 0, completed = 0, failed = 0, repacks = 0, steps = 0;
    double dof_updates = 0.0, busy = 0.0;
    bool stop = false;
    std::thread worker;
    dgx_batch *batch = nullptr;
    cudaStream_t stream = nullptr;
    int steps_per_check = 8;
    double stall_seconds = 0.0;   // test hook: the worker sleeps this long per check
};

namespace dgx {
namespace {

int validate(const dgx_request &r) {
    if (r.n < 1 || r.n > 8192) return DGX_ERR_INVALID;
    if (r.order < 0 || r.order > kMaxOrder) return DGX_ERR_UNSUPPORTED;
    if (r.equation != DGX_ADVECTION && r.equation != DGX_EULER) return DGX_ERR_INVALID;
    if (r.precision != DGX_FP32 && r.precision != DGX_FP64) return DGX_ERR_UNSUPPORTED;
    if (!(r.t_end > 0.0) || !(r.lx > 0.0) || !(r.ly > 0.0)) return DGX_ERR_INVALID;
    if (r.dt <= 0.0 && !(r.cfl > 0.0)) return DGX_ERR_INVALID;
    return DGX_OK;
}

void release_solve(dgx_server *s, Request *q) {
    if (q->solver) dgx_solver_destroy(q->solver);
    q->solver = nullptr;
    q->mesh = nullptr;   // owned by the mesh cache
    s->in_use -= std::min(s->in_use, q->bytes);
}

// create the solver of a request (worker thread, lock not held)
int start_solve(dgx_server *s, Request *q, dgx_mesh *mesh) {
    dgx_solver_desc d;
    d.order = q->r.order;
    d.equation = q->r.equation;
    d.flux = q->r.flux;
    d.precision = q->r.precision;
    d.integrator = DGX_RK4;
    d.gamma = q->r.gamma;
    d.ax = q->r.ax;
    d.ay = q->r.ay;
    int rc = dgx_solver_create(mesh, &d, &q->solver);
    if (!rc) rc = dgx_project_ic(q->solver, q->r.ic, q->r.params);
    if (!rc) rc = q->r.dt > 0.0 ? dgx_set_dt(q->solver, DGX_DT_FIXED, q->r.dt, 0.7)
                                : dgx_set_dt(q->solver, DGX_DT_CFL, 0.0, q->r.cfl);
    if (!rc) rc = dgx_set_end_time(q->solver, q->r.t_end);
    if (!rc) {
        int nv = 0, np = 0;
        dgx_solver_info(q->solver, &nv, &np, nullptr, nullptr);
        q->dofs = static_cast<long long>(nv) * np * 2LL * q->r.n * q->r.n;
    }
    (void)s;
    return rc;
}

dgx_mesh *cached_mesh(dgx_server *s, const dgx_request &r, int *rc) {
    const MeshKey key{r.n, r.lx, r.ly, r.jitter, r.seed};
    auto it = s->meshes.find(key);
    if (it != s->meshes.end()) return it->second;
    dgx_mesh *m = nullptr;
    *rc = dgx_mesh_create_periodic_square(r.n, r.lx, r.ly, 0.0, 0.0, r.jitter, r.seed, &m);
    if (*rc) return nullptr;
    s->meshes[key] = m;
    return m;
}

void finish(dgx_server *s, Request *q, int state, int status) {
    q->state = state;
    q->status = status;
    q->finished = Clock::now();
    if (state == kDone) {
        s->completed++;
        s->latencies.push_back(std::chrono::duration<double>(q->finished - q->submitted).count());
    } else if (state == kFailed) {
        s->failed++;
    }
}

void worker_main(dgx_server *s) {
    cudaSetDevice(s->device);
    cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    std::vector<double> t, dt;
    std::vector<unsigned int> st;
    std::vector<long long> stp;
    for (;;) {
        bool changed = false;
        std::vector<Request *> admit;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->active.empty() && s->queue.empty() && !s->stop) {
                s->idle_cv.notify_all();
                s->cv.wait(lk, [&] { return s->stop || !s->queue.empty(); });
            }
            if (s->stop) break;
            // admission by device-memory footprint and slot count, in arrival order
            while (!s->queue.empty() && static_cast<int>(s->active.size() + admit.size()) < s->max_active) {
                Request *q = s->queue.front();
                if (q->cancel) {
                    s->queue.pop_front();
                    q->state = kCancelled;
                    continue;
                }
                const MeshKey key{q->r.n, q->r.lx, q->r.ly, q->r.jitter, q->r.seed};
                const size_t need = estimate_bytes(q->r, s->meshes.count(key) > 0);
                if (s->in_use + need > s->budget && !(s->active.empty() && admit.empty())) break;
                s->queue.pop_front();
                q->bytes = need;
                s->in_use += need;
                admit.push_back(q);
                s->in_transit++;
            }
        }
        for (Request *q : admit) {
            int rc = DGX_OK;
            dgx_mesh *m = cached_mesh(s, q->r, &rc);   // the cache is the worker's alone
            if (!rc) rc = start_solve(s, q, m);
            std::lock_guard<std::mutex> lk(s->mu);
            s->in_transit--;
            if (rc) {
                release_solve(s, q);
                finish(s, q, kFailed, rc);
            } else {
                q->state = kRunning;
                q->started = Clock::now();
                s->active.push_back(q);
                changed = true;
            }
        }
        if (s->active.empty()) continue;
        // repack the active set into one batch
        if (changed || !s->batch) {
            if (s->batch) dgx_batch_destroy(s->batch);
            s->batch = nullptr;
            std::vector<dgx_solver *> sv;
            for (Request *q : s->active) sv.push_back(q->solver);
            int rc = dgx_batch_create(sv.data(), static_cast<int>(sv.size()), &s->batch);
            s->repacks++;
            if (rc) {
                std::lock_guard<std::mutex> lk(s->mu);
                for (Request *q : s->active) { release_solve(s, q); finish(s, q, kFailed, rc); }
                s->active.clear();
                continue;
            }
        }
        const auto t0 = Clock::now();
        dgx_batch_run(s->batch, s->steps_per_check, s->stream);
        const size_t n = s->active.size();
        t.resize(n); dt.resize(n); st.resize(n); stp.resize(n);
        int rc = dgx_batch_progress(s->batch, t.data(), dt.data(), st.data(), stp.data(), s->stream);
        if (s->stall_seconds > 0.0)   // host-side fault injection: a stalled worker
            std::this_thread::sleep_for(std::chrono::duration<double>(s->stall_seconds));
        const auto t1 = Clock::now();
        std::vector<Request *> keep;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->busy += std::chrono::duration<double>(t1 - t0).count();
            s->steps += s->steps_per_check;
            for (size_t i = 0; i < n; ++i) {
                Request *q = s->active[i];
                const long long done_steps = rc == DGX_OK ? stp[i] : q->steps;
                s->dof_updates += static_cast<double>(done_steps - q->steps) * q->dofs;
                q->steps = done_steps;
                const bool bad = rc != DGX_OK || st[i] != 0;
                const bool done = !bad && (t[i] >= q->r.t_end || dt[i] == 0.0);
                if (bad || done || q->cancel) {
                    if (done) {
                        dgx_conserved_totals(q->solver, q->totals, s->stream);
                        q->t_final = t[i];
                        if (q->r.keep_state) {
                            q->result.resize(q->solver->s.n);
                            dgx_get_state(q->solver, q->result.data());
                        }
                    }
                    release_solve(s, q);
                    if (q->cancel && !done) q->state = kCancelled;
                    else finish(s, q, done ? kDone : kFailed, done ? DGX_OK : DGX_ERR_NONFINITE);
                } else {
                    keep.push_back(q);
                }
            }
            if (keep.size() != n) {
                s->active.swap(keep);
                if (s->batch) dgx_batch_destroy(s->batch);
                s->batch = nullptr;
            }
        }
    }
    if (s->batch) dgx_batch_destroy(s->batch);
    s->batch = nullptr;
    for (Request *q : s->active) release_solve(s, q);
    s->active.clear();
    for (auto &kv : s->meshes) dgx_mesh_destroy(kv.second);
    s->meshes.clear();
    cudaStreamDestroy(s->stream);
}

}  // namespace
}  // namespace dgx

extern "C" {

int dgx_server_create(size_t budget_bytes, int max_active, dgx_server **out) {
    if (!out || budget_bytes == 0 || max_active <= 0) { set_error("need a budget and max_active > 0"); return DGX_ERR_INVALID; }
    dgx_server *s = new (std::nothrow) dgx_server();
    if (!s) { set_error("host allocation failed"); return DGX_ERR_NOMEM; }
    s->budget = budget_bytes;
    s->max_active = max_active;
    cudaGetDevice(&s->device);
    s->worker = std::thread(worker_main, s);
    *out = s;
    return DGX_OK;
}

int dgx_server_submit(dgx_server *s, const dgx_request *r, long long *id) {
    if (!s || !r) { set_error("NULL argument"); return DGX_ERR_INVALID; }
    int rc = validate(*r);
    if (rc) { set_error("invalid request"); return rc; }
    if (estimate_bytes(*r, false) > s->budget) { set_error("request needs more device memory than the budget"); return DGX_ERR_BUSY; }
    Request *q = new (std::nothrow) Request();
    if (!q) { set_error("host allocation failed"); return DGX_ERR_NOMEM; }
    q->r = *r;
    q->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        q->id = s->next_id++;
        s->all[q->id] = q;
        s->queue.push_back(q);
        s->submitted++;
    }
    s->cv.notify_one();
    if (id) *id = q->id;
    return DGX_OK;
}

int dgx_server_status(dgx_server *s, long long id, int *state, double *latency_s) {
    if (!s) return DGX_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) { set_error("unknown request %lld", id); return DGX_ERR_NOT_FOUND; }
    Request *q = it->second;
    if (state) *state = q->state;
    if (latency_s)
        *latency_s = (q->state == kDone || q->state == kFailed)
                         ? std::chrono::duration<double>(q->finished - q->submitted).count()
                         : -1.0;
    return q->state == kFailed ? q->status : DGX_OK;
}

int dgx_server_result(dgx_server *s, long long id, double *c, size_t c_len, double *totals, int *steps,
                      double *t_final) {
    if (!s) return DGX_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) { set_error("unknown request %lld", id); return DGX_ERR_NOT_FOUND; }
    Request *q = it->second;
    if (q->state != kDone) { set_error("request %lld has not finished", id); return q->state == kFailed ? q->status : DGX_ERR_BUSY; }
    if (c) {
        if (q->result.empty() || c_len < q->result.size()) { set_error("state not kept or buffer too small"); return DGX_ERR_INVALID; }
        std::memcpy(c, q->result.data(), q->result.size() * sizeof(double));
    }
    if (totals) std::memcpy(totals, q->totals, sizeof(q->totals));
    if (steps) *steps = static_cast<int>(q->steps);
    if (t_final) *t_final = q->t_final;
    return DGX_OK;
}

int dgx_server_cancel(dgx_server *s, long long id) {
    if (!s) return DGX_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) { set_error("unknown request %lld", id); return DGX_ERR_NOT_FOUND; }
    it->second->cancel = true;
    return DGX_OK;
}

int dgx_server_release(dgx_server *s, long long id) {
    if (!s) return DGX_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return DGX_ERR_NOT_FOUND;
    Request *q = it->second;
    if (q->state == kQueued || q->state == kRunning) { set_error("request %lld is still live", id); return DGX_ERR_BUSY; }
    delete q;
    s->all.erase(it);
    return DGX_OK;
}

int dgx_server_wait_idle(dgx_server *s, double timeout_s) {
    if (!s) return DGX_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->idle_cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return s->queue.empty() && s->active.empty() && s->in_transit == 0; });
    if (!ok) { set_error("server still busy after %.1f s", timeout_s); return DGX_ERR_TIMEOUT; }
    return DGX_OK;
}

int dgx_server_get_stats(dgx_server *s, dgx_server_stats *out) {
    if (!s || !out) return DGX_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->active = static_cast<long long>(s->active.size());
    out->queued = static_cast<long long>(s->queue.size());
    out->dof_updates = s->dof_updates;
    out->busy_seconds = s->busy;
    out->repacks = s->repacks;
    out->steps = s->steps;
    out->device_bytes_in_use = s->in_use;
    if (!s->latencies.empty()) {
        std::vector<double> l = s->latencies;
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) {
            const size_t i = std::min(l.size() - 1, static_cast<size_t>(p * (l.size() - 1) + 0.5));
            return l[i];
        };
        out->p50_latency_s = pct(0.50);
        out->p99_latency_s = pct(0.99);
        out->max_latency_s = l.back();
    }
    return DGX_OK;
}

int dgx_server_set_steps_per_check(dgx_server *s, int k) {
    if (!s || k <= 0) return DGX_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    s->steps_per_check = k;
    return DGX_OK;
}

int dgx_server_inject_stall(dgx_server *s, double seconds) {
    if (!s || seconds < 0) return DGX_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    s->stall_seconds = seconds;
    return DGX_OK;
}

int dgx_server_destroy(dgx_server *s) {
    if (!s) return DGX_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (auto &kv : s->all) delete kv.second;
    delete s;
    return DGX_OK;
}

}  // extern "C"
