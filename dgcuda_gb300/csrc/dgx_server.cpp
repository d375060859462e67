// dgx_server.cpp -- continuous batching of solve requests on one GPU.
//
// New, no counterpart in the reference (which runs one solve per process).
// Clients submit solve requests (mesh spec, order, equation, initial
// condition, end time) at any time.  A worker thread admits queued requests
// while the device-memory budget and the slot limit allow.  It creates their
// solvers, whose state then stays resident on the device, and repacks the
// active set into a batch (per-class work lists + a CUDA-graph step) whenever
// solves join or finish.  It advances the batch a few steps at a time, and
// while the GPU runs those steps it admits the next requests (their meshes
// are generated and checked on the host meanwhile; their uploads and
// projections queue behind the steps); then it gathers every solve's time in
// one copy, and retires the solves that reached their end time, recording
// time-to-solution.  Requests that arrive while
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
#include <set>
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

// device footprint of a request's mesh and solver blocks (their size classes)
size_t mesh_estimate(const dgx_request &r) {
    const size_t E = 2 * static_cast<size_t>(r.n) * r.n, S = 3 * static_cast<size_t>(r.n) * r.n;
    const size_t red = std::min<size_t>((E + 255) / 256, kReduceLen) + 1;
    const size_t mesh = E * (6 * 8 + 3 * 4 + 6 * 8 + 3 * 4 + 5 * 4 + 9 * 4 + 5 * 8 + 9 * 8 + 4) +
                        S * (4 * 4 + 3 * 8) + red * 8 + 20 * 256;
    return BlockPool::size_class(mesh);
}
size_t solver_estimate(const dgx_request &r) {
    const size_t E = 2 * static_cast<size_t>(r.n) * r.n;
    const size_t np = static_cast<size_t>(num_modes(r.order)), nv = r.equation == DGX_EULER ? 4 : 1;
    const size_t vb = r.precision == DGX_FP64 ? 8 : 4;
    const size_t nvec = r.precision == DGX_FP32_COMP ? 5 : 4;   // c, ua, ub, acc (+ lo)
    return BlockPool::size_class(nvec * (nv * np * E * vb + 64 + 256) + 256);
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
    // shared meshes, refcounted by their solvers; meshes no running solve uses
    // stay cached (least recently used first out) while the budget allows
    struct CachedMesh {
        dgx_mesh *mesh = nullptr;
        size_t bytes = 0;
        long long last_use = 0;
    };
    std::map<MeshKey, CachedMesh> meshes;
    size_t mesh_bytes = 0;   // footprint of the cached meshes, counted against the budget
    long long use_tick = 0;
    dgx::BlockPool *pool = nullptr;   // mesh and solver blocks, recycled
    double *red = nullptr;            // conserved-total scratch: terms, partials, sums
    size_t red_elems = 0, red_solves = 0;
    std::vector<double> sums;
    // pinned host memory of an admission round: mesh uploads (bump-allocated,
    // reused once the stream has passed them) and the meshes' minimum diameters
    unsigned char *stage = nullptr;
    size_t stage_cap = 0, stage_off = 0;
    double *min_diam = nullptr;
    size_t min_diam_cap = 0;
    std::vector<double> latencies;
    long long next_id = 1, submitted = 0, completed = 0, failed = 0, repacks = 0, steps = 0;
    double dof_updates = 0.0, busy = 0.0;
    double admit_s = 0.0, repack_s = 0.0, retire_s = 0.0, idle_s = 0.0;   // worker time by phase
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
    if (r.precision != DGX_FP32 && r.precision != DGX_FP64 && r.precision != DGX_FP32_COMP) return DGX_ERR_UNSUPPORTED;
    if (!(r.t_end > 0.0) || !(r.lx > 0.0) || !(r.ly > 0.0)) return DGX_ERR_INVALID;
    if (r.dt <= 0.0 && !(r.cfl > 0.0)) return DGX_ERR_INVALID;
    return DGX_OK;
}

void release_solve(dgx_server *s, Request *q) {
    if (q->solver) dgx_solver_destroy(q->solver);   // its blocks go back to the pool
    q->solver = nullptr;
    q->mesh = nullptr;   // owned by the mesh cache
    s->in_use -= std::min(s->in_use, q->bytes);
}

MeshKey mesh_key(const dgx_request &r) { return MeshKey{r.n, r.lx, r.ly, r.jitter, r.seed}; }

// Drop cached meshes that no running solve uses, least recently used first,
// until `free_target` bytes of the budget are free or only `keep_idle` idle
// meshes remain (lock held; keys in `pinned` are about to be used).
void evict_idle_meshes(dgx_server *s, size_t free_target, size_t keep_idle, const std::set<MeshKey> &pinned) {
    std::vector<std::pair<long long, MeshKey>> idle;
    for (auto &kv : s->meshes)
        if (kv.second.mesh && kv.second.mesh->refs.load() == 1 && !pinned.count(kv.first))
            idle.emplace_back(kv.second.last_use, kv.first);
    std::sort(idle.begin(), idle.end());
    size_t left = idle.size();
    for (auto &it : idle) {
        const bool room = s->in_use + s->mesh_bytes + free_target <= s->budget;
        if (room && left <= keep_idle) break;
        auto m = s->meshes.find(it.second);
        s->mesh_bytes -= std::min(s->mesh_bytes, m->second.bytes);
        dgx_mesh_destroy(m->second.mesh);
        s->meshes.erase(m);
        --left;
    }
}

// pinned staging for one mesh upload of the current admission round
unsigned char *stage_bytes(dgx_server *s, size_t bytes) {
    bytes = (bytes + 255) & ~static_cast<size_t>(255);
    if (s->stage_off + bytes > s->stage_cap) {
        if (cudaStreamSynchronize(s->stream) != cudaSuccess) return nullptr;   // the arena's copies are done
        s->stage_off = 0;
        if (bytes > s->stage_cap) {
            if (s->stage) cudaFreeHost(s->stage);
            s->stage = nullptr;
            s->stage_cap = 0;
            const size_t cap = std::max(bytes, static_cast<size_t>(16) << 20);
            if (cudaMallocHost(&s->stage, cap) != cudaSuccess) {
                cudaGetLastError();
                s->stage = nullptr;
                return nullptr;   // the build falls back to a pageable copy
            }
            s->stage_cap = cap;
        }
    }
    unsigned char *p = s->stage + s->stage_off;
    s->stage_off += bytes;
    return p;
}

// the request's mesh, from the cache or built (worker thread, lock not held;
// the cache entry and its bytes were reserved at admission).  A mesh built here
// gets its minimum diameter at the round's synchronisation: its slot is
// appended to `fresh`.
dgx_mesh *cached_mesh(dgx_server *s, const dgx_request &r, int *rc,
                      std::vector<std::pair<dgx_mesh *, size_t>> &fresh) {
    const MeshKey key = mesh_key(r);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->meshes.find(key);
        if (it != s->meshes.end() && it->second.mesh) {
            it->second.last_use = ++s->use_tick;
            return it->second.mesh;
        }
    }
    const size_t E = 2 * static_cast<size_t>(r.n) * r.n, S = 3 * static_cast<size_t>(r.n) * r.n;
    std::vector<double> V(6 * E);
    std::vector<int> es(3 * E), sd(4 * S);
    dgx_mesh *m = nullptr;
    *rc = periodic_square_arrays(r.n, r.lx, r.ly, 0.0, 0.0, r.jitter, r.seed, V.data(), es.data(), sd.data());
    if (!*rc) {
        const double *Vs[6] = {V.data(), V.data() + E, V.data() + 2 * E, V.data() + 3 * E, V.data() + 4 * E, V.data() + 5 * E};
        const int *ep[3] = {es.data(), es.data() + E, es.data() + 2 * E};
        const int *sp[4] = {sd.data(), sd.data() + S, sd.data() + 2 * S, sd.data() + 3 * S};
        MeshBuildAsync as;
        as.stage = [s](size_t bytes) { return stage_bytes(s, bytes); };
        as.min_diam = fresh.size() < s->min_diam_cap ? s->min_diam + fresh.size() : nullptr;
        *rc = mesh_build(static_cast<int>(E), static_cast<int>(S), Vs, ep, sp, s->pool, s->stream,
                         as.min_diam ? &as : nullptr, &m);
        if (!*rc && as.min_diam) fresh.emplace_back(m, fresh.size());
    }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->meshes.find(key);
    if (*rc) {
        if (it != s->meshes.end() && !it->second.mesh) {   // give the reservation back
            s->mesh_bytes -= std::min(s->mesh_bytes, it->second.bytes);
            s->meshes.erase(it);
        }
        return nullptr;
    }
    if (it == s->meshes.end()) {
        it = s->meshes.emplace(key, dgx_server::CachedMesh{}).first;
        it->second.bytes = mesh_estimate(r);
        s->mesh_bytes += it->second.bytes;
    }
    it->second.mesh = m;
    it->second.last_use = ++s->use_tick;
    return m;
}

// create the solver of a request (worker thread, lock not held): block from the
// pool, initial scalars (dt rule, cfl, end time) and the projected initial
// condition queued on the server's stream, no host synchronisation
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
    const bool fixed = q->r.dt > 0.0;
    // device scalars: [3] fixed dt, [4] cfl, [5] t_end (the values dgx_set_dt and
    // dgx_set_end_time write)
    const double scal[8] = {0.0, 0.0, 0.0, fixed ? q->r.dt : 0.0, fixed ? 0.7 : q->r.cfl, q->r.t_end, 0.0, 0.0};
    int rc = solver_build(mesh, &d, s->pool, scal, s->stream, &q->solver);
    if (!rc) {
        q->solver->s.dt_mode = fixed ? DGX_DT_FIXED : DGX_DT_CFL;
        rc = project_ic_on(q->solver, q->r.ic, q->r.params, s->stream);
    }
    if (!rc) {
        int nv = 0, np = 0;
        dgx_solver_info(q->solver, &nv, &np, nullptr, nullptr);
        q->dofs = static_cast<long long>(nv) * np * 2LL * q->r.n * q->r.n;
    }
    return rc;
}

// Conserved totals of finished solves: all their reductions queued on the
// server's stream, one copy back (the same kernels, grid and order as
// dgx_conserved_totals, so the same bits).
int retire_totals(dgx_server *s, const std::vector<Request *> &done) {
    if (done.empty()) return DGX_OK;
    size_t emax = 0;
    for (Request *q : done) emax = std::max(emax, static_cast<size_t>(q->solver->mesh->d.num_elem));
    if (emax > s->red_elems || done.size() > s->red_solves) {
        if (s->red) cudaFree(s->red);   // the stream is idle here
        s->red = nullptr;
        s->red_elems = std::max(emax, s->red_elems);
        s->red_solves = std::max(done.size(), s->red_solves);
        const size_t n = s->red_elems + kReduceLen + 1 + 4 * s->red_solves;
        if (cudaMalloc(&s->red, n * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            s->red = nullptr;
            s->red_elems = s->red_solves = 0;
            set_error("conserved-total scratch allocation failed");
            return DGX_ERR_NOMEM;
        }
    }
    double *terms = s->red, *partials = s->red + s->red_elems, *sums = partials + kReduceLen + 1;
    for (size_t j = 0; j < done.size(); ++j) {
        const dgx_solver *sv = done[j]->solver;
        int rc = conserved_sums_async(sv->s, sv->mesh->d, terms, partials, sums + 4 * j, s->stream);
        if (rc) return rc;
    }
    s->sums.resize(4 * done.size());
    DGX_TRY_CUDA(cudaMemcpyAsync(s->sums.data(), sums, sizeof(double) * 4 * done.size(), cudaMemcpyDeviceToHost,
                                 s->stream));
    DGX_TRY_CUDA(cudaStreamSynchronize(s->stream));
    for (size_t j = 0; j < done.size(); ++j) {
        Request *q = done[j];
        const double phi0 = tables(q->solver->s.order).phi[0];
        for (int n = 0; n < q->solver->s.nv; ++n) q->totals[n] = s->sums[4 * j + n] * phi0 * 0.5;
    }
    return DGX_OK;
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

constexpr size_t kIdleMeshes = 32;   // idle meshes kept for requests that share them

void worker_main(dgx_server *s) {
    cudaSetDevice(s->device);
    cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    std::vector<double> t, dt;
    std::vector<unsigned int> st;
    std::vector<long long> stp;
    bool repack = false;   // the active set changed since the batch was built
    for (;;) {
        std::vector<Request *> admit;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->active.empty() && s->queue.empty() && !s->stop) {
                s->idle_cv.notify_all();
                const auto tw = Clock::now();
                s->cv.wait(lk, [&] { return s->stop || !s->queue.empty(); });
                s->idle_s += std::chrono::duration<double>(Clock::now() - tw).count();
            }
            if (s->stop) break;
            // admission by device-memory footprint and slot count, in arrival order
            std::set<MeshKey> pinned;
            while (!s->queue.empty() && static_cast<int>(s->active.size() + admit.size()) < s->max_active) {
                Request *q = s->queue.front();
                if (q->cancel) {
                    s->queue.pop_front();
                    q->state = kCancelled;
                    continue;
                }
                const MeshKey key = mesh_key(q->r);
                const bool cached = s->meshes.count(key) > 0;
                const size_t need = solver_estimate(q->r) + (cached ? 0 : mesh_estimate(q->r));
                pinned.insert(key);
                if (s->in_use + s->mesh_bytes + need > s->budget) evict_idle_meshes(s, need, 0, pinned);
                if (s->in_use + s->mesh_bytes + need > s->budget && !(s->active.empty() && admit.empty())) break;
                s->queue.pop_front();
                if (!cached) {   // reserve the mesh's bytes until it is built
                    auto &cm = s->meshes[key];
                    cm.bytes = mesh_estimate(q->r);
                    s->mesh_bytes += cm.bytes;
                }
                q->bytes = solver_estimate(q->r);
                s->in_use += q->bytes;
                admit.push_back(q);
                s->in_transit++;
            }
        }
        // (1) the running solves' next steps go on the stream first, so that
        // the admission round's host work (mesh generation and checks) below
        // runs while the GPU steps; its uploads and projections queue behind
        // the steps on the same stream
        const auto tp = Clock::now();
        auto tb = tp;   // when the steps were queued
        bool stepped = false;
        if (!s->active.empty()) {
            if (repack || !s->batch) {
                if (s->batch) dgx_batch_destroy(s->batch);
                s->batch = nullptr;
                std::vector<dgx_solver *> sv;
                for (Request *q : s->active) sv.push_back(q->solver);
                int rc = dgx_batch_create(sv.data(), static_cast<int>(sv.size()), &s->batch);
                s->repacks++;
                repack = false;
                if (rc) {
                    std::lock_guard<std::mutex> lk(s->mu);
                    for (Request *q : s->active) { release_solve(s, q); finish(s, q, kFailed, rc); }
                    s->active.clear();
                }
            }
            if (s->batch) {
                tb = Clock::now();
                {
                    std::lock_guard<std::mutex> lk(s->mu);
                    s->repack_s += std::chrono::duration<double>(tb - tp).count();
                }
                dgx_batch_run(s->batch, s->steps_per_check, s->stream);
                stepped = true;
            }
        }
        const auto t0 = Clock::now();
        // (2) the admission round
        std::vector<Request *> started;
        std::vector<std::pair<dgx_mesh *, size_t>> fresh;
        s->stage_off = 0;   // the previous round's uploads have completed
        if (admit.size() > s->min_diam_cap) {
            if (s->min_diam) cudaFreeHost(s->min_diam);
            s->min_diam = nullptr;
            s->min_diam_cap = 0;
            const size_t cap = std::max(admit.size(), static_cast<size_t>(256));
            if (cudaMallocHost(&s->min_diam, cap * sizeof(double)) == cudaSuccess) s->min_diam_cap = cap;
            else cudaGetLastError();   // meshes are then built synchronously
        }
        for (Request *q : admit) {
            int rc = DGX_OK;
            dgx_mesh *m = cached_mesh(s, q->r, &rc, fresh);
            if (!rc) rc = start_solve(s, q, m);
            if (!rc) { started.push_back(q); continue; }
            std::lock_guard<std::mutex> lk(s->mu);
            s->in_transit--;
            release_solve(s, q);
            finish(s, q, kFailed, rc);
        }
        cudaError_t admit_err = cudaSuccess;
        if (!admit.empty()) {   // the host's part of the round (the GPU meanwhile runs the steps)
            std::lock_guard<std::mutex> lk(s->mu);
            s->admit_s += std::chrono::duration<double>(Clock::now() - t0).count();
        }
        if (!started.empty() || !fresh.empty()) {
            // one synchronisation for the whole admission round (and the steps
            // queued before it): the uploads and projections have run, and any
            // fault of theirs shows here
            admit_err = cudaStreamSynchronize(s->stream);
            for (auto &f : fresh) f.first->d.min_diam = s->min_diam[f.second];
        }
        // (3) the steps' progress: finished solves read back and released
        if (stepped) {
            const size_t n = s->active.size();
            t.resize(n); dt.resize(n); st.resize(n); stp.resize(n);
            int rc = dgx_batch_progress(s->batch, t.data(), dt.data(), st.data(), stp.data(), s->stream);
            if (s->stall_seconds > 0.0)   // host-side fault injection: a stalled worker
                std::this_thread::sleep_for(std::chrono::duration<double>(s->stall_seconds));
            const auto t1 = Clock::now();
            std::vector<Request *> keep, done, leaving;
            std::vector<double> t_done;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                s->busy += std::chrono::duration<double>(t1 - tb).count();
                s->steps += s->steps_per_check;
                for (size_t i = 0; i < n; ++i) {
                    Request *q = s->active[i];
                    const long long done_steps = rc == DGX_OK ? stp[i] : q->steps;
                    s->dof_updates += static_cast<double>(done_steps - q->steps) * q->dofs;
                    q->steps = done_steps;
                    const bool bad = rc != DGX_OK || st[i] != 0;
                    const bool fin = !bad && (t[i] >= q->r.t_end || dt[i] == 0.0);
                    if (fin) {
                        done.push_back(q);
                        t_done.push_back(t[i]);
                    } else if (bad || q->cancel) {
                        leaving.push_back(q);
                    } else {
                        keep.push_back(q);
                    }
                }
            }
            const int trc = retire_totals(s, done);
            for (size_t j = 0; j < done.size() && !trc; ++j) {
                Request *q = done[j];
                q->t_final = t_done[j];
                if (q->r.keep_state) {
                    q->result.resize(q->solver->s.n);
                    dgx_get_state(q->solver, q->result.data());
                }
            }
            std::lock_guard<std::mutex> lk(s->mu);
            for (Request *q : done) {
                release_solve(s, q);
                if (trc) finish(s, q, kFailed, trc);
                else finish(s, q, kDone, DGX_OK);
            }
            for (Request *q : leaving) {
                release_solve(s, q);
                if (q->cancel) q->state = kCancelled;
                else finish(s, q, kFailed, DGX_ERR_NONFINITE);
            }
            if (keep.size() != n) {
                s->active.swap(keep);
                if (s->batch) dgx_batch_destroy(s->batch);
                s->batch = nullptr;
                repack = true;
                evict_idle_meshes(s, 0, kIdleMeshes, std::set<MeshKey>());
            }
            s->retire_s += std::chrono::duration<double>(Clock::now() - t1).count();
        }
        // (4) the admitted solves join the active set; the next round repacks
        if (!started.empty()) {
            std::lock_guard<std::mutex> lk(s->mu);
            for (Request *q : started) {
                s->in_transit--;
                if (admit_err != cudaSuccess) {
                    release_solve(s, q);
                    finish(s, q, kFailed, DGX_ERR_CUDA);
                    continue;
                }
                q->state = kRunning;
                q->started = Clock::now();
                s->active.push_back(q);
                repack = true;
            }
        }
    }
    if (s->batch) dgx_batch_destroy(s->batch);
    s->batch = nullptr;
    cudaStreamSynchronize(s->stream);
    for (Request *q : s->active) release_solve(s, q);
    s->active.clear();
    for (auto &kv : s->meshes)
        if (kv.second.mesh) dgx_mesh_destroy(kv.second.mesh);
    s->meshes.clear();
    s->mesh_bytes = 0;
    if (s->red) cudaFree(s->red);
    s->red = nullptr;
    if (s->stage) cudaFreeHost(s->stage);
    if (s->min_diam) cudaFreeHost(s->min_diam);
    s->stage = nullptr;
    s->min_diam = nullptr;
    s->pool->trim();
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
    // released blocks kept for reuse: a quarter of the budget, at most 8 GiB
    s->pool = new (std::nothrow) BlockPool(std::min(budget_bytes / 4, static_cast<size_t>(8) << 30));
    if (!s->pool) { delete s; set_error("host allocation failed"); return DGX_ERR_NOMEM; }
    cudaGetDevice(&s->device);
    s->worker = std::thread(worker_main, s);
    *out = s;
    return DGX_OK;
}

int dgx_server_submit(dgx_server *s, const dgx_request *r, long long *id) {
    if (!s || !r) { set_error("NULL argument"); return DGX_ERR_INVALID; }
    int rc = validate(*r);
    if (rc) { set_error("invalid request"); return rc; }
    if (mesh_estimate(*r) + solver_estimate(*r) > s->budget) { set_error("request needs more device memory than the budget"); return DGX_ERR_BUSY; }
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
    out->admit_seconds = s->admit_s;
    out->repack_seconds = s->repack_s;
    out->retire_seconds = s->retire_s;
    out->idle_seconds = s->idle_s;
    out->pool_hits = s->pool->hits();
    out->pool_misses = s->pool->misses();
    out->cached_meshes = static_cast<long long>(s->meshes.size());
    out->repacks = s->repacks;
    out->steps = s->steps;
    out->device_bytes_in_use = s->in_use + s->mesh_bytes;
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
    delete s->pool;
    delete s;
    return DGX_OK;
}

}  // extern "C"
