// dgx_batch.cu -- many independent solves advanced together.
//
// Solves are grouped into classes of equal (precision, order, equation).  Each
// class has work lists of (solve, element tile) items and one batched stage
// kernel per RK stage walks them, so solves of uneven sizes share every launch.
// One batched CFL kernel computes every solve's dt.  A time step -- the CFL
// launch, then per class its four stage launches on its own stream -- is
// captured once as a CUDA graph and replayed.  Per class, the kernel options
// (TMA prefetch of the epilogue operands, flat or persistent grid) are chosen
// by timing (dgx_batch_autotune).  This generalises the reference's one-solve
// loop (src/2d/conservation/time_integrator.cu:252-429); it has no counterpart
// there.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "dgx_internal.h"

namespace dgx {
namespace {

struct BatchClass {
    int precision = 0, order = 0, equation = 0;
    int bnd = 0;                             // the class's meshes have boundary sides
    std::vector<int> solves;                 // indices into the batch's solver list
    StageArgs *d_args[4] = {nullptr, nullptr, nullptr, nullptr};
    int2 *d_items = nullptr;
    int n_items = 0;
    int nslot = 0;
    int prefetch = 1;                        // tuned option
    int pre_plane = 0;                       // values per prefetched plane (largest of the solves)
    int persistent = 0;                      // tuned option: 0 flat grid, k > 0: k CTAs per SM
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    long long dofs = 0;
    std::vector<StageArgs> h_args;           // host copy of d_args (stage-major), for the parameter launches
    std::vector<int> tiles;                  // tiles of each solve
};

// elements per work item of the batched CFL kernel (8 per thread)
constexpr int kCflItemElems = 2048;

int num_sms() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    return sms;
}

}  // namespace
}  // namespace dgx

using namespace dgx;

struct dgx_batch {
    std::vector<dgx_solver *> solvers;
    const double **d_scal = nullptr;        // each solve's device scalars
    const unsigned int **d_status = nullptr;
    const long long **d_steps = nullptr;
    double *d_progress = nullptr;          // [n][4]: t, dt, status, steps
    std::vector<double> h_progress;        // host copy
    DeviceBlock block;                     // every device array of the batch, one allocation
    std::vector<BatchClass> classes;
    DtArgs *d_dt = nullptr;
    int2 *d_cfl_items = nullptr;
    int n_cfl_items = 0;
    cudaStream_t cap = nullptr;
    cudaEvent_t start = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long dofs = 0;
    long long launches = 0;
    long long launches_per_step = 0;
    // one launch per stage for every class (dgx_batch_fused.cu): FP32 batches
    // whose meshes have no boundary sides; 0 off, else the kernel variant (2
    // or 3 CTAs per SM)
    int fused = 0;
    bool fusable = false;
    StageArgs *d_fargs = nullptr;          // [stage][solve], solves in the items' class order
    int4 *d_fitems = nullptr;
    int n_fitems = 0;
    size_t fsmem = 0;
};

namespace dgx {
namespace {

int class_launch(dgx_batch *b, BatchClass &k, int stage, cudaStream_t st) {
    if (k.persistent == 0) {
        // the flat grid: the solves' arguments as kernel parameters, up to
        // kParamSolves solves per launch
        const size_t ns = k.solves.size();
        static thread_local BatchParamArgs p;
        p.nslot = k.nslot;
        // stage 1 of a compensated class prefetches the state's low part
        p.prefetch = ((stage >= 1 || k.precision == DGX_FP32_COMP) && k.prefetch) ? k.pre_plane : 0;
        p.bnd = k.bnd;
        for (size_t j0 = 0; j0 < ns; j0 += kParamSolves) {
            const int n = static_cast<int>(std::min<size_t>(kParamSolves, ns - j0));
            int t = 0;
            for (int j = 0; j < n; ++j) {
                p.args[j] = k.h_args[stage * ns + j0 + j];
                p.tile_start[j] = t;
                t += k.tiles[j0 + j];
            }
            p.tile_start[n] = t;
            p.n = n;
            const int rc = launch_batch_param(k.precision, k.order, k.equation, p, t, st);
            if (rc) return rc;
            if (t > 0) b->launches++;
        }
        return DGX_OK;
    }
    BatchStageArgs a;
    a.args = k.d_args[stage];
    a.items = k.d_items;
    a.n_items = k.n_items;
    a.nslot = k.nslot;
    a.prefetch = ((stage >= 1 || k.precision == DGX_FP32_COMP) && k.prefetch) ? k.pre_plane : 0;
    a.bnd = k.bnd;
    if (k.persistent > 0) a.grid = std::min(k.n_items, num_sms() * k.persistent);
    else a.grid = k.n_items;
    const int rc = launch_batch_stage(k.precision, k.order, k.equation, a, st);
    if (!rc && a.grid > 0) b->launches++;
    return rc;
}

// The per-solve stage arguments of one class for its options, stage-major
// (host[stage * solves + j]); sets the class's slot count and prefetch plane,
// and turns the prefetch off when it would not fit in shared memory.
int class_host_args(dgx_batch *b, BatchClass &k, std::vector<StageArgs> &host) {
    const size_t ns = k.solves.size();
    host.resize(4 * ns);
    int nslot = 0, plane = 0;
    for (int stage = 0; stage < 4; ++stage) {
        for (size_t j = 0; j < ns; ++j) {
            dgx_solver *sv = b->solvers[k.solves[j]];
            SolverDev &s = sv->s;
            const int saved = s.prefetch;
            s.prefetch = k.prefetch;
            StageArgs &h = host[stage * ns + j];
            h = rk4_stage_args(sv, stage);
            s.prefetch = saved;
            nslot = std::max(nslot, h.nslot);
            plane = std::max(plane, h.prefetch);
        }
    }
    k.nslot = nslot;
    k.pre_plane = plane;
    const int pp = k.prefetch ? k.pre_plane : 0;
    const size_t smem = k.precision == DGX_FP64 ? batch_smem_f64(k.order, k.equation, nslot, pp)
                                                : batch_smem_f32(k.order, k.equation, nslot, pp);
    if (k.prefetch && smem > 200 * 1024) {
        k.prefetch = 0;
        return class_host_args(b, k, host);
    }
    return DGX_OK;
}

// set the class kernel's shared-memory limit outside any capture (grid 0: no launch)
int class_configure(BatchClass &k) {
    BatchStageArgs probe{k.d_args[1], k.d_items, 0, 0, k.nslot, k.prefetch ? k.pre_plane : 0, k.bnd};
    int rc = launch_batch_stage(k.precision, k.order, k.equation, probe, nullptr);
    if (rc) return rc;
    static thread_local BatchParamArgs pp;
    pp.n = 0;
    pp.nslot = k.nslot;
    pp.prefetch = k.prefetch ? k.pre_plane : 0;
    pp.bnd = k.bnd;
    return launch_batch_param(k.precision, k.order, k.equation, pp, 0, nullptr);
}

int fused_upload(dgx_batch *b);

// Upload the per-solve stage arguments of one class for its current options
// (the four stages' arrays are contiguous: one copy).
int class_upload(dgx_batch *b, BatchClass &k) {
    std::vector<StageArgs> host;
    int rc = class_host_args(b, k, host);
    if (rc) return rc;
    DGX_TRY_CUDA(cudaMemcpy(k.d_args[0], host.data(), host.size() * sizeof(StageArgs), cudaMemcpyHostToDevice));
    k.h_args = host;
    rc = class_configure(k);
    if (!rc) rc = fused_upload(b);
    return rc;
}

// Order of the classes in the fused work list: costliest tiles first, so the
// last wave of the launch is filled with the cheapest ones (work per element
// and stage ~ modes x variables x the volume and side points)
long long fused_cost(const BatchClass &k) {
    const int np = (k.order + 1) * (k.order + 2) / 2, nv = k.equation == DGX_EULER ? 4 : 1;
    return static_cast<long long>(np) * nv * (num_quad(k.order) + 3 * num_quad1(k.order));
}
std::vector<int> fused_class_order(const dgx_batch *b) {
    std::vector<int> ord(b->classes.size());
    for (size_t c = 0; c < ord.size(); ++c) ord[c] = static_cast<int>(c);
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int x, int y) { return fused_cost(b->classes[x]) > fused_cost(b->classes[y]); });
    return ord;
}

// The fused launches' stage arguments: every class's current per-solve
// arguments (its own options), in the work list's class order; and the
// launch's shared memory, the largest any class needs.
int fused_upload(dgx_batch *b) {
    if (!b->fusable) return DGX_OK;
    const std::vector<int> ord = fused_class_order(b);
    size_t ns = 0;
    for (auto &k : b->classes) ns += k.solves.size();
    std::vector<StageArgs> host(4 * ns);
    size_t base = 0, smem = 0;
    for (int c : ord) {
        const BatchClass &k = b->classes[c];
        const size_t n = k.solves.size();
        for (int stage = 0; stage < 4; ++stage)
            for (size_t j = 0; j < n; ++j) host[stage * ns + base + j] = k.h_args[stage * n + j];
        base += n;
        smem = std::max(smem, batch_smem_f32(k.order, k.equation, k.nslot, k.prefetch ? k.pre_plane : 0));
    }
    DGX_TRY_CUDA(cudaMemcpy(b->d_fargs, host.data(), host.size() * sizeof(StageArgs), cudaMemcpyHostToDevice));
    b->fsmem = smem;
    // set the kernels' shared-memory limits outside any capture (no launch)
    for (int v = 2; v <= 3; ++v) {
        FusedStageArgs f{b->d_fargs, b->d_fitems, 0, v};
        const int rc = launch_batch_fused_f32(f, smem, nullptr);
        if (rc) return rc;
    }
    return DGX_OK;
}

int fused_launch(dgx_batch *b, int stage, cudaStream_t st) {
    size_t ns = 0;
    for (auto &k : b->classes) ns += k.solves.size();
    FusedStageArgs f{b->d_fargs + stage * ns, b->d_fitems, b->n_fitems, b->fused};
    const int rc = launch_batch_fused_f32(f, b->fsmem, st);
    if (!rc && b->n_fitems > 0) b->launches++;
    return rc;
}

// one step without the graph
int step_direct(dgx_batch *b, cudaStream_t st) {
    int rc = launch_batch_dt(b->d_dt, b->d_cfl_items, b->n_cfl_items, st);
    if (rc) return rc;
    b->launches++;
    if (b->fused) {
        for (int stage = 0; stage < 4 && !rc; ++stage) rc = fused_launch(b, stage, st);
        return rc;
    }
    for (auto &k : b->classes)
        for (int stage = 0; stage < 4; ++stage) {
            rc = class_launch(b, k, stage, st);
            if (rc) return rc;
        }
    return DGX_OK;
}

void destroy_graph(dgx_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Capture one step: CFL on the capture stream, then each class's four stages on
// its own stream (classes are independent), joined back.
int build_graph(dgx_batch *b) {
    destroy_graph(b);
    const long long l0 = b->launches;
    DGX_TRY_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
    int rc = launch_batch_dt(b->d_dt, b->d_cfl_items, b->n_cfl_items, b->cap);
    b->launches++;
    if (!rc) rc = cudaEventRecord(b->start, b->cap) == cudaSuccess ? DGX_OK : DGX_ERR_CUDA;
    // fused: the four stage launches of every class on the capture stream
    for (int stage = 0; b->fused && stage < 4 && !rc; ++stage) rc = fused_launch(b, stage, b->cap);
    for (auto &k : b->classes) {
        if (rc || b->fused) break;
        if (cudaStreamWaitEvent(k.stream, b->start, 0) != cudaSuccess) { rc = DGX_ERR_CUDA; break; }
        for (int stage = 0; stage < 4 && !rc; ++stage) rc = class_launch(b, k, stage, k.stream);
        if (!rc && cudaEventRecord(k.done, k.stream) != cudaSuccess) rc = DGX_ERR_CUDA;
        if (!rc && cudaStreamWaitEvent(b->cap, k.done, 0) != cudaSuccess) rc = DGX_ERR_CUDA;
    }
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(b->cap, &g);
    if (rc || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (!rc) set_error("graph capture failed: %s", cudaGetErrorString(ce));
        return rc ? rc : DGX_ERR_CUDA;
    }
    b->graph = g;
    DGX_TRY_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
    b->launches_per_step = b->launches - l0;
    b->launches = l0;
    return DGX_OK;
}

__global__ void progress_kernel(const double *const *scal, const unsigned int *const *status,
                                const long long *const *steps, int n, double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[4 * i] = scal[i][1];
    out[4 * i + 1] = scal[i][0];
    out[4 * i + 2] = static_cast<double>(*status[i]);
    out[4 * i + 3] = static_cast<double>(*steps[i]);
}

void batch_free(dgx_batch *b) {
    destroy_graph(b);
    block_free(b->block);
    for (auto &k : b->classes) {
        if (k.stream) cudaStreamDestroy(k.stream);
        if (k.done) cudaEventDestroy(k.done);
    }
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->start) cudaEventDestroy(b->start);
    delete b;
}

}  // namespace
}  // namespace dgx

extern "C" {

int dgx_batch_create(dgx_solver *const *solvers, int n, dgx_batch **out) {
    if (!solvers || n <= 0 || !out) { set_error("need at least one solver"); return DGX_ERR_INVALID; }
    *out = nullptr;
    dgx_batch *b = new (std::nothrow) dgx_batch();
    if (!b) { set_error("host allocation failed"); return DGX_ERR_NOMEM; }
    for (int i = 0; i < n; ++i) {
        if (!solvers[i]) { set_error("solver %d is NULL", i); batch_free(b); return DGX_ERR_INVALID; }
        for (int j = 0; j < i; ++j)
            if (solvers[j] == solvers[i]) { set_error("solver %d appears twice", i); batch_free(b); return DGX_ERR_INVALID; }
        if (solvers[i]->s.precision == DGX_FP32_BF16X3) {
            set_error("solver %d: batches take FP32 and FP64 solvers", i);
            batch_free(b);
            return DGX_ERR_UNSUPPORTED;
        }
        if (solvers[i]->s.limiter) {
            set_error("solver %d: batches do not apply the limiter", i);
            batch_free(b);
            return DGX_ERR_UNSUPPORTED;
        }
        if (solvers[i]->s.integrator != DGX_RK4) {
            set_error("solver %d: batches take RK4 solvers only", i);
            batch_free(b);
            return DGX_ERR_UNSUPPORTED;
        }
        b->solvers.push_back(solvers[i]);
    }
    // classes
    for (int i = 0; i < n; ++i) {
        const SolverDev &s = solvers[i]->s;
        BatchClass *k = nullptr;
        const int bnd = solvers[i]->mesh->d.num_boundary > 0 ? 1 : 0;
        for (auto &c : b->classes)
            if (c.precision == s.precision && c.order == s.order && c.equation == s.equation && c.bnd == bnd) k = &c;
        if (!k) {
            b->classes.emplace_back();
            k = &b->classes.back();
            k->precision = s.precision;
            k->order = s.order;
            k->equation = s.equation;
            k->bnd = bnd;
        }
        k->solves.push_back(i);
        k->dofs += static_cast<long long>(s.n);
        b->dofs += static_cast<long long>(s.n);
    }
    int rc = DGX_OK;
    std::vector<DtArgs> dts(n);
    std::vector<int2> cfl_items;
    for (int i = 0; i < n; ++i) {
        dts[i] = make_dt_args(solvers[i]->s, solvers[i]->mesh->d);
        // one work item per kCflItemElems elements (the maximum is exact in any
        // partition): the per-item reduction, atomics and argument loads then
        // cost little beside the item's loads
        if (dts[i].euler) {
            const int want = (dts[i].E + kCflItemElems - 1) / kCflItemElems;
            dts[i].nblocks = std::max(1, std::min(dts[i].nblocks, want));
        }
        for (int blk = 0; blk < dts[i].nblocks; ++blk) cfl_items.push_back(make_int2(i, blk));
    }
    b->n_cfl_items = static_cast<int>(cfl_items.size());
    std::vector<std::vector<int2>> items(b->classes.size());
    std::vector<std::vector<StageArgs>> args(b->classes.size());
    for (size_t c = 0; c < b->classes.size() && !rc; ++c) {
        BatchClass &k = b->classes[c];
        for (size_t j = 0; j < k.solves.size(); ++j) {
            const int ntiles = b->solvers[k.solves[j]]->mesh->d.num_tiles;
            for (int t = 0; t < ntiles; ++t) items[c].push_back(make_int2(static_cast<int>(j), t));
            k.tiles.push_back(ntiles);
        }
        k.n_items = static_cast<int>(items[c].size());
        rc = class_host_args(b, k, args[c]);
        if (!rc) k.h_args = args[c];
    }
    if (rc) { batch_free(b); return rc; }
    // the fused work list: (index into the fused arguments, tile, class code),
    // costliest classes first
    b->fusable = true;
    for (auto &k : b->classes)
        if ((k.precision != DGX_FP32 && k.precision != DGX_FP32_COMP) || k.bnd || k.order > kFusedMaxOrder)
            b->fusable = false;
    std::vector<int4> fitems;
    if (b->fusable) {
        int base = 0;
        for (int c : fused_class_order(b)) {
            const BatchClass &k = b->classes[c];
            const int code = 2 * k.order + (k.equation == DGX_EULER ? 1 : 0);
            for (size_t j = 0; j < k.solves.size(); ++j)
                for (int t = 0; t < k.tiles[j]; ++t) fitems.push_back(make_int4(base + static_cast<int>(j), t, code, 0));
            base += static_cast<int>(k.solves.size());
        }
        b->n_fitems = static_cast<int>(fitems.size());
    }
    // one device block for every array of the batch, filled by one copy
    BlockLayout L;
    const size_t oScal = L.take<const double *>(n), oStat = L.take<const unsigned int *>(n),
                 oSteps = L.take<const long long *>(n), oDt = L.take<DtArgs>(n), oCfl = L.take<int2>(cfl_items.size());
    std::vector<size_t> oArgs(b->classes.size()), oItems(b->classes.size());
    for (size_t c = 0; c < b->classes.size(); ++c) {
        oArgs[c] = L.take<StageArgs>(args[c].size());
        oItems[c] = L.take<int2>(items[c].size());
    }
    const size_t oFItems = L.take<int4>(fitems.size());
    const size_t upload = L.size;
    const size_t oProg = L.take<double>(4 * static_cast<size_t>(n));
    const size_t oFArgs = L.take<StageArgs>(b->fusable ? 4 * static_cast<size_t>(n) : 0);
    rc = block_alloc(b->block, L.size, nullptr);
    if (rc) { batch_free(b); return rc; }
    std::vector<unsigned char> stage(upload, 0);
    auto put = [&](size_t off, const void *src, size_t bytes) {
        if (bytes) std::memcpy(stage.data() + off, src, bytes);
    };
    {
        std::vector<const double *> sc(n);
        std::vector<const unsigned int *> stt(n);
        std::vector<const long long *> stp(n);
        for (int i = 0; i < n; ++i) {
            sc[i] = solvers[i]->s.scal;
            stt[i] = solvers[i]->s.status;
            stp[i] = solvers[i]->s.steps;
        }
        put(oScal, sc.data(), sizeof(double *) * n);
        put(oStat, stt.data(), sizeof(unsigned int *) * n);
        put(oSteps, stp.data(), sizeof(long long *) * n);
    }
    put(oDt, dts.data(), sizeof(DtArgs) * n);
    put(oFItems, fitems.data(), sizeof(int4) * fitems.size());
    put(oCfl, cfl_items.data(), sizeof(int2) * cfl_items.size());
    for (size_t c = 0; c < b->classes.size(); ++c) {
        put(oArgs[c], args[c].data(), sizeof(StageArgs) * args[c].size());
        put(oItems[c], items[c].data(), sizeof(int2) * items[c].size());
    }
    b->d_scal = block_at<const double *>(b->block, oScal);
    b->d_status = block_at<const unsigned int *>(b->block, oStat);
    b->d_steps = block_at<const long long *>(b->block, oSteps);
    b->d_dt = block_at<DtArgs>(b->block, oDt);
    b->d_cfl_items = block_at<int2>(b->block, oCfl);
    b->d_progress = block_at<double>(b->block, oProg);
    b->d_fitems = block_at<int4>(b->block, oFItems);
    b->d_fargs = block_at<StageArgs>(b->block, oFArgs);
    b->h_progress.assign(4 * static_cast<size_t>(n), 0.0);
    for (size_t c = 0; c < b->classes.size(); ++c) {
        BatchClass &k = b->classes[c];
        StageArgs *a0 = block_at<StageArgs>(b->block, oArgs[c]);
        for (int st = 0; st < 4; ++st) k.d_args[st] = a0 + st * k.solves.size();
        k.d_items = block_at<int2>(b->block, oItems[c]);
    }
    if (cudaMemcpy(b->block.base, stage.data(), upload, cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("batch upload failed");
        batch_free(b);
        return DGX_ERR_CUDA;
    }
    for (auto &k : b->classes) {
        if (cudaStreamCreateWithFlags(&k.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&k.done, cudaEventDisableTiming) != cudaSuccess)
            rc = DGX_ERR_CUDA;
        if (!rc) rc = class_configure(k);
        if (rc) break;
    }
    if (!rc) rc = fused_upload(b);
    if (!rc && (cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess ||
                cudaEventCreateWithFlags(&b->start, cudaEventDisableTiming) != cudaSuccess))
        rc = DGX_ERR_CUDA;
    if (!rc) rc = build_graph(b);
    if (rc) {
        if (!dgx_last_error()[0]) set_error("batch creation failed");
        batch_free(b);
        return rc;
    }
    *out = b;
    return DGX_OK;
}

int dgx_batch_destroy(dgx_batch *b) {
    if (!b) return DGX_ERR_INVALID;
    cudaDeviceSynchronize();
    batch_free(b);
    return DGX_OK;
}

int dgx_batch_step(dgx_batch *b, void *stream) {
    if (!b || !b->exec) return DGX_ERR_INVALID;
    DGX_TRY_CUDA(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)));
    b->launches += b->launches_per_step;
    return DGX_OK;
}

int dgx_batch_run(dgx_batch *b, int steps, void *stream) {
    if (!b || steps < 0) return DGX_ERR_INVALID;
    for (int i = 0; i < steps; ++i) {
        int rc = dgx_batch_step(b, stream);
        if (rc) return rc;
    }
    return DGX_OK;
}

int dgx_batch_info(const dgx_batch *b, int *num_classes, int *num_items, long long *dofs,
                   long long *launches_per_step) {
    if (!b) return DGX_ERR_INVALID;
    int items = 0;
    for (auto &k : b->classes) items += k.n_items;
    if (num_classes) *num_classes = static_cast<int>(b->classes.size());
    if (num_items) *num_items = items;
    if (dofs) *dofs = b->dofs;
    if (launches_per_step) *launches_per_step = b->launches_per_step;
    return DGX_OK;
}

int dgx_batch_class_options(const dgx_batch *b, int cls, int *order, int *equation, int *prefetch,
                            int *persistent) {
    if (!b || cls < 0 || cls >= static_cast<int>(b->classes.size())) return DGX_ERR_INVALID;
    const auto &k = b->classes[cls];
    if (order) *order = k.order;
    if (equation) *equation = k.equation;
    if (prefetch) *prefetch = k.prefetch;
    if (persistent) *persistent = k.persistent;
    return DGX_OK;
}

int dgx_batch_progress(dgx_batch *b, double *t, double *dt, unsigned int *status, long long *steps,
                       void *stream) {
    if (!b) return DGX_ERR_INVALID;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int n = static_cast<int>(b->solvers.size());
    progress_kernel<<<(n + 127) / 128, 128, 0, st>>>(b->d_scal, b->d_status, b->d_steps, n, b->d_progress);
    DGX_CHECK_LAUNCH();
    DGX_TRY_CUDA(cudaMemcpyAsync(b->h_progress.data(), b->d_progress, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, st));
    DGX_TRY_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < n; ++i) {
        if (t) t[i] = b->h_progress[4 * i];
        if (dt) dt[i] = b->h_progress[4 * i + 1];
        if (status) status[i] = static_cast<unsigned int>(b->h_progress[4 * i + 2]);
        if (steps) steps[i] = static_cast<long long>(b->h_progress[4 * i + 3]);
    }
    return DGX_OK;
}

int dgx_batch_set_options(dgx_batch *b, int cls, int prefetch, int persistent) {
    if (!b || cls < 0 || cls >= static_cast<int>(b->classes.size())) return DGX_ERR_INVALID;
    auto &k = b->classes[cls];
    k.prefetch = prefetch ? 1 : 0;
    k.persistent = persistent < 0 ? 0 : persistent;
    int rc = class_upload(b, k);
    if (!rc) rc = build_graph(b);
    return rc;
}

int dgx_batch_set_fused(dgx_batch *b, int mode) {
    if (!b || (mode != 0 && mode != 2 && mode != 3)) { set_error("fused mode is 0, 2 or 3"); return DGX_ERR_INVALID; }
    if (mode && !b->fusable) {
        set_error("the fused launch takes FP32 batches whose meshes have no boundary sides, orders up to %d",
                  kFusedMaxOrder);
        return DGX_ERR_UNSUPPORTED;
    }
    b->fused = mode;
    return build_graph(b);
}

int dgx_batch_get_fused(const dgx_batch *b, int *mode, int *available) {
    if (!b) return DGX_ERR_INVALID;
    if (mode) *mode = b->fused;
    if (available) *available = b->fusable ? 1 : 0;
    return DGX_OK;
}

int dgx_batch_launch_count(const dgx_batch *b, long long *count) {
    if (!b || !count) return DGX_ERR_INVALID;
    *count = b->launches;
    return DGX_OK;
}

// Time the candidate options of every class on the live batch, keep the
// fastest, and rebuild the graph.  The solves' states, times and step counts
// are saved before and restored after, so the batch continues as if untuned.
int dgx_batch_autotune(dgx_batch *b, int reps, void *stream) {
    if (!b) return DGX_ERR_INVALID;
    if (reps <= 0) reps = 3;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DGX_TRY_CUDA(cudaStreamSynchronize(st));
    // save
    const size_t n = b->solvers.size();
    std::vector<void *> saved(n, nullptr), saved_lo(n, nullptr);
    std::vector<double> scal(8 * n);
    std::vector<long long> steps(n);
    int rc = DGX_OK;
    for (size_t i = 0; i < n && !rc; ++i) {
        SolverDev &s = b->solvers[i]->s;
        const size_t bytes = s.n * (s.precision == DGX_FP64 ? 8 : 4);
        if (cudaMalloc(&saved[i], bytes) != cudaSuccess) { set_error("autotune backup allocation failed"); rc = DGX_ERR_NOMEM; break; }
        if (s.lo && (cudaMalloc(&saved_lo[i], bytes) != cudaSuccess ||
                     cudaMemcpy(saved_lo[i], s.lo, bytes, cudaMemcpyDeviceToDevice) != cudaSuccess)) {
            set_error("autotune backup of the low part failed");
            rc = DGX_ERR_NOMEM;
            break;
        }
        if (cudaMemcpy(saved[i], s.c, bytes, cudaMemcpyDeviceToDevice) != cudaSuccess ||
            cudaMemcpy(&scal[8 * i], s.scal, 8 * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(&steps[i], s.steps, sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = DGX_ERR_CUDA;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!rc && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) rc = DGX_ERR_CUDA;
    // one CFL launch gives every solve a dt for the timed stage launches
    if (!rc) rc = launch_batch_dt(b->d_dt, b->d_cfl_items, b->n_cfl_items, st);
    const int cand[][2] = {{1, 0}, {0, 0}, {1, 2}, {0, 2}, {1, 4}};
    for (auto &k : b->classes) {
        if (rc) break;
        float best = 1e30f;
        int bp = k.prefetch, bq = k.persistent;
        for (auto &c : cand) {
            k.prefetch = c[0];
            k.persistent = c[1];
            rc = class_upload(b, k);
            if (rc) break;
            if (c[0] && !k.prefetch) continue;    // prefetch does not fit
            for (int w = 0; w < 1 && !rc; ++w)
                for (int stage = 1; stage < 4 && !rc; ++stage) rc = class_launch(b, k, stage, st);
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps && !rc; ++r)
                for (int stage = 1; stage < 4 && !rc; ++stage) rc = class_launch(b, k, stage, st);
            cudaEventRecord(e1, st);
            if (rc) break;
            if (cudaEventSynchronize(e1) != cudaSuccess) { rc = DGX_ERR_CUDA; break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) { best = ms; bp = c[0]; bq = c[1]; }
        }
        k.prefetch = bp;
        k.persistent = bq;
        if (!rc) rc = class_upload(b, k);
    }
    // then the whole step: the tuned per-class launches against the fused
    // launch of both variants (graph steps; the states are restored below)
    if (!rc && b->fusable) {
        float best = 1e30f;
        int bf = 0;
        for (int mode : {0, 2, 3}) {
            b->fused = mode;
            rc = build_graph(b);
            if (rc) break;
            if (cudaGraphLaunch(b->exec, st) != cudaSuccess) { rc = DGX_ERR_CUDA; break; }
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps && !rc; ++r)
                if (cudaGraphLaunch(b->exec, st) != cudaSuccess) rc = DGX_ERR_CUDA;
            cudaEventRecord(e1, st);
            if (rc || cudaEventSynchronize(e1) != cudaSuccess) { rc = rc ? rc : DGX_ERR_CUDA; break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) { best = ms; bf = mode; }
        }
        b->fused = bf;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    // restore
    for (size_t i = 0; i < n; ++i) {
        SolverDev &s = b->solvers[i]->s;
        if (!saved[i]) continue;
        const size_t bytes = s.n * (s.precision == DGX_FP64 ? 8 : 4);
        if (saved_lo[i]) {
            if (cudaMemcpy(s.lo, saved_lo[i], bytes, cudaMemcpyDeviceToDevice) != cudaSuccess) rc = rc ? rc : DGX_ERR_CUDA;
            cudaFree(saved_lo[i]);
        }
        if (cudaMemcpy(s.c, saved[i], bytes, cudaMemcpyDeviceToDevice) != cudaSuccess ||
            cudaMemcpy(s.scal, &scal[8 * i], 8 * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(s.steps, &steps[i], sizeof(long long), cudaMemcpyHostToDevice) != cudaSuccess)
            rc = rc ? rc : DGX_ERR_CUDA;
        cudaFree(saved[i]);
    }
    if (!rc) rc = build_graph(b);
    return rc;
}

}  // extern "C"
