// dgx_api.cu -- the C ABI (include/dgx.h): meshes, solvers, state, RHS and
// RK-stage calls.  Host orchestration only; the arithmetic is in
// dgx_stage_f32.cu / dgx_stage_f64.cu / dgx_misc.cu.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <new>
#include <vector>

#include "dgx_internal.h"
#include "dgx_tc_layout.h"

namespace dgx {

namespace {
thread_local char g_err[512] = "";
std::mutex g_init_mu;
bool g_tables_ready[64] = {false};

// The BF16x3 path: its tables, and the tensor-core self-test passed once on
// this device (dgx_tc_selftest).
bool g_tc_ready[64] = {};
int ensure_tensor_cores() {
    int dev = 0;
    DGX_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device index %d out of range", dev); return DGX_ERR_UNSUPPORTED; }
    {
        std::lock_guard<std::mutex> lk(g_init_mu);
        if (g_tc_ready[dev]) return DGX_OK;
    }
    int major = 0, minor = 0;
    DGX_TRY_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    DGX_TRY_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3) {
        set_error("the BF16x3 path is built for sm_103a; this device is sm_%d%d", major, minor);
        return DGX_ERR_UNSUPPORTED;
    }
    int bad_ss = -1, bad_ts = -1;
    int rc = dgx_tc_selftest(0, &bad_ss, &bad_ts, nullptr);
    if (rc) return rc;
    if (bad_ss || bad_ts) {
        set_error("tensor-core self-test failed (%d, %d wrong elements)", bad_ss, bad_ts);
        return DGX_ERR_UNSUPPORTED;
    }
    rc = tc_images_upload();
    if (!rc) rc = upload_tables_tc();
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_init_mu);
    g_tc_ready[dev] = true;
    return DGX_OK;
}

int ensure_device_tables() {
    int dev = 0;
    DGX_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device index %d out of range", dev); return DGX_ERR_UNSUPPORTED; }
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (g_tables_ready[dev]) return DGX_OK;
    int rc = upload_tables_f32_nb();
    if (!rc) rc = upload_tables_f32_b();
    if (!rc) rc = upload_tables_f64_nb();
    if (!rc) rc = upload_tables_f64_b();
    if (!rc) rc = upload_tables_misc();
    if (!rc) rc = upload_tables_fused();
    if (!rc) g_tables_ready[dev] = true;
    return rc;
}

template <typename T>
int dalloc(T **p, size_t count, size_t *acct) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
        return DGX_ERR_NOMEM;
    }
    if (acct) *acct += count * sizeof(T);
    return DGX_OK;
}

void mesh_free(dgx_mesh *m) {
    block_free(m->block);
    delete m;
}

void mesh_release(dgx_mesh *m) {
    if (m && m->refs.fetch_sub(1) == 1) mesh_free(m);
}

cudaStream_t as_stream(void *s) { return static_cast<cudaStream_t>(s); }

// Tiles of kTile consecutive elements: for every element side, the shared-memory
// slot that will hold the neighbour's trace (inside the tile: 3*l + side; outside:
// the tile's next halo slot), and per tile the list of halo (element, side) pairs.
void build_tiles(int E, const int *const es[3], const int *le, const int *re, const int *ls,
                 const int *rs, std::vector<int> &words, std::vector<int> &hoff,
                 std::vector<int> &hlist, int &max_halo) {
    const int ntiles = (E + kTile - 1) / kTile;
    words.assign(3 * static_cast<size_t>(E), 0);
    hoff.assign(ntiles + 1, 0);
    hlist.clear();
    hlist.reserve(E);
    max_halo = 0;
    for (int b = 0; b < ntiles; ++b) {
        hoff[b] = static_cast<int>(hlist.size());
        const int lo = b * kTile, hi = std::min(E, lo + kTile);
        for (int e = lo; e < hi; ++e)
            for (int k = 0; k < 3; ++k) {
                const int s = es[k][e];
                const int il = (le[s] == e) ? 1 : 0;   // the reference's rule (time_integrator.cu:153)
                const int ne = il ? re[s] : le[s];
                const int ns = il ? rs[s] : ls[s];
                int w;
                if (ne < 0) w = ne;
                else if (ne >= lo && ne < hi) w = pack_side_word(3 * (ne - lo) + ns, il);
                else {
                    const int h = static_cast<int>(hlist.size()) - hoff[b];
                    hlist.push_back(pack_halo(ne, ns));
                    w = pack_side_word(3 * kTile + h, il);
                }
                words[static_cast<size_t>(k) * E + e] = w;
            }
        max_halo = std::max(max_halo, static_cast<int>(hlist.size()) - hoff[b]);
    }
    hoff[ntiles] = static_cast<int>(hlist.size());
}

size_t elem_size(const SolverDev &s) { return s.precision == DGX_FP64 ? sizeof(double) : sizeof(float); }

int stage_launch(dgx_solver *sv, int mode, const void *u, const void *c, void *acc, void *out,
                 double dt, double t, cudaStream_t st) {
    const StageArgs a = make_stage_args(sv, mode, u, c, acc, out, dt, t);
    const int rc = launch_stage(sv->s.precision, sv->s.order, sv->s.equation, a, st);
    if (!rc) sv->launches++;
    return rc;
}

int run_stage_raw(dgx_solver *sv, int stage, cudaStream_t st);

// One stage, then (DGX_OPT_LIMITER) the limiter on the state the stage wrote
int run_stage(dgx_solver *sv, int stage, cudaStream_t st) {
    int rc = run_stage_raw(sv, stage, st);
    SolverDev &s = sv->s;
    if (rc || !s.limiter) return rc;
    void *out = s.c;
    if (s.integrator == DGX_RK4 && stage < 3) out = stage == 1 ? s.ub : s.ua;
    else if (s.integrator == DGX_RK2 && stage == 0) out = s.ua;
    rc = limit_state(s, sv->mesh->d, out, st);
    if (!rc) sv->launches++;
    return rc;
}

int run_stage_raw(dgx_solver *sv, int stage, cudaStream_t st) {
    SolverDev &s = sv->s;
    int rc;
    const int nst = num_stages(s.integrator);
    if (stage < 0 || stage >= nst) { set_error("stage must be 0..%d", nst - 1); return DGX_ERR_INVALID; }
    if (stage == 0) {
        rc = launch_dt(s, sv->mesh->d, st);
        if (rc) return rc;
        sv->launches++;
    }
    if (s.integrator == DGX_RK2) {
        // k1 at the state, ua = c + k1/2; then c += k2 with k2 at ua
        // (rk2_tempstorage / rk2, time_integrator.cu:445-464, 518-580)
        if (stage == 0) return stage_launch(sv, 5, s.c, nullptr, nullptr, s.ua, 0.0, 0.0, st);
        return stage_launch(sv, 6, s.ua, s.c, nullptr, s.c, 0.0, 0.0, st);
    }
    if (s.integrator == DGX_FE) {
        // ua = c + k, then commit ua to c (neighbouring tiles read c while the
        // stage runs, so it cannot be updated in place; eval_rhs_fe,
        // time_integrator.cu:622-700)
        rc = stage_launch(sv, 5, s.c, nullptr, nullptr, s.ua, 0.0, 0.0, st);
        if (rc) return rc;
        rc = commit_state(s, s.c, s.ua, st);
        if (!rc) sv->launches++;
        return rc;
    }
    const StageArgs a = rk4_stage_args(sv, stage);
    rc = launch_stage(s.precision, s.order, s.equation, a, st);
    if (!rc) sv->launches++;
    return rc;
}

int write_scalar(SolverDev &s, int idx, double v) {
    DGX_TRY_CUDA(cudaMemcpy(s.scal + idx, &v, sizeof(double), cudaMemcpyHostToDevice));
    return DGX_OK;
}

}  // namespace

StageArgs make_stage_args(dgx_solver *sv, int mode, const void *u, const void *c, void *acc,
                          void *out, double dt, double t) {
    SolverDev &s = sv->s;
    const MeshDev &m = sv->mesh->d;
    StageArgs a;
    a.E = m.num_elem;
    a.mode = mode;
    a.flux = s.flux;
    a.gamma = s.gamma;
    a.ax = s.ax;
    a.ay = s.ay;
    a.gammaf = static_cast<float>(s.gamma);
    a.axf = static_cast<float>(s.ax);
    a.ayf = static_cast<float>(s.ay);
    // the epilogue operands of stages 2-4 are the solver's own buffers (16-byte
    // slack at their end for the widened prefetch slices)
    const bool comp_pre = s.precision == DGX_FP32_COMP && mode == 1;   // the low part into stage 1
    if (s.prefetch && ((mode >= 2 && mode <= 4) || comp_pre) && c && acc) {
        const int align = 16 / static_cast<int>(elem_size(s));   // values per 16 bytes
        a.prefetch = m.num_elem % align == 0 ? kTile : kTile + align;
    } else {
        a.prefetch = 0;
    }
    a.status = s.status;
    a.u = u;
    a.c = c;
    a.acc = acc;
    a.out = out;
    a.nbr = m.nbr;
    a.halo_off = m.halo_off;
    a.halo_list = m.halo_list;
    a.nslot = 3 * kTile + m.max_halo;
    a.scal = s.scal;
    a.dt = dt;
    a.t = t;
    // stage node c_s by kernel mode: RK4 (1..4) 0, 1/2, 1/2, 1; RK2 (5, 6) 0,
    // 1/2; forward Euler (5) 0
    static const double kNode[7] = {0.0, 0.0, 0.5, 0.5, 1.0, 0.0, 0.5};
    double node = kNode[mode < 0 || mode > 6 ? 0 : mode];
    if (s.stage_time == DGX_STAGE_TIME_REFERENCE)   // t_{n+1} + c_s dt (Euler RK4/RK2) or t_n
        node = (s.equation == DGX_EULER && s.integrator != DGX_FE) ? 1.0 + node : 0.0;
    a.stage_c = node;
    a.alpha = (mode == 5 && s.integrator == DGX_RK2) ? 0.5 : 1.0;
    a.bc_kind = s.bc_kind;
    a.bc_ic = s.bc_ic;
    a.hook_float = s.hook_math == DGX_HOOK_MATH_REFERENCE ? 1 : 0;
    for (int i = 0; i < 4; ++i) a.bc_state[i] = s.bc_state[i];
    for (int i = 0; i < 8; ++i) a.bc_params[i] = s.bc_params[i];
    a.V = m.V;
    a.bnd = m.num_boundary > 0 ? 1 : 0;
    a.tc_img = s.precision == DGX_FP32_BF16X3 ? tc_image(s.order) : nullptr;
    if (s.precision == DGX_FP64) {
        a.geo = m.geo64;
        a.fn = m.fn64;
    } else {
        a.geo = m.geo32;
        a.fn = m.fn32;
    }
    a.aux = nullptr;
    a.rk13 = 0;
    a.comp = 0;
    return a;
}

// Classic RK4 (time_integrator.cu:194-218) over the buffers c (state), ua, ub
// (stage inputs) and acc.  The reference keeps k1..k4; the 16-pass fused form
// keeps acc = c + k1/6 (+ k2/3 + k3/3) written by every stage.  The 13-pass
// form writes the accumulator once: with u2 = c + k1/2 and u3 = c + k2/2,
//   c + k1/6 + k2/3 + k3/3 = c + ((u2 - c) + 2 (u3 - c) + k3) / 3,
// so stage 1 reads c and writes u2 (2 passes), stage 2 reads u2 and c and
// writes u3 (3), stage 3 reads u3, c and u2 and writes u4 = c + k3 over u2 and
// the accumulator (5), stage 4 reads u4 and the accumulator and writes c (3).
// The differences u2 - c, u3 - c are exact (Sterbenz) for steps that change a
// coefficient by less than half its value, so the accumulator's rounding is
// of the order of the 16-pass form's.
//
// DGX_FP32_COMP keeps the increments apart from the state and the state as
// c + lo (19 state passes: 4, 5, 5, 5): stage 1 reads c and lo and writes
// u2 = c + k1/2 and D = lo + k1/6 (in acc); stages 2, 3 read their input, c and
// D and write u3 = c + k2/2 (u4 = c + k3) and D + k/3; stage 4 reads u4, c and
// D and writes the two-sum of c and D + k4/6 as the new (c, lo).  The FP32
// rounding of u2..u4, which only feed the right-hand sides, costs ~1e-7 over
// thousands of steps; the rounding of a stored state, which the plain forms
// accumulate step after step, none.
StageArgs rk4_stage_args(dgx_solver *sv, int stage) {
    SolverDev &s = sv->s;
    const bool rk13 = !s.limiter && s.precision != DGX_FP32_COMP;
    StageArgs a;
    switch (stage) {
    case 0: a = make_stage_args(sv, 1, s.c, s.c, s.acc, s.ua, 0.0, 0.0); break;
    case 1: a = make_stage_args(sv, 2, s.ua, s.c, s.acc, s.ub, 0.0, 0.0); break;
    case 2: a = make_stage_args(sv, 3, s.ub, s.c, s.acc, s.ua, 0.0, 0.0); break;
    default: a = make_stage_args(sv, 4, s.ua, s.c, s.acc, s.c, 0.0, 0.0); break;
    }
    a.rk13 = rk13 ? 1 : 0;
    if (rk13 && stage == 2) a.aux = s.ua;   // u2, overwritten in place by u4
    if (s.precision == DGX_FP32_COMP) {
        a.comp = 1;
        if (stage == 0 || stage == 3) a.aux = s.lo;   // read by stage 1, written by stage 4
    }
    return a;
}

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}


int mesh_build(int num_elem, int num_sides, const double *const Vs[6], const int *const es[3],
               const int *const sd[4], BlockPool *pool, cudaStream_t st, const MeshBuildAsync *async,
               dgx_mesh **out) {
    if (!out) { set_error("out is NULL"); return DGX_ERR_INVALID; }
    *out = nullptr;
    if (num_elem <= 0 || num_sides <= 0 || num_elem > (1 << 28)) {
        set_error("num_elem must be in 1..2^28 and num_sides >= 1");
        return DGX_ERR_INVALID;
    }
    for (int i = 0; i < 6; ++i) if (!Vs[i]) { set_error("vertex array is NULL"); return DGX_ERR_INVALID; }
    for (int i = 0; i < 3; ++i) if (!es[i]) { set_error("elem_s array is NULL"); return DGX_ERR_INVALID; }
    for (int i = 0; i < 4; ++i) if (!sd[i]) { set_error("side array is NULL"); return DGX_ERR_INVALID; }
    const double *V1x = Vs[0], *V1y = Vs[1], *V2x = Vs[2], *V2y = Vs[3], *V3x = Vs[4], *V3y = Vs[5];
    const int *left_elem = sd[0], *right_elem = sd[1], *left_side_number = sd[2], *right_side_number = sd[3];
    // host validation of the connectivity (the reference trusts its mesh file)
    int nb = 0;
    for (int s = 0; s < num_sides; ++s) {
        const int L = left_elem[s], Rr = right_elem[s], ls = left_side_number[s], rs = right_side_number[s];
        if (L < 0 || L >= num_elem || ls < 0 || ls > 2) { set_error("side %d: bad left element/side", s); return DGX_ERR_INVALID; }
        if (es[ls][L] != s) { set_error("side %d: elem_s of its left element does not point back", s); return DGX_ERR_INVALID; }
        if (Rr >= 0) {
            if (Rr >= num_elem || rs < 0 || rs > 2) { set_error("side %d: bad right element/side", s); return DGX_ERR_INVALID; }
            if (Rr == L) { set_error("side %d: left and right element coincide", s); return DGX_ERR_INVALID; }
            if (es[rs][Rr] != s) { set_error("side %d: elem_s of its right element does not point back", s); return DGX_ERR_INVALID; }
        } else {
            if (Rr < -3) { set_error("side %d: boundary tag %d outside -3..-1", s, Rr); return DGX_ERR_INVALID; }
            ++nb;
        }
    }
    for (int e = 0; e < num_elem; ++e) {
        for (int k = 0; k < 3; ++k)
            if (es[k][e] < 0 || es[k][e] >= num_sides) { set_error("element %d: side index out of range", e); return DGX_ERR_INVALID; }
        const double J = (V2x[e] - V1x[e]) * (V3y[e] - V1y[e]) - (V3x[e] - V1x[e]) * (V2y[e] - V1y[e]);
        if (!(J > 0.0)) { set_error("element %d is not counter-clockwise (J = %g)", e, J); return DGX_ERR_INVALID; }
    }

    dgx_mesh *m = new (std::nothrow) dgx_mesh();
    if (!m) { set_error("host allocation failed"); return DGX_ERR_NOMEM; }
    cudaGetDevice(&m->device);
    MeshDev &d = m->d;
    d.num_elem = num_elem;
    d.num_sides = num_sides;
    d.num_boundary = nb;
    const size_t E = num_elem, S = num_sides;
    std::vector<int> words, hoff, hlist;
    build_tiles(num_elem, es, left_elem, right_elem, left_side_number, right_side_number, words,
                hoff, hlist, d.max_halo);
    d.num_tiles = static_cast<int>(hoff.size()) - 1;
    d.total_halo = static_cast<int>(hlist.size());
    // one block: the arrays uploaded from the host first (one copy), then the
    // ones the geometry kernels compute, then the reduction scratch
    BlockLayout L;
    const size_t oV = L.take<double>(6 * E), oEs = L.take<int>(3 * E), oSd = L.take<int>(4 * S),
                 oNbr = L.take<int>(3 * E), oHoff = L.take<int>(hoff.size()), oHl = L.take<int>(hlist.size());
    const size_t upload = L.size;
    const size_t oJ = L.take<double>(E), oXr = L.take<double>(E), oYr = L.take<double>(E),
                 oXs = L.take<double>(E), oYs = L.take<double>(E), oDiam = L.take<double>(E),
                 oLen = L.take<double>(S), oNx = L.take<double>(S), oNy = L.take<double>(S),
                 oG32 = L.take<float>(5 * E), oF32 = L.take<float>(9 * E), oG64 = L.take<double>(5 * E),
                 oF64 = L.take<double>(9 * E);
    // the minimum-diameter reduction: one partial per block of its fixed grid, then the result
    const int red_len = static_cast<int>(std::min<size_t>((E + 255) / 256, kReduceLen));
    const size_t oRed = L.take<double>(red_len + 1);
    int rc = block_alloc(m->block, L.size, pool);
    if (rc) { delete m; return rc; }
    const DeviceBlock &b = m->block;
    d.V = block_at<double>(b, oV); d.elem_s = block_at<int>(b, oEs); d.sides = block_at<int>(b, oSd);
    d.nbr = block_at<int>(b, oNbr); d.halo_off = block_at<int>(b, oHoff); d.halo_list = block_at<int>(b, oHl);
    d.J = block_at<double>(b, oJ); d.xr = block_at<double>(b, oXr); d.yr = block_at<double>(b, oYr);
    d.xs = block_at<double>(b, oXs); d.ys = block_at<double>(b, oYs); d.diam = block_at<double>(b, oDiam);
    d.len = block_at<double>(b, oLen); d.nx = block_at<double>(b, oNx); d.ny = block_at<double>(b, oNy);
    d.geo32 = block_at<float>(b, oG32); d.fn32 = block_at<float>(b, oF32);
    d.geo64 = block_at<double>(b, oG64); d.fn64 = block_at<double>(b, oF64);
    std::vector<unsigned char> pageable;
    unsigned char *stage = async && async->stage ? async->stage(upload) : nullptr;
    if (!stage) {
        pageable.assign(upload, 0);
        stage = pageable.data();
    }
    auto put = [&](size_t off, const void *src, size_t bytes) {
        if (bytes) std::memcpy(stage + off, src, bytes);
    };
    for (int i = 0; i < 6; ++i) put(oV + i * E * sizeof(double), Vs[i], E * sizeof(double));
    for (int i = 0; i < 3; ++i) put(oEs + i * E * sizeof(int), es[i], E * sizeof(int));
    for (int i = 0; i < 4; ++i) put(oSd + i * S * sizeof(int), sd[i], S * sizeof(int));
    put(oNbr, words.data(), words.size() * sizeof(int));
    put(oHoff, hoff.data(), hoff.size() * sizeof(int));
    put(oHl, hlist.data(), hlist.size() * sizeof(int));
    // from pageable memory the call returns once the bytes are staged, so
    // `pageable` may go; pinned staging belongs to the caller
    const cudaError_t ce = cudaMemcpyAsync(b.base, stage, upload, cudaMemcpyHostToDevice, st);
    if (ce != cudaSuccess) { set_error("mesh upload failed: %s", cudaGetErrorString(ce)); mesh_free(m); return DGX_ERR_CUDA; }
    rc = mesh_geometry(d, block_at<double>(b, oRed), red_len, async ? async->min_diam : nullptr, st);
    if (!rc && !async && cudaStreamSynchronize(st) != cudaSuccess) { set_error("geometry kernels failed"); rc = DGX_ERR_CUDA; }
    if (rc) {
        if (async) cudaStreamSynchronize(st);   // queued work may still read the block
        mesh_free(m);
        return rc;
    }
    *out = m;
    return DGX_OK;
}

int solver_build(dgx_mesh *mesh, const dgx_solver_desc *desc, BlockPool *pool, const double *scal_init,
                 cudaStream_t st, dgx_solver **out) {
    if (!mesh || !desc || !out) { set_error("NULL argument"); return DGX_ERR_INVALID; }
    *out = nullptr;
    if (desc->order < 0 || desc->order > kMaxOrder) { set_error("order %d outside 0..%d", desc->order, kMaxOrder); return DGX_ERR_UNSUPPORTED; }
    if (desc->equation != DGX_ADVECTION && desc->equation != DGX_EULER) { set_error("unknown equation"); return DGX_ERR_INVALID; }
    if (desc->flux != DGX_FLUX_CENTRAL && desc->flux != DGX_FLUX_LLF) { set_error("unknown flux"); return DGX_ERR_INVALID; }
    if (desc->precision != DGX_FP32 && desc->precision != DGX_FP64 && desc->precision != DGX_FP32_BF16X3 &&
        desc->precision != DGX_FP32_COMP) {
        set_error("unknown precision %d", desc->precision);
        return DGX_ERR_INVALID;
    }
    if (desc->precision == DGX_FP32_COMP && desc->integrator != DGX_RK4) {
        set_error("the compensated FP32 precision serves RK4");
        return DGX_ERR_UNSUPPORTED;
    }
    if (desc->precision == DGX_FP32_BF16X3) {
        if (desc->order < kTcMinOrder || desc->order > kTcMaxOrder) {
            set_error("the BF16x3 path serves orders %d..%d", kTcMinOrder, kTcMaxOrder);
            return DGX_ERR_UNSUPPORTED;
        }
        int rc = ensure_tensor_cores();
        if (rc) return rc;
    }
    if (desc->integrator != DGX_RK4 && desc->integrator != DGX_RK2 && desc->integrator != DGX_FE) {
        set_error("unknown integrator %d", desc->integrator);
        return DGX_ERR_INVALID;
    }
    if (desc->equation == DGX_EULER && !(desc->gamma > 1.0)) { set_error("gamma must be > 1"); return DGX_ERR_INVALID; }
    int rc = ensure_device_tables();
    if (rc) return rc;
    dgx_solver *sv = new (std::nothrow) dgx_solver();
    if (!sv) { set_error("host allocation failed"); return DGX_ERR_NOMEM; }
    SolverDev &s = sv->s;
    s.order = desc->order;
    s.np = num_modes(desc->order);
    s.nv = desc->equation == DGX_EULER ? 4 : 1;
    s.equation = desc->equation;
    s.flux = desc->flux;
    s.precision = desc->precision;
    s.gamma = desc->gamma;
    s.ax = desc->ax;
    s.ay = desc->ay;
    s.integrator = desc->integrator;
    s.n = static_cast<size_t>(s.nv) * s.np * mesh->d.num_elem;
    const size_t es = elem_size(s);
    // one block: the device scalars (scal[8], lam_bits, counter, status, steps,
    // chg_bits packed in 96 bytes), then c and ua for every integrator, and for
    // RK4 its accumulator and a second stage input, each with 64 bytes of slack
    // (the epilogue prefetch widens each slice to 16-byte boundaries)
    constexpr size_t kHdr = 96;
    BlockLayout L;
    const size_t oHdr = L.take<unsigned char>(kHdr);
    const int nbuf = s.integrator == DGX_RK4 ? (s.precision == DGX_FP32_COMP ? 5 : 4) : 2;
    size_t oBuf[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < nbuf; ++i) oBuf[i] = L.take<unsigned char>(s.n * es + 64);
    rc = block_alloc(sv->block, L.size, pool);
    if (rc) { delete sv; return rc; }
    unsigned char *hdr = block_at<unsigned char>(sv->block, oHdr);
    s.scal = reinterpret_cast<double *>(hdr);
    s.lam_bits = reinterpret_cast<unsigned long long *>(hdr + 64);
    s.counter = reinterpret_cast<unsigned int *>(hdr + 72);
    s.status = reinterpret_cast<unsigned int *>(hdr + 76);
    s.steps = reinterpret_cast<long long *>(hdr + 80);
    s.chg_bits = reinterpret_cast<unsigned long long *>(hdr + 88);
    void *bufs[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    for (int i = 0; i < nbuf; ++i) bufs[i] = block_at<unsigned char>(sv->block, oBuf[i]);
    s.c = bufs[0]; s.ua = bufs[1]; s.acc = bufs[2]; s.ub = bufs[3]; s.lo = bufs[4];
    // the scalars by a kernel (its arguments are captured at launch): a copy
    // from pageable memory would first wait for the stream
    const double def[8] = {0.0, 0.0, 0.0, 0.0, 0.7, 0.0, 0.0, 0.0};
    rc = init_solver_scalars(hdr, scal_init ? scal_init : def, st);
    cudaError_t ce = rc ? cudaErrorLaunchFailure : cudaMemsetAsync(s.c, 0, s.n * es, st);
    if (ce == cudaSuccess && s.lo) ce = cudaMemsetAsync(s.lo, 0, s.n * es, st);
    if (ce != cudaSuccess) {
        set_error("solver init failed: %s", cudaGetErrorString(ce));
        cudaStreamSynchronize(st);
        block_free(sv->block);
        delete sv;
        return DGX_ERR_CUDA;
    }
    mesh->refs.fetch_add(1);
    sv->mesh = mesh;
    sv->device_bytes = L.size;
    *out = sv;
    return DGX_OK;
}

}  // namespace dgx

using namespace dgx;

extern "C" {

int dgx_version(void) { return DGX_VERSION; }

const char *dgx_last_error(void) { return g_err; }

const char *dgx_status_string(int status) {
    switch (status) {
    case DGX_OK: return "ok";
    case DGX_ERR_INVALID: return "invalid argument";
    case DGX_ERR_CUDA: return "CUDA error";
    case DGX_ERR_NOMEM: return "out of memory";
    case DGX_ERR_UNSUPPORTED: return "unsupported";
    case DGX_ERR_NONFINITE: return "non-finite or unphysical state";
    case DGX_ERR_BUSY: return "busy";
    case DGX_ERR_NOT_FOUND: return "not found";
    case DGX_ERR_TIMEOUT: return "timeout";
    default: return "unknown status";
    }
}

int dgx_tables(int p, int *dims, double *r1, double *r2, double *w, double *r_oned, double *w_oned,
               double *basis, double *grad_x, double *grad_y, double *basis_side,
               double *basis_vertex) {
    if (p < 0 || p > kMaxOrder) { set_error("order %d outside 0..%d", p, kMaxOrder); return DGX_ERR_UNSUPPORTED; }
    const Tables &T = tables(p);
    if (dims) { dims[0] = T.np; dims[1] = T.nq; dims[2] = T.nq1; }
    auto cp = [](double *dst, const double *src, int n) { if (dst) std::memcpy(dst, src, sizeof(double) * n); };
    cp(r1, T.r1, T.nq);
    cp(r2, T.r2, T.nq);
    cp(w, T.w, T.nq);
    cp(r_oned, T.s1, T.nq1);
    cp(w_oned, T.w1, T.nq1);
    cp(basis, T.phi, T.np * T.nq);
    cp(grad_x, T.gx, T.np * T.nq);
    cp(grad_y, T.gy, T.np * T.nq);
    cp(basis_side, T.side, 3 * T.np * T.nq1);
    cp(basis_vertex, T.vert, 3 * T.np);
    return DGX_OK;
}

int dgx_mesh_create(int num_elem, int num_sides, const double *V1x, const double *V1y,
                    const double *V2x, const double *V2y, const double *V3x, const double *V3y,
                    const int *elem_s1, const int *elem_s2, const int *elem_s3,
                    const int *left_elem, const int *right_elem, const int *left_side_number,
                    const int *right_side_number, dgx_mesh **out) {
    const double *Vs[6] = {V1x, V1y, V2x, V2y, V3x, V3y};
    const int *es[3] = {elem_s1, elem_s2, elem_s3};
    const int *sd[4] = {left_elem, right_elem, left_side_number, right_side_number};
    return mesh_build(num_elem, num_sides, Vs, es, sd, nullptr, nullptr, nullptr, out);
}

int dgx_mesh_destroy(dgx_mesh *mesh) {
    if (!mesh) return DGX_ERR_INVALID;
    mesh_release(mesh);
    return DGX_OK;
}

int dgx_mesh_geometry(const dgx_mesh *mesh, double *J, double *xr, double *yr, double *xs,
                      double *ys, double *diameter, double *s_length, double *Nx, double *Ny) {
    if (!mesh) return DGX_ERR_INVALID;
    const MeshDev &d = mesh->d;
    const size_t E = d.num_elem * sizeof(double), S = d.num_sides * sizeof(double);
    struct { double *h; const double *dv; size_t n; } cps[] = {
        {J, d.J, E}, {xr, d.xr, E}, {yr, d.yr, E}, {xs, d.xs, E}, {ys, d.ys, E},
        {diameter, d.diam, E}, {s_length, d.len, S}, {Nx, d.nx, S}, {Ny, d.ny, S}};
    for (auto &c : cps)
        if (c.h) DGX_TRY_CUDA(cudaMemcpy(c.h, c.dv, c.n, cudaMemcpyDeviceToHost));
    return DGX_OK;
}

int dgx_mesh_min_diameter(const dgx_mesh *mesh, double *out) {
    if (!mesh || !out) return DGX_ERR_INVALID;
    *out = mesh->d.min_diam;
    return DGX_OK;
}

int dgx_mesh_info(const dgx_mesh *mesh, int *num_elem, int *num_sides, int *num_boundary) {
    if (!mesh) return DGX_ERR_INVALID;
    if (num_elem) *num_elem = mesh->d.num_elem;
    if (num_sides) *num_sides = mesh->d.num_sides;
    if (num_boundary) *num_boundary = mesh->d.num_boundary;
    return DGX_OK;
}

int dgx_solver_create(dgx_mesh *mesh, const dgx_solver_desc *desc, dgx_solver **out) {
    int rc = solver_build(mesh, desc, nullptr, nullptr, nullptr, out);
    if (rc) return rc;
    if (cudaStreamSynchronize(nullptr) != cudaSuccess) {
        set_error("solver initialisation failed: %s", cudaGetErrorString(cudaGetLastError()));
        dgx_solver_destroy(*out);
        *out = nullptr;
        return DGX_ERR_CUDA;
    }
    return DGX_OK;
}

int dgx_solver_destroy(dgx_solver *sv) {
    if (!sv) return DGX_ERR_INVALID;
    block_free(sv->block);
    if (sv->s.prev) cudaFree(sv->s.prev);
    if (sv->s.tot_scratch) cudaFree(sv->s.tot_scratch);
    if (sv->mesh) mesh_release(sv->mesh);
    delete sv;
    return DGX_OK;
}

int dgx_solver_info(const dgx_solver *sv, int *num_vars, int *n_p, size_t *state_bytes,
                    size_t *device_bytes) {
    if (!sv) return DGX_ERR_INVALID;
    if (num_vars) *num_vars = sv->s.nv;
    if (n_p) *n_p = sv->s.np;
    if (state_bytes) *state_bytes = sv->s.n * elem_size(sv->s);
    if (device_bytes) *device_bytes = sv->device_bytes;
    return DGX_OK;
}

int dgx_set_state(dgx_solver *sv, const double *c) {
    if (!sv || !c) return DGX_ERR_INVALID;
    SolverDev &s = sv->s;
    if (s.precision == DGX_FP64) {
        DGX_TRY_CUDA(cudaMemcpy(s.c, c, s.n * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        std::vector<float> tmp(s.n);
        for (size_t i = 0; i < s.n; ++i) tmp[i] = static_cast<float>(c[i]);
        DGX_TRY_CUDA(cudaMemcpy(s.c, tmp.data(), s.n * sizeof(float), cudaMemcpyHostToDevice));
        if (s.lo) {   // the part of each value the FP32 state does not hold
            for (size_t i = 0; i < s.n; ++i) tmp[i] = static_cast<float>(c[i] - static_cast<double>(static_cast<float>(c[i])));
            DGX_TRY_CUDA(cudaMemcpy(s.lo, tmp.data(), s.n * sizeof(float), cudaMemcpyHostToDevice));
        }
    }
    return DGX_OK;
}

int dgx_get_state(dgx_solver *sv, double *c) {
    if (!sv || !c) return DGX_ERR_INVALID;
    SolverDev &s = sv->s;
    DGX_TRY_CUDA(cudaDeviceSynchronize());
    if (s.precision == DGX_FP64) {
        DGX_TRY_CUDA(cudaMemcpy(c, s.c, s.n * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        std::vector<float> tmp(s.n);
        DGX_TRY_CUDA(cudaMemcpy(tmp.data(), s.c, s.n * sizeof(float), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < s.n; ++i) c[i] = tmp[i];
        if (s.lo) {   // state = c + lo
            DGX_TRY_CUDA(cudaMemcpy(tmp.data(), s.lo, s.n * sizeof(float), cudaMemcpyDeviceToHost));
            for (size_t i = 0; i < s.n; ++i) c[i] += tmp[i];
        }
    }
    return DGX_OK;
}

int dgx_set_state_f32(dgx_solver *sv, const float *c, void *stream) {
    if (!sv || !c) return DGX_ERR_INVALID;
    SolverDev &s = sv->s;
    if (s.precision != DGX_FP64) {
        DGX_TRY_CUDA(cudaMemcpyAsync(s.c, c, s.n * sizeof(float), cudaMemcpyHostToDevice, as_stream(stream)));
        if (s.lo) DGX_TRY_CUDA(cudaMemsetAsync(s.lo, 0, s.n * sizeof(float), as_stream(stream)));
        return DGX_OK;
    }
    // stage through the (between steps unused) stage-input buffer, then widen on the device
    DGX_TRY_CUDA(cudaMemcpyAsync(s.ua, c, s.n * sizeof(float), cudaMemcpyHostToDevice, as_stream(stream)));
    return convert_state(s.ua, 0, s.c, 1, s.n, as_stream(stream));
}

int dgx_get_state_f32(dgx_solver *sv, float *c, void *stream) {
    if (!sv || !c) return DGX_ERR_INVALID;
    SolverDev &s = sv->s;
    if (s.precision != DGX_FP64) {
        DGX_TRY_CUDA(cudaMemcpyAsync(c, s.c, s.n * sizeof(float), cudaMemcpyDeviceToHost, as_stream(stream)));
        return DGX_OK;
    }
    int rc = convert_state(s.c, 1, s.ua, 0, s.n, as_stream(stream));
    if (rc) return rc;
    DGX_TRY_CUDA(cudaMemcpyAsync(c, s.ua, s.n * sizeof(float), cudaMemcpyDeviceToHost, as_stream(stream)));
    return DGX_OK;
}

int dgx_state_device_ptr(dgx_solver *sv, void **ptr) {
    if (!sv || !ptr) return DGX_ERR_INVALID;
    *ptr = sv->s.c;
    return DGX_OK;
}

int dgx_project_ic(dgx_solver *sv, int ic, const double *params) {
    const int rc = project_ic_on(sv, ic, params, nullptr);
    if (rc) return rc;
    DGX_TRY_CUDA(cudaDeviceSynchronize());
    return DGX_OK;
}

}  // extern "C"

namespace dgx {

int project_ic_on(dgx_solver *sv, int ic, const double *params, cudaStream_t st) {
    if (!sv) return DGX_ERR_INVALID;
    if (ic < DGX_IC_GAUSSIAN || ic > DGX_IC_LINEAR) { set_error("unknown initial condition %d", ic); return DGX_ERR_INVALID; }
    if (sv->s.equation == DGX_EULER && (ic == DGX_IC_GAUSSIAN || ic == DGX_IC_POLY || ic == DGX_IC_LINEAR)) {
        set_error("initial condition %d is scalar", ic);
        return DGX_ERR_INVALID;
    }
    if (sv->s.equation == DGX_ADVECTION && ic != DGX_IC_GAUSSIAN && ic != DGX_IC_POLY && ic != DGX_IC_CONSTANT &&
        ic != DGX_IC_LINEAR) {
        set_error("initial condition %d needs the Euler equations", ic);
        return DGX_ERR_INVALID;
    }
    int rc = project_ic(sv->s, sv->mesh->d, ic, params, st);
    if (rc) return rc;
    sv->launches++;
    if (sv->s.lo) DGX_TRY_CUDA(cudaMemsetAsync(sv->s.lo, 0, sv->s.n * sizeof(float), st));   // state = c
    return DGX_OK;
}

}  // namespace dgx

extern "C" {

int dgx_rhs_eval(dgx_solver *sv, const void *u, void *k, double dt, double t, void *stream) {
    if (!sv || !u || !k) return DGX_ERR_INVALID;
    if (u == k) { set_error("u and k must not alias"); return DGX_ERR_INVALID; }
    return stage_launch(sv, 0, u, nullptr, nullptr, k, dt, t, as_stream(stream));
}

int dgx_set_dt(dgx_solver *sv, int dt_mode, double dt, double cfl) {
    if (!sv) return DGX_ERR_INVALID;
    if (dt_mode != DGX_DT_FIXED && dt_mode != DGX_DT_CFL) { set_error("unknown dt mode"); return DGX_ERR_INVALID; }
    if (dt_mode == DGX_DT_FIXED && !(dt > 0.0)) { set_error("fixed dt must be > 0"); return DGX_ERR_INVALID; }
    if (dt_mode == DGX_DT_CFL && !(cfl > 0.0)) { set_error("cfl must be > 0"); return DGX_ERR_INVALID; }
    sv->s.dt_mode = dt_mode;
    int rc = write_scalar(sv->s, 3, dt_mode == DGX_DT_FIXED ? dt : 0.0);
    if (!rc) rc = write_scalar(sv->s, 4, cfl);
    return rc;
}

int dgx_set_end_time(dgx_solver *sv, double t_end) {
    if (!sv) return DGX_ERR_INVALID;
    return write_scalar(sv->s, 5, t_end);
}

int dgx_rk_stage(dgx_solver *sv, int stage, void *stream) {
    if (!sv) return DGX_ERR_INVALID;
    return run_stage(sv, stage, as_stream(stream));
}

int dgx_step(dgx_solver *sv, void *stream) {
    if (!sv) return DGX_ERR_INVALID;
    for (int st = 0; st < num_stages(sv->s.integrator); ++st) {
        int rc = run_stage(sv, st, as_stream(stream));
        if (rc) return rc;
    }
    return DGX_OK;
}

int dgx_time(dgx_solver *sv, double *t, double *dt, void *stream) {
    if (!sv) return DGX_ERR_INVALID;
    double h[3];
    DGX_TRY_CUDA(cudaMemcpyAsync(h, sv->s.scal, sizeof(h), cudaMemcpyDeviceToHost, as_stream(stream)));
    DGX_TRY_CUDA(cudaStreamSynchronize(as_stream(stream)));
    if (t) *t = h[1];
    if (dt) *dt = h[0];
    return DGX_OK;
}

int dgx_reset_time(dgx_solver *sv, double t) {
    if (!sv) return DGX_ERR_INVALID;
    int rc = write_scalar(sv->s, 1, t);
    if (!rc) rc = write_scalar(sv->s, 2, t);
    if (!rc) rc = write_scalar(sv->s, 0, 0.0);
    if (rc) return rc;
    DGX_TRY_CUDA(cudaMemset(sv->s.steps, 0, sizeof(long long)));
    DGX_TRY_CUDA(cudaMemset(sv->s.status, 0, sizeof(unsigned int)));
    return DGX_OK;
}

int dgx_run(dgx_solver *sv, double t_end, int max_steps, int *steps, double *t, void *stream) {
    if (!sv) return DGX_ERR_INVALID;
    if (!(t_end > 0.0) && max_steps <= 0) { set_error("need t_end > 0 or max_steps > 0"); return DGX_ERR_INVALID; }
    cudaStream_t st = as_stream(stream);
    int rc = write_scalar(sv->s, 5, t_end > 0.0 ? t_end : 0.0);
    if (rc) return rc;
    long long s0 = 0, sn = 0;
    DGX_TRY_CUDA(cudaMemcpy(&s0, sv->s.steps, sizeof(s0), cudaMemcpyDeviceToHost));
    int issued = 0;
    for (;;) {
        int chunk = 16;
        if (max_steps > 0 && max_steps - issued < chunk) chunk = max_steps - issued;
        for (int i = 0; i < chunk; ++i) {
            rc = dgx_step(sv, stream);
            if (rc) return rc;
        }
        issued += chunk;
        double h[2];
        unsigned int status = 0;
        DGX_TRY_CUDA(cudaMemcpyAsync(h, sv->s.scal, sizeof(h), cudaMemcpyDeviceToHost, st));
        DGX_TRY_CUDA(cudaMemcpyAsync(&sn, sv->s.steps, sizeof(sn), cudaMemcpyDeviceToHost, st));
        DGX_TRY_CUDA(cudaMemcpyAsync(&status, sv->s.status, sizeof(status), cudaMemcpyDeviceToHost, st));
        DGX_TRY_CUDA(cudaStreamSynchronize(st));
        if (status & kStatusCopyTimeout) { set_error("a bounded wait for an asynchronous copy ran out"); return DGX_ERR_TIMEOUT; }
        if (status) { set_error("state became non-finite or unphysical (flags %u)", status); return DGX_ERR_NONFINITE; }
        const bool done_t = t_end > 0.0 && (h[1] >= t_end || h[0] == 0.0);
        const bool done_n = max_steps > 0 && issued >= max_steps;
        if (done_t || done_n) {
            if (steps) *steps = static_cast<int>(sn - s0);
            if (t) *t = h[1];
            return DGX_OK;
        }
    }
}

int dgx_conserved_totals(dgx_solver *sv, double *out, void *stream) {
    if (!sv || !out) return DGX_ERR_INVALID;
    int rc = conserved_totals(sv->s, sv->mesh->d, out, as_stream(stream));
    if (!rc) sv->launches += 2 * sv->s.nv * 2;
    return rc;
}

int dgx_solver_set_boundary(dgx_solver *sv, int kind, int ic, const double *params) {
    if (!sv) return DGX_ERR_INVALID;
    SolverDev &s = sv->s;
    switch (kind) {
    case DGX_BC_NONE: s.bc_kind = 0; return DGX_OK;
    case DGX_BC_FREESTREAM: {
        if (s.equation != DGX_EULER || !params) { set_error("the free-stream state needs the Euler equations and {rho, u, v, p}"); return DGX_ERR_INVALID; }
        const double rho = params[0], u = params[1], v = params[2], p = params[3];
        if (!(rho > 0) || !(p > 0)) { set_error("free-stream density and pressure must be positive"); return DGX_ERR_INVALID; }
        s.bc_state[0] = rho;
        s.bc_state[1] = rho * u;
        s.bc_state[2] = rho * v;
        s.bc_state[3] = p / (s.gamma - 1.0) + 0.5 * rho * (u * u + v * v);
        s.bc_kind = 1;
        return DGX_OK;
    }
    case DGX_BC_EXACT:
        if (s.equation != DGX_ADVECTION || (ic != DGX_IC_GAUSSIAN && ic != DGX_IC_POLY && ic != DGX_IC_LINEAR)) {
            set_error("the exact Dirichlet boundary needs advection and a scalar initial condition");
            return DGX_ERR_INVALID;
        }
        s.bc_ic = ic;
        for (int i = 0; i < 8; ++i) s.bc_params[i] = params ? params[i] : 0.0;
        s.bc_kind = 2;
        return DGX_OK;
    case DGX_BC_PROBLEM:
        if (s.equation != DGX_EULER || ic < DGX_IC_CYLINDER || ic > DGX_IC_THREEPOINT || !params) {
            set_error("problem boundaries need the Euler equations, a problem initial condition and its params");
            return DGX_ERR_INVALID;
        }
        s.bc_ic = ic;
        for (int i = 0; i < 8; ++i) s.bc_params[i] = params[i];
        s.bc_kind = 3;
        return DGX_OK;
    default: set_error("unknown boundary kind %d", kind); return DGX_ERR_INVALID;
    }
}

int dgx_solver_set_option(dgx_solver *sv, int option, int value) {
    if (!sv) return DGX_ERR_INVALID;
    switch (option) {
    case DGX_OPT_PREFETCH: sv->s.prefetch = value ? 1 : 0; return DGX_OK;
    case DGX_OPT_LIMITER:
        if (value && sv->s.order != 1) { set_error("the limiter serves p = 1"); return DGX_ERR_UNSUPPORTED; }
        if (value && sv->s.precision == DGX_FP32_COMP) {
            set_error("the limiter changes stage states the compensated precision keeps apart from its increments");
            return DGX_ERR_UNSUPPORTED;
        }
        sv->s.limiter = value ? 1 : 0;
        return DGX_OK;
    case DGX_OPT_STAGE_TIME:
        if (value != DGX_STAGE_TIME_EXACT && value != DGX_STAGE_TIME_REFERENCE) {
            set_error("unknown stage-time rule %d", value);
            return DGX_ERR_INVALID;
        }
        sv->s.stage_time = value;
        return DGX_OK;
    case DGX_OPT_HOOK_MATH:
        if (value != DGX_HOOK_MATH_DOUBLE && value != DGX_HOOK_MATH_REFERENCE) {
            set_error("unknown hook arithmetic %d", value);
            return DGX_ERR_INVALID;
        }
        sv->s.hook_math = value;
        return DGX_OK;
    default: set_error("unknown option %d", option); return DGX_ERR_INVALID;
    }
}

int dgx_limit(dgx_solver *sv, void *stream) {
    if (!sv) return DGX_ERR_INVALID;
    if (sv->s.order != 1) { set_error("the limiter serves p = 1"); return DGX_ERR_UNSUPPORTED; }
    const int rc = limit_state(sv->s, sv->mesh->d, sv->s.c, as_stream(stream));
    if (!rc) sv->launches++;
    return rc;
}

int dgx_state_change(dgx_solver *sv, const void *prev, double *max_change, void *stream) {
    if (!sv || !prev || !max_change) return DGX_ERR_INVALID;
    const int rc = state_change(sv->s, prev, max_change, as_stream(stream));
    if (!rc) sv->launches++;
    return rc;
}

int dgx_run_steady(dgx_solver *sv, double tol, int max_steps, int *steps, double *change, void *stream) {
    if (!sv || !(tol >= 0.0) || max_steps <= 0) { set_error("need tol >= 0 and max_steps > 0"); return DGX_ERR_INVALID; }
    SolverDev &s = sv->s;
    cudaStream_t st = as_stream(stream);
    const size_t bytes = s.n * elem_size(s);
    if (!s.prev) {
        char *p = nullptr;
        int rc = dalloc(&p, bytes, &sv->device_bytes);
        if (rc) return rc;
        s.prev = p;
    }
    double chg = INFINITY;
    int n = 0;
    while (n < max_steps) {
        DGX_TRY_CUDA(cudaMemcpyAsync(s.prev, s.c, bytes, cudaMemcpyDeviceToDevice, st));
        int rc = dgx_step(sv, stream);
        if (rc) return rc;
        ++n;
        rc = state_change(s, s.prev, &chg, st);
        if (rc) return rc;
        sv->launches++;
        unsigned status = 0;
        DGX_TRY_CUDA(cudaMemcpy(&status, s.status, sizeof(status), cudaMemcpyDeviceToHost));
        if (status & kStatusCopyTimeout) { set_error("a bounded wait for an asynchronous copy ran out"); return DGX_ERR_TIMEOUT; }
        if (status) { set_error("state became non-finite or unphysical (flags %u)", status); return DGX_ERR_NONFINITE; }
        if (chg <= tol) break;
    }
    if (steps) *steps = n;
    if (change) *change = chg;
    return DGX_OK;
}

int dgx_max_wave_speed(dgx_solver *sv, double *out, void *stream) {
    if (!sv || !out) return DGX_ERR_INVALID;
    DGX_TRY_CUDA(cudaMemcpyAsync(out, sv->s.scal + 6, sizeof(double), cudaMemcpyDeviceToHost, as_stream(stream)));
    DGX_TRY_CUDA(cudaStreamSynchronize(as_stream(stream)));
    return DGX_OK;
}

int dgx_launch_count(const dgx_solver *sv, long long *count) {
    if (!sv || !count) return DGX_ERR_INVALID;
    *count = sv->launches;
    return DGX_OK;
}

}  // extern "C"
