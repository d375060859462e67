// dgx_misc.cu -- one-time and per-step support kernels: FP64 geometry,
// initial-condition projection, the on-device CFL time step, deterministic
// conserved-total reductions and state conversions.
#include <cmath>
#include <vector>

#include <cstring>

#include "dgx_internal.h"
#include "dgx_ic.cuh"

namespace dgx {

namespace {

constexpr int kThreads = 256;

Tables *g_dev_tables[64] = {nullptr};   // FP64 tables per device, p = 0..kMaxOrder

int dev_tables(const Tables **out) {
    int dev = 0;
    DGX_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device index out of range"); return DGX_ERR_UNSUPPORTED; }
    if (!g_dev_tables[dev]) {
        Tables host[kMaxOrder + 1];
        for (int p = 0; p <= kMaxOrder; ++p) host[p] = tables(p);
        Tables *d = nullptr;
        DGX_TRY_CUDA(cudaMalloc(&d, sizeof(host)));
        DGX_TRY_CUDA(cudaMemcpy(d, host, sizeof(host), cudaMemcpyHostToDevice));
        g_dev_tables[dev] = d;
    }
    *out = g_dev_tables[dev];
    return DGX_OK;
}

// ---------------------------------------------------------------------------
// Geometry (FP64), src/2d/conservation/conserv_kernels.cu:338-514
// ---------------------------------------------------------------------------
__global__ void elem_geometry_kernel(MeshDev m) {
    const int E = m.num_elem;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const size_t SE = E;
    const double x1 = m.V[e], y1 = m.V[SE + e], x2 = m.V[2 * SE + e], y2 = m.V[3 * SE + e];
    const double x3 = m.V[4 * SE + e], y3 = m.V[5 * SE + e];
    const double J = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
    m.J[e] = J;
    m.xr[e] = x2 - x1; m.yr[e] = y2 - y1;
    m.xs[e] = x3 - x1; m.ys[e] = y3 - y1;
    // inscribed-circle diameter 2 area / semi-perimeter (Heron, :355-373)
    const double a = hypot(x1 - x2, y1 - y2), b = hypot(x2 - x3, y2 - y3), c = hypot(x1 - x3, y1 - y3);
    const double k = 0.5 * (a + b + c);
    m.diam[e] = 2.0 * sqrt(k * (k - a) * (k - b) * (k - c)) / k;
    m.geo32[e] = static_cast<float>(1.0 / J);
    m.geo32[SE + e] = static_cast<float>(x2 - x1);
    m.geo32[2 * SE + e] = static_cast<float>(y2 - y1);
    m.geo32[3 * SE + e] = static_cast<float>(x3 - x1);
    m.geo32[4 * SE + e] = static_cast<float>(y3 - y1);
    m.geo64[e] = 1.0 / J;
    m.geo64[SE + e] = x2 - x1;
    m.geo64[2 * SE + e] = y2 - y1;
    m.geo64[3 * SE + e] = x3 - x1;
    m.geo64[4 * SE + e] = y3 - y1;
}

// length and unit normal of each side, from the left element's local side,
// oriented away from the left element's opposite vertex (:410-498)
__global__ void side_geometry_kernel(MeshDev m) {
    const int S = m.num_sides;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const size_t SE = m.num_elem, SS = S;
    const int L = m.sides[s], ls = m.sides[2 * SS + s];
    const double px[3] = {m.V[L], m.V[2 * SE + L], m.V[4 * SE + L]};
    const double py[3] = {m.V[SE + L], m.V[3 * SE + L], m.V[5 * SE + L]};
    const int a = ls, b = (ls + 1) % 3, o = (ls + 2) % 3;
    const double dx = px[b] - px[a], dy = py[b] - py[a];
    const double len = hypot(dx, dy);
    double nx = -dy / len, ny = dx / len;
    const double tx = px[o] - 0.5 * (px[a] + px[b]), ty = py[o] - 0.5 * (py[a] + py[b]);
    if (nx * tx + ny * ty > 0) { nx = -nx; ny = -ny; }
    m.len[s] = len; m.nx[s] = nx; m.ny[s] = ny;
}

// side factors for the hot path, per element and local side
__global__ void elem_side_kernel(MeshDev m) {
    const int E = m.num_elem;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const size_t SE = E;
    for (int k = 0; k < 3; ++k) {
        const int s = m.elem_s[k * SE + e];
        m.fn32[(3 * k + 0) * SE + e] = static_cast<float>(m.nx[s]);
        m.fn32[(3 * k + 1) * SE + e] = static_cast<float>(m.ny[s]);
        m.fn32[(3 * k + 2) * SE + e] = static_cast<float>(0.5 * m.len[s]);
        m.fn64[(3 * k + 0) * SE + e] = m.nx[s];
        m.fn64[(3 * k + 1) * SE + e] = m.ny[s];
        m.fn64[(3 * k + 2) * SE + e] = 0.5 * m.len[s];
    }
}

// deterministic block reductions (fixed tree, fixed order of partials)
template <int OP>   // 0 sum, 1 min
__device__ double red_op(double a, double b) { return OP == 0 ? a + b : fmin(a, b); }

template <int OP>
__global__ void reduce_kernel(const double *x, size_t n, double *partial, double init) {
    __shared__ double sh[kThreads];
    double acc = init;
    const size_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const size_t lo = blockIdx.x * chunk, hi = lo + chunk < n ? lo + chunk : n;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) acc = red_op<OP>(acc, x[i]);
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = red_op<OP>(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// per-element products c_{n,0,e} * J_e for the conserved totals; lo (the
// compensated precision's low part of the state, or null) is added to c first
template <typename T>
__global__ void mass_terms_kernel(const T *c, const T *lo, const double *J, int E, int np, int n, double *out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < E) {
        const size_t i = static_cast<size_t>(n) * np * E + e;
        double v = static_cast<double>(c[i]);
        if (lo) v += static_cast<double>(lo[i]);
        out[e] = v * J[e];
    }
}

// ---------------------------------------------------------------------------
// Initial conditions (FP64), conserv_kernels.cu:167-187, euler.cu:31-59
// ---------------------------------------------------------------------------
struct IcArgs { double P[8]; };

// L2 projection onto the modes: c_{n,i} = sum_q w_q U_n(x_q) phi_i(q) (the
// basis is orthonormal with the reference triangle's area folded into w).  A
// block takes kProjTile elements: its threads first evaluate the initial
// condition at every (element, point) pair into shared memory, then sum every
// (element, mode) pair over the points in order, so no per-thread accumulator
// array spills and the transcendental work is done once per point.
constexpr int kProjTile = 32;

template <typename T>
__global__ void __launch_bounds__(kThreads) project_kernel(MeshDev m, const Tables *tabs, int p, int nv, int ic,
                                                           IcArgs A, double g, T *c) {
    __shared__ double sU[kMaxQuad * 4 * kProjTile];   // [q][n][element of the tile]
    const int E = m.num_elem;
    const int e0 = blockIdx.x * kProjTile;
    const Tables &Tb = tabs[p];
    const int nq = Tb.nq, np = Tb.np;
    const size_t SE = E;
    for (int idx = threadIdx.x; idx < nq * kProjTile; idx += blockDim.x) {
        const int q = idx / kProjTile, l = idx % kProjTile, e = e0 + l;
        if (e >= E) continue;
        const double v1x = m.V[e], v1y = m.V[SE + e], v2x = m.V[2 * SE + e], v2y = m.V[3 * SE + e];
        const double v3x = m.V[4 * SE + e], v3y = m.V[5 * SE + e];
        const double r = Tb.r1[q], s = Tb.r2[q];
        const double x = r * v2x + s * v3x + (1 - r - s) * v1x;
        const double y = r * v2y + s * v3y + (1 - r - s) * v1y;
        double U[4] = {0.0, 0.0, 0.0, 0.0};
        ic_eval(ic, A.P, g, x, y, U);
        for (int n = 0; n < 4; ++n) sU[(q * 4 + n) * kProjTile + l] = U[n];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < np * kProjTile; idx += blockDim.x) {
        const int i = idx / kProjTile, l = idx % kProjTile, e = e0 + l;
        if (e >= E) continue;
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int q = 0; q < nq; ++q) {
            const double wq = Tb.w[q], ph = Tb.phi[i * nq + q];
#pragma unroll
            for (int n = 0; n < 4; ++n) acc[n] += wq * sU[(q * 4 + n) * kProjTile + l] * ph;
        }
        for (int n = 0; n < nv; ++n) c[(static_cast<size_t>(n) * np + i) * SE + e] = static_cast<T>(acc[n]);
    }
}

// ---------------------------------------------------------------------------
// Time step: per-step maximum cell-average wave speed (euler.cu:252-278) and
// dt = cfl * min diameter / lambda / (2p+1), clipped at t_end
// (time_integrator.cu:252-270).  The last block to finish computes dt, so the
// whole step stays on the device.
// ---------------------------------------------------------------------------
__device__ void finish_dt(const DtArgs &a, double lam) {
    double *sc = a.scal;
    const double t = sc[1], t_end = sc[5];
    double dt;
    if (a.cfl_mode) dt = sc[4] * a.min_diam / lam / (2.0 * a.order + 1.0);
    else dt = sc[3];
    if (!(lam == lam) || !(dt > 0.0) || !isfinite(dt)) {   // NaN state or no progress possible
        atomicOr(a.status, kStatusNonFinite);
        dt = 0.0;
    }
    double tn = t + dt;
    if (t_end > 0.0) {
        if (t >= t_end) { dt = 0.0; tn = t; }
        else if (t + dt > t_end) { dt = t_end - t; tn = t_end; }
    }
    sc[0] = dt;
    sc[2] = t;
    sc[1] = tn;
    sc[6] = lam;
    if (dt > 0.0) *a.steps += 1;
}

template <typename T>
__device__ void cfl_block(const DtArgs &a, int block, int nblocks) {
    __shared__ double sh[kThreads / 32];
    double lmax = 0.0;
    unsigned int bad = 0;
    if (a.euler) {
        const T *c = static_cast<const T *>(a.c);
        const size_t SE = a.E, NPE = static_cast<size_t>(a.np) * SE;
        // in the state's precision: an FP32 state carries FP32 rounding anyway,
        // and FP64 division and square root run at a small fraction of the
        // FP32 rate on this GPU
        const T phi0 = static_cast<T>(a.phi0), gm = static_cast<T>(a.gamma);
#pragma unroll 4
        for (int e = block * blockDim.x + threadIdx.x; e < a.E; e += nblocks * blockDim.x) {
            const T rho = c[e] * phi0;
            const T ru = c[NPE + e] * phi0;
            const T rv = c[2 * NPE + e] * phi0;
            const T E = c[3 * NPE + e] * phi0;
            const T p = (gm - T(1)) * (E - (ru * ru + rv * rv) / T(2) / rho);
            if (!(rho > T(0)) || !(p > T(0))) bad |= kStatusNegative;
            const T cs = sqrt(gm * p / rho);
            const T sp = sqrt(ru * ru + rv * rv) / rho;
            const double lam = static_cast<double>(sp + cs);
            if (!(lam == lam)) bad |= kStatusNonFinite;
            else lmax = fmax(lmax, lam);
        }
    }
    for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = lmax;
    if (bad) atomicOr(a.status, bad);
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) m = fmax(m, sh[w]);
        // non-negative doubles order like their bit patterns
        atomicMax(a.lam_bits, static_cast<unsigned long long>(__double_as_longlong(m)));
        __threadfence();
        const unsigned int done = atomicAdd(a.counter, 1u);
        if (done == static_cast<unsigned>(nblocks) - 1) {
            __threadfence();
            const double lam = a.euler ? __longlong_as_double(static_cast<long long>(atomicAdd(a.lam_bits, 0ull)))
                                       : a.amax;
            const unsigned int st = atomicAdd(a.status, 0u);
            finish_dt(a, st ? __longlong_as_double(0x7ff8000000000000ll) : lam);
            *a.lam_bits = 0ull;
            *a.counter = 0u;
        }
    }
}

template <typename T>
__global__ void cfl_kernel(DtArgs a) {
    cfl_block<T>(a, blockIdx.x, gridDim.x);
}

__global__ void batch_cfl_kernel(const DtArgs *args, const int2 *items, int n_items) {
    for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
        const int2 w = items[it];
        const DtArgs a = args[w.x];
        if (a.is_double) cfl_block<double>(a, w.y, a.nblocks);
        else cfl_block<float>(a, w.y, a.nblocks);
        __syncthreads();
    }
}

template <typename T>
__global__ void convert_kernel(const void *src, int src_double, T *dst, size_t n) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        dst[i] = src_double ? static_cast<T>(static_cast<const double *>(src)[i])
                            : static_cast<T>(static_cast<const float *>(src)[i]);
}

int blocks_for(size_t n) { return static_cast<int>((n + kThreads - 1) / kThreads); }

// deterministic reduction of x[0..n) with a fixed grid (scratch_len partials);
// the result to the device double *result
int reduce_dev(const double *x, size_t n, int op, double *scratch, int scratch_len, double *result,
               cudaStream_t st) {
    int grid = static_cast<int>((n + kThreads - 1) / kThreads);
    if (grid > scratch_len) grid = scratch_len;
    if (grid < 1) grid = 1;
    if (op == 0) reduce_kernel<0><<<grid, kThreads, 0, st>>>(x, n, scratch, 0.0);
    else reduce_kernel<1><<<grid, kThreads, 0, st>>>(x, n, scratch, INFINITY);
    DGX_CHECK_LAUNCH();
    if (op == 0) reduce_kernel<0><<<1, kThreads, 0, st>>>(scratch, grid, result, 0.0);
    else reduce_kernel<1><<<1, kThreads, 0, st>>>(scratch, grid, result, INFINITY);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

// the same, result to *host (synchronous)
int reduce_host(const double *x, size_t n, int op, double *scratch, int scratch_len, double *host,
                cudaStream_t st) {
    const int rc = reduce_dev(x, n, op, scratch, scratch_len, scratch + scratch_len, st);
    if (rc) return rc;
    DGX_TRY_CUDA(cudaMemcpyAsync(host, scratch + scratch_len, sizeof(double), cudaMemcpyDeviceToHost, st));
    DGX_TRY_CUDA(cudaStreamSynchronize(st));
    return DGX_OK;
}

}  // namespace

int upload_tables_misc() {
    const Tables *t = nullptr;
    return dev_tables(&t);
}

int mesh_geometry(MeshDev &m, double *scratch, int scratch_len, double *min_diam_dst, cudaStream_t st) {
    const int E = m.num_elem, S = m.num_sides;
    elem_geometry_kernel<<<blocks_for(E), kThreads, 0, st>>>(m);
    DGX_CHECK_LAUNCH();
    side_geometry_kernel<<<blocks_for(S), kThreads, 0, st>>>(m);
    DGX_CHECK_LAUNCH();
    elem_side_kernel<<<blocks_for(E), kThreads, 0, st>>>(m);
    DGX_CHECK_LAUNCH();
    // minimum inscribed diameter (exact: min is order independent)
    if (!min_diam_dst) return reduce_host(m.diam, E, 1, scratch, scratch_len, &m.min_diam, st);
    const int rc = reduce_dev(m.diam, E, 1, scratch, scratch_len, scratch + scratch_len, st);
    if (rc) return rc;
    DGX_TRY_CUDA(cudaMemcpyAsync(min_diam_dst, scratch + scratch_len, sizeof(double), cudaMemcpyDeviceToHost, st));
    return DGX_OK;
}

int project_ic(const SolverDev &s, const MeshDev &m, int ic, const double *params, cudaStream_t st) {
    const Tables *tabs = nullptr;
    int rc = dev_tables(&tabs);
    if (rc) return rc;
    IcArgs A;
    for (int i = 0; i < 8; ++i) A.P[i] = params ? params[i] : 0.0;
    const int grid = (m.num_elem + kProjTile - 1) / kProjTile;
    if (s.precision == DGX_FP64)
        project_kernel<double><<<grid, kThreads, 0, st>>>(m, tabs, s.order, s.nv, ic, A, s.gamma,
                                                          static_cast<double *>(s.c));
    else
        project_kernel<float><<<grid, kThreads, 0, st>>>(m, tabs, s.order, s.nv, ic, A, s.gamma,
                                                         static_cast<float *>(s.c));
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

DtArgs make_dt_args(const SolverDev &s, const MeshDev &m) {
    DtArgs a;
    a.c = s.c;
    a.E = m.num_elem;
    a.np = s.np;
    a.is_double = s.precision == DGX_FP64;
    a.euler = s.equation == DGX_EULER && s.dt_mode == DGX_DT_CFL;
    a.cfl_mode = s.dt_mode == DGX_DT_CFL;
    a.order = s.order;
    a.gamma = s.gamma;
    a.phi0 = tables(s.order).phi[0];
    a.amax = std::sqrt(s.ax * s.ax + s.ay * s.ay);
    a.min_diam = m.min_diam;
    a.scal = s.scal;
    a.lam_bits = s.lam_bits;
    a.counter = s.counter;
    a.status = s.status;
    a.steps = s.steps;
    a.nblocks = 1;
    if (a.euler) {
        a.nblocks = blocks_for(m.num_elem);
        if (a.nblocks > 152 * 8) a.nblocks = 152 * 8;
    }
    return a;
}

int launch_dt(SolverDev &s, const MeshDev &m, cudaStream_t st) {
    const DtArgs a = make_dt_args(s, m);
    if (a.is_double) cfl_kernel<double><<<a.nblocks, kThreads, 0, st>>>(a);
    else cfl_kernel<float><<<a.nblocks, kThreads, 0, st>>>(a);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

int launch_batch_dt(const DtArgs *args, const int2 *items, int n_items, cudaStream_t st) {
    int grid = n_items < 152 * 16 ? n_items : 152 * 16;
    if (grid > 0) batch_cfl_kernel<<<grid, kThreads, 0, st>>>(args, items, n_items);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

int conserved_totals(SolverDev &s, const MeshDev &m, double *out, cudaStream_t st) {
    const int E = m.num_elem;
    const int len = kReduceLen;
    // per-element terms and the reduction's partials: allocated on the first
    // call and kept with the solver, so a loop that checks conservation every
    // step neither allocates nor waits for the device in cudaFree
    if (!s.tot_scratch) {
        void *p = nullptr;
        if (cudaMalloc(&p, sizeof(double) * (static_cast<size_t>(E) + len + 1)) != cudaSuccess) {
            cudaGetLastError();
            set_error("cudaMalloc of %zu bytes for the totals failed", sizeof(double) * (static_cast<size_t>(E) + len + 1));
            return DGX_ERR_NOMEM;
        }
        s.tot_scratch = static_cast<double *>(p);
    }
    double *terms = s.tot_scratch;
    double *scratch = s.tot_scratch + E;
    const double phi0 = tables(s.order).phi[0];
    int rc = DGX_OK;
    for (int n = 0; n < s.nv && rc == DGX_OK; ++n) {
        if (s.precision == DGX_FP64)
            mass_terms_kernel<double><<<blocks_for(E), kThreads, 0, st>>>(
                static_cast<const double *>(s.c), nullptr, m.J, E, s.np, n, terms);
        else
            mass_terms_kernel<float><<<blocks_for(E), kThreads, 0, st>>>(
                static_cast<const float *>(s.c), static_cast<const float *>(s.lo), m.J, E, s.np, n, terms);
        if (cudaGetLastError() != cudaSuccess) { rc = DGX_ERR_CUDA; break; }
        double sum = 0.0;
        rc = reduce_host(terms, E, 0, scratch, len, &sum, st);
        out[n] = sum * phi0 * 0.5;
    }
    return rc;
}

namespace {
struct Words12 { unsigned long long w[12]; };
__global__ void init_words_kernel(unsigned long long *dst, Words12 v) {
    if (threadIdx.x < 12) dst[threadIdx.x] = v.w[threadIdx.x];
}
}  // namespace

int init_solver_scalars(void *hdr, const double *scal8, cudaStream_t st) {
    Words12 v{};
    std::memcpy(v.w, scal8, 8 * sizeof(double));
    init_words_kernel<<<1, 32, 0, st>>>(static_cast<unsigned long long *>(hdr), v);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

int conserved_sums_async(const SolverDev &s, const MeshDev &m, double *terms, double *scratch,
                         double *dev_sums, cudaStream_t st) {
    const int E = m.num_elem;
    for (int n = 0; n < s.nv; ++n) {
        if (s.precision == DGX_FP64)
            mass_terms_kernel<double><<<blocks_for(E), kThreads, 0, st>>>(
                static_cast<const double *>(s.c), nullptr, m.J, E, s.np, n, terms);
        else
            mass_terms_kernel<float><<<blocks_for(E), kThreads, 0, st>>>(
                static_cast<const float *>(s.c), static_cast<const float *>(s.lo), m.J, E, s.np, n, terms);
        DGX_CHECK_LAUNCH();
        const int rc = reduce_dev(terms, E, 0, scratch, kReduceLen, dev_sums + n, st);
        if (rc) return rc;
    }
    return DGX_OK;
}

int convert_state(const void *src, int src_is_double, void *dst, int dst_is_double, size_t n,
                  cudaStream_t st) {
    int grid = blocks_for(n);
    if (grid > 152 * 16) grid = 152 * 16;
    if (dst_is_double) convert_kernel<double><<<grid, kThreads, 0, st>>>(src, src_is_double, static_cast<double *>(dst), n);
    else convert_kernel<float><<<grid, kThreads, 0, st>>>(src, src_is_double, static_cast<float *>(dst), n);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

// Forward Euler's commit of the new state: dst = src for `words` 32-bit words,
// unless the step did not advance (dt == 0 at the end time: the stage kernel
// then wrote nothing).  16-byte vectors when both ends are 16-byte aligned.
__global__ void commit_kernel(const unsigned *__restrict__ src, unsigned *__restrict__ dst, size_t words,
                              const double *__restrict__ scal) {
    if (scal[0] == 0.0) return;
    const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
    size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
    size_t done = 0;
    if (vec) {
        const size_t nv = words / 4;
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
        for (size_t j = i; j < nv; j += stride) d4[j] = s4[j];
        done = nv * 4;
    }
    for (size_t j = done + i; j < words; j += stride) dst[j] = src[j];
}

int commit_state(const SolverDev &s, void *dst, const void *src, cudaStream_t st) {
    const size_t words = s.n * (s.precision == DGX_FP64 ? 2 : 1);
    int grid = blocks_for(words / 4 + 1);
    if (grid > 152 * 8) grid = 152 * 8;
    commit_kernel<<<grid, kThreads, 0, st>>>(static_cast<const unsigned *>(src), static_cast<unsigned *>(dst), words,
                                             s.scal);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

}  // namespace dgx
