// dgx_limit.cu -- the p = 1 slope limiter and the steady-state convergence
// monitor.
//
// Limiter.  The reference carries a "standard limiter for p = 1" (limit_c,
// src/2d/conservation/conserv_kernels.cu:522-621) whose calls are commented
// out (time_integrator.cu:302,332,363) and whose bounds umin/umax are never
// set.  This is the limiter it describes, in its Barth-Jespersen form: per
// element and conserved variable, with u0 the cell average, m/M the minimum
// and maximum of the cell averages of the element and of its neighbours across
// its three sides (a boundary side contributes the element itself), and u_j
// the trace at each side Gauss point,
//     phi_j = min(1, (M - u0)/(u_j - u0))  if u_j > u0,
//             min(1, (m - u0)/(u_j - u0))  if u_j < u0,   1 otherwise,
// the two linear modes are scaled by min_j phi_j.  The cell average is
// unchanged (the limiter is conservative) and neighbours read only cell
// averages, so the kernel limits the state in place.
//
// Convergence monitor.  The reference's disabled steady-state test
// (time_integrator.cu:247-251, 401-421; check_convergence,
// conserv_kernels.cu:943-947) takes the largest change of any coefficient in
// one step against TOL = 5e-8.  state_change computes that maximum (FP64,
// order-independent); dgx_run_steady steps until it falls below a tolerance.
#include <cmath>
#include <cstring>

#include "dgx_internal.h"

namespace dgx {
namespace {

constexpr int kThreads = 256;

struct LimitArgs {
    const int *elem_s;   // [3][E]
    const int *sides;    // [4][S]
    int E, S, nv;
    double phi0;
    double side[3][3][2];   // p = 1 traces: side[k][i][j] = phi_i at point j of side k
};

template <typename T>
__global__ void limit_kernel(T *c, LimitArgs a) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.E) return;
    const size_t E = static_cast<size_t>(a.E);
    int nb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int s = a.elem_s[k * E + e];
        const int le = a.sides[s], re = a.sides[a.S + s];
        const int other = le == e ? re : le;
        nb[k] = other >= 0 ? other : e;
    }
    for (int n = 0; n < a.nv; ++n) {
        T *cn = c + static_cast<size_t>(n) * 3 * E;
        const double c0 = static_cast<double>(cn[e]), c1 = static_cast<double>(cn[E + e]),
                     c2 = static_cast<double>(cn[2 * E + e]);
        const double u0 = c0 * a.phi0;
        double lo = u0, hi = u0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double un = static_cast<double>(cn[nb[k]]) * a.phi0;
            lo = fmin(lo, un);
            hi = fmax(hi, un);
        }
        double phi = 1.0;
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const double uj = c0 * a.side[k][0][j] + c1 * a.side[k][1][j] + c2 * a.side[k][2][j];
                const double d = uj - u0;
                double pj = 1.0;
                if (d > 0.0) pj = fmin(1.0, (hi - u0) / d);
                else if (d < 0.0) pj = fmin(1.0, (lo - u0) / d);
                phi = fmin(phi, pj);
            }
        if (phi < 1.0) {
            cn[E + e] = static_cast<T>(c1 * phi);
            cn[2 * E + e] = static_cast<T>(c2 * phi);
        }
    }
}

// largest |c - prev| as the bits of a non-negative double (order-independent max)
template <typename T>
__global__ void change_kernel(const T *c, const T *prev, size_t n, unsigned long long *out) {
    __shared__ double sh[kThreads / 32];
    double m = 0.0;
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const double d = fabs(static_cast<double>(c[i]) - static_cast<double>(prev[i]));
        m = (d == d) ? fmax(m, d) : INFINITY;   // a NaN state never reads as converged
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) b = fmax(b, sh[w]);
        atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(b)));
    }
}

}  // namespace

int limit_state(const SolverDev &s, const MeshDev &m, void *state, cudaStream_t st) {
    LimitArgs a;
    a.elem_s = m.elem_s;
    a.sides = m.sides;
    a.E = m.num_elem;
    a.S = m.num_sides;
    a.nv = s.nv;
    const Tables &T = tables(1);
    a.phi0 = T.phi[0];
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 2; ++j) a.side[k][i][j] = T.side[(k * T.np + i) * T.nq1 + j];
    const int grid = (m.num_elem + kThreads - 1) / kThreads;
    if (grid == 0) return DGX_OK;
    if (s.precision == DGX_FP64) limit_kernel<double><<<grid, kThreads, 0, st>>>(static_cast<double *>(state), a);
    else limit_kernel<float><<<grid, kThreads, 0, st>>>(static_cast<float *>(state), a);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

int state_change(const SolverDev &s, const void *prev, double *out, cudaStream_t st) {
    DGX_TRY_CUDA(cudaMemsetAsync(s.chg_bits, 0, sizeof(unsigned long long), st));
    int grid = static_cast<int>((s.n + kThreads - 1) / kThreads);
    if (grid > 152 * 8) grid = 152 * 8;
    if (grid > 0) {
        if (s.precision == DGX_FP64)
            change_kernel<double><<<grid, kThreads, 0, st>>>(static_cast<const double *>(s.c),
                                                             static_cast<const double *>(prev), s.n, s.chg_bits);
        else
            change_kernel<float><<<grid, kThreads, 0, st>>>(static_cast<const float *>(s.c),
                                                            static_cast<const float *>(prev), s.n, s.chg_bits);
        DGX_CHECK_LAUNCH();
    }
    unsigned long long bits = 0;
    DGX_TRY_CUDA(cudaMemcpyAsync(&bits, s.chg_bits, sizeof(bits), cudaMemcpyDeviceToHost, st));
    DGX_TRY_CUDA(cudaStreamSynchronize(st));
    double v;
    static_assert(sizeof(v) == sizeof(bits), "double bits");
    std::memcpy(&v, &bits, sizeof(v));
    *out = v;
    return DGX_OK;
}

}  // namespace dgx
