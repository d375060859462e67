// ref_gpu_harness.cu -- TEST INFRASTRUCTURE ONLY (a test reference and a reported
// baseline, never the product path).
//
// Runs the reference's own CUDA solvers, compiled from its unmodified sources,
// on a mesh and initial state given in a binary file, and writes the state they
// reach.  Built twice (oracle/Makefile):
//  * Euler (default): src/2d/conservation (conserv.cu, conserv_kernels.cu,
//    conserv_kernels_wrappers.cu, time_integrator.cu, main.cu, euler/euler.cu)
//    and src/2d/{quadrature,basis}.cu.  This file plays the part of the
//    reference's problem file (src/2d/conservation/euler/supersonic/
//    supersonic.cu:1-124): the physics hooks, and a driver that repeats
//    run_dgcuda's set-up (src/2d/conservation/main.cu:54-170) with the arrays
//    filled directly instead of read_mesh and the initial coefficients set
//    directly instead of init_conditions, then calls the reference's own
//    time_integrate_rk4 (src/2d/conservation/time_integrator.cu:221-434)
//    unchanged (CFL time step, run to t_end).
//  * Advection (-DREF_ADVECTION): src/2d/2dadvec (2dadvec.cu with its kernels
//    and wrappers) and src/2d/{time_integrator,quadrature,basis}.cu.  The
//    driver repeats src/2d/main.cu:40-196 the same way and calls that
//    time_integrate_rk4 (src/2d/time_integrator.cu:89-315) unchanged (fixed dt,
//    a number of steps); boundary sides tagged -1 take its exact data
//    (boundary_exact, 2dadvec_kernels.cu:184-186).
//  * Euler with a problem file's own hooks (-DREF_PROBLEM=1, 2, 3: the
//    cylinder, supersonic-vortex and three-point files) for meshes with
//    boundary sides.
//
// Three build adaptations, made here rather than in the reference's files:
//  * cudaThreadSynchronize (removed in CUDA 13) maps to cudaDeviceSynchronize;
//  * cudaMemcpyToSymbol with a symbol NAME (a string; the runtime dropped that
//    form) resolves the name to the symbol below;
//  * __syncthreads() compiles to nothing.  The reference calls it inside
//    `if (idx < n)` blocks of its per-side and per-element kernels, which use
//    no shared memory: a barrier some threads of a block never reach.  Its only
//    kernels with shared memory, the min/max reductions, are not called (the
//    set-up takes the minimum radius on the host, as run_dgcuda does).
// printf is routed to a counter: the Euler time loop prints "\rt = ..." once
// per step, which gives the number of steps taken.
//
// Usage: ref_gpu_euler|ref_gpu_cylinder|ref_gpu_supersonic|ref_gpu_threepoint|ref_gpu_advec <in.bin> <out.bin>
//   in:  int32 E, S, p, steps, rk2 (Euler: 1 runs time_integrate_rk2), 0;
//        double t (Euler: end time; advection: dt);
//        double V[6][E] (V1x V1y V2x V2y V3x V3y); int32 elem_s[3][E];
//        int32 sides[4][S] (left_elem right_elem left_side right_side);
//        double c[NV][Np][E] (NV = 4 Euler, 1 advection)
//   out: int32 steps, 0; double seconds (time_integrate_rk4, wall clock),
//        min_r (Euler; 0 for advection); double c[NV][Np][E]
#include <cuda_runtime.h>

#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define cudaThreadSynchronize cudaDeviceSynchronize

static cudaError_t ref_symbol_copy(const char *name, const void *src, size_t count);
// the name-based form the reference calls (conserv_kernels.cu:73-106)
cudaError_t cudaMemcpyToSymbol(const char *name, const void *src, size_t count, size_t offset = 0,
                               cudaMemcpyKind kind = cudaMemcpyHostToDevice) {
    (void)offset;
    (void)kind;
    return ref_symbol_copy(name, src, count);
}

static int g_steps = 0;
static int ref_printf(const char *fmt, ...) {
    if (std::strncmp(fmt, "\rt = ", 5) == 0) ++g_steps;
    return 0;
}

#ifndef REF_PROBLEM
#define REF_PROBLEM 0
#endif
#define printf ref_printf
#define __syncthreads() ((void)0)
#if REF_ADVECTION
#include "2dadvec/2dadvec.cu"
#elif REF_PROBLEM == 1
// the reference's cylinder problem file, its own hooks (its main renamed)
#define main ref_problem_main
#include "conservation/euler/cylinder/cylinder.cu"
#undef main
#elif REF_PROBLEM == 2
// the reference's supersonic-vortex problem file, its own hooks
#define main ref_problem_main
#include "conservation/euler/supersonic/supersonic.cu"
#undef main
#elif REF_PROBLEM == 3
// the reference's three-point shock problem file, its own hooks
#define main ref_problem_main
#include "conservation/euler/threepoint/threepoint.cu"
#undef main
#else
#include "conservation/euler/euler.cu"
#endif
#undef __syncthreads
#undef printf

#if REF_ADVECTION
constexpr int kVars = 1;
#else
constexpr int kVars = 4;
#endif
#if !REF_ADVECTION && REF_PROBLEM == 0
// ---- the problem: periodic meshes only, gamma 1.4 -------------------------
int limiter = NO_LIMITER;
int time_integrator = RK4;

__device__ double get_GAMMA() { return 1.4; }
__device__ void U0(double *U, double x, double y) {   // unused: the state is set directly
    (void)x;
    (void)y;
    U[0] = 1.0;
    U[1] = 0.0;
    U[2] = 0.0;
    U[3] = 1.0 / 0.4;
}
__device__ void U_inflow(double *U, double x, double y, double t) { U0(U, x, y); (void)t; }
__device__ void U_outflow(double *U, double x, double y, double t) { U0(U, x, y); (void)t; }
__device__ void reflecting_boundary(double *U_left, double *U_right, double v1x, double v1y, double v2x,
                                    double v2y, double v3x, double v3y, double nx, double ny, int j,
                                    int left_side, int n_quad1d) {
    for (int n = 0; n < 4; ++n) U_right[n] = U_left[n];
    (void)v1x; (void)v1y; (void)v2x; (void)v2y; (void)v3x; (void)v3y;
    (void)nx; (void)ny; (void)j; (void)left_side; (void)n_quad1d;
}

#endif

static cudaError_t ref_symbol_copy(const char *name, const void *src, size_t count) {
#define REF_SYMBOL(s) \
    if (std::strcmp(name, #s) == 0) return cudaMemcpyToSymbol(s, src, count);
#if !REF_ADVECTION
    REF_SYMBOL(N)
#endif
    REF_SYMBOL(basis)
    REF_SYMBOL(basis_grad_x)
    REF_SYMBOL(basis_grad_y)
    REF_SYMBOL(basis_side)
    REF_SYMBOL(basis_vertex)
    REF_SYMBOL(w)
    REF_SYMBOL(w_oned)
    REF_SYMBOL(r1)
    REF_SYMBOL(r2)
    REF_SYMBOL(r_oned)
#undef REF_SYMBOL
    std::fprintf(stderr, "unknown symbol %s\n", name);
    return cudaErrorInvalidSymbol;
}

template <typename T>
static bool read_vec(FILE *f, std::vector<T> &v, size_t n) {
    v.resize(n);
    return std::fread(v.data(), sizeof(T), n, f) == n;
}

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE *fi = std::fopen(argv[1], "rb");
    if (!fi) { std::fprintf(stderr, "cannot open %s\n", argv[1]); return 2; }
    int hdr[6];
    double t_in = 0.0;   // Euler: end time; advection: dt
    if (std::fread(hdr, sizeof(int), 6, fi) != 6 || std::fread(&t_in, sizeof(double), 1, fi) != 1) {
        std::fprintf(stderr, "bad header\n");
        return 2;
    }
    const int num_elem = hdr[0], num_sides = hdr[1], n = hdr[2], timesteps = hdr[3], use_rk2 = hdr[4];
    if (num_elem <= 0 || num_sides <= 0 || n < 0 || n > 5 || !(t_in > 0.0) || (REF_ADVECTION && timesteps < 1) ||
        use_rk2 < 0 || use_rk2 > 1 || (REF_ADVECTION && use_rk2)) {
        std::fprintf(stderr, "bad sizes\n");
        return 2;
    }
    const int n_p = (n + 1) * (n + 2) / 2;
    const size_t E = num_elem, S = num_sides;
    std::vector<double> V, c0;
    std::vector<int> es, sd;
    if (!read_vec(fi, V, 6 * E) || !read_vec(fi, es, 3 * E) || !read_vec(fi, sd, 4 * S) ||
        !read_vec(fi, c0, kVars * n_p * E)) {
        std::fprintf(stderr, "short input\n");
        return 2;
    }
    std::fclose(fi);
    for (size_t s = 0; s < S; ++s) {
        const int L = sd[s], R = sd[S + s], ls = sd[2 * S + s], rs = sd[3 * S + s];
        // boundary sides: Euler -1 reflecting, -2 outflow, -3 inflow only with a
        // problem file's hooks; advection -1, the exact data of its
        // boundary_exact (2dadvec_kernels.cu:184-186), with a right side number
        // in 0..2 (its surface kernel indexes the side tables by it)
        const bool bnd_ok = REF_ADVECTION ? (R == -1 && rs >= 0 && rs <= 2)
                                          : (REF_PROBLEM != 0 && R >= -3 && R <= -1);
        if (L < 0 || L >= num_elem || ls < 0 || ls > 2 || ((R < 0 || R >= num_elem || rs < 0 || rs > 2) && !bnd_ok)) {
            std::fprintf(stderr, "side %zu: the harness takes periodic meshes, advection boundary sides -1, or Euler boundary sides with a problem file\n", s);
            return 2;
        }
    }
    for (size_t e = 0; e < 3 * E; ++e)
        if (es[e] < 0 || es[e] >= num_sides) { std::fprintf(stderr, "bad elem_s\n"); return 2; }

    double *V1x = V.data(), *V1y = V1x + E, *V2x = V1y + E, *V2y = V2x + E, *V3x = V2y + E, *V3y = V3x + E;
    int *elem_s1 = es.data(), *elem_s2 = elem_s1 + E, *elem_s3 = elem_s2 + E;
    int *left_elem = sd.data(), *right_elem = left_elem + S, *left_side_number = right_elem + S,
        *right_side_number = left_side_number + S;
    // side end points: local side k of the left element joins its vertices k and k+1
    std::vector<double> sx1(S), sy1(S), sx2(S), sy2(S);
    for (size_t s = 0; s < S; ++s) {
        const int L = left_elem[s], k = left_side_number[s];
        const double vx[3] = {V1x[L], V2x[L], V3x[L]}, vy[3] = {V1y[L], V2y[L], V3y[L]};
        sx1[s] = vx[k];
        sy1[s] = vy[k];
        sx2[s] = vx[(k + 1) % 3];
        sy2[s] = vy[(k + 1) % 3];
    }

    // the reference driver's set-up (Euler: conservation/main.cu:68-163;
    // advection: src/2d/main.cu:101-186)
#if !REF_ADVECTION
    // the integrator the problem file would pick, chosen here (init_gpu sizes
    // its stage buffers by it, conserv.cu:238-253)
    time_integrator = use_rk2 ? RK2 : RK4;
#endif
    init_gpu(num_elem, num_sides, n_p, V1x, V1y, V2x, V2y, V3x, V3y, left_side_number, right_side_number,
             sx1.data(), sy1.data(), sx2.data(), sy2.data(), elem_s1, elem_s2, elem_s3, left_elem, right_elem);
    checkCudaError("error after gpu init.");
#if REF_ADVECTION
    const int n_threads = 128;
#else
    set_N(local_N);
    const int n_threads = 256;
#endif
    const int n_blocks_elem = (num_elem / n_threads) + ((num_elem % n_threads) ? 1 : 0);
    const int n_blocks_sides = (num_sides / n_threads) + ((num_sides % n_threads) ? 1 : 0);
    double min_r = 0.0;
#if !REF_ADVECTION
    preval_inscribed_circles<<<n_blocks_elem, n_threads>>>(d_J, d_V1x, d_V1y, d_V2x, d_V2y, d_V3x, d_V3y, num_elem);
    std::vector<double> radius(E);
    cudaMemcpy(radius.data(), d_J, E * sizeof(double), cudaMemcpyDeviceToHost);
    min_r = radius[0];
    for (size_t i = 1; i < E; ++i) min_r = radius[i] < min_r ? radius[i] : min_r;
#endif
    preval_jacobian<<<n_blocks_elem, n_threads>>>(d_J, d_V1x, d_V1y, d_V2x, d_V2y, d_V3x, d_V3y, num_elem);
    cudaDeviceSynchronize();
    preval_side_length<<<n_blocks_sides, n_threads>>>(d_s_length, d_s_V1x, d_s_V1y, d_s_V2x, d_s_V2y, num_sides);
    preval_normals<<<n_blocks_sides, n_threads>>>(d_Nx, d_Ny, d_s_V1x, d_s_V1y, d_s_V2x, d_s_V2y, d_V1x, d_V1y,
                                                  d_V2x, d_V2y, d_V3x, d_V3y, d_left_side_number, num_sides);
    cudaDeviceSynchronize();
#if !REF_ADVECTION
    cudaFree(d_s_V1x);
    cudaFree(d_s_V2x);
    cudaFree(d_s_V1y);
    cudaFree(d_s_V2y);
#endif
    preval_normals_direction<<<n_blocks_sides, n_threads>>>(d_Nx, d_Ny, d_V1x, d_V1y, d_V2x, d_V2y, d_V3x, d_V3y,
                                                            d_left_elem, d_left_side_number, num_sides);
    preval_partials<<<n_blocks_elem, n_threads>>>(d_V1x, d_V1y, d_V2x, d_V2y, d_V3x, d_V3y, d_xr, d_yr, d_xs, d_ys,
                                                  num_elem);
    cudaDeviceSynchronize();
    checkCudaError("error after prevals.");
    double *r1_local, *r2_local, *w_local, *s_r, *oned_w_local;
    int n_quad, n_quad1d;
    set_quadrature(n, &r1_local, &r2_local, &w_local, &s_r, &oned_w_local, &n_quad, &n_quad1d);
    preval_basis(r1_local, r2_local, s_r, w_local, oned_w_local, n_quad, n_quad1d, n_p);
    cudaDeviceSynchronize();
    // the initial coefficients, in the reference's layout c[n][i][e]
    cudaMemcpy(d_c, c0.data(), c0.size() * sizeof(double), cudaMemcpyHostToDevice);
    checkCudaError("error before time integration.");

    cudaDeviceSynchronize();
    const auto t0 = std::chrono::steady_clock::now();
#if REF_ADVECTION
    time_integrate_rk4(t_in, n_quad, n_quad1d, n_p, n, num_elem, num_sides, 0, 0, timesteps);
    g_steps = timesteps;
#else
    if (use_rk2)
        time_integrate_rk2(n_quad, n_quad1d, n_p, n, num_elem, num_sides, t_in, min_r);
    else
        time_integrate_rk4(n_quad, n_quad1d, n_p, n, num_elem, num_sides, t_in, min_r);
#endif
    cudaDeviceSynchronize();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    checkCudaError("error after time integration.");

    std::vector<double> c(c0.size());
    cudaMemcpy(c.data(), d_c, c.size() * sizeof(double), cudaMemcpyDeviceToHost);
    FILE *fo = std::fopen(argv[2], "wb");
    if (!fo) { std::fprintf(stderr, "cannot write %s\n", argv[2]); return 2; }
    const int oh[2] = {g_steps, 0};
    std::fwrite(oh, sizeof(int), 2, fo);
    std::fwrite(&secs, sizeof(double), 1, fo);
    std::fwrite(&min_r, sizeof(double), 1, fo);
    std::fwrite(c.data(), sizeof(double), c.size(), fo);
    std::fclose(fo);
    return 0;
}
