/*
 * dgx.h -- C ABI of the GB300-native 2D discontinuous-Galerkin RHS and time-step
 * core (a drop-in for thePerv/DGCUDA's 2D DG hot path).
 *
 * Plain C: pointers, sizes and status codes only; no CUDA or C++ types.  Streams
 * are passed as `void *` holding a `cudaStream_t` (NULL = the legacy default
 * stream).  Every function returns an int status (DGX_OK == 0, negative on
 * error) and never exits the process; `dgx_status_string` names a status and
 * `dgx_last_error` gives the message of the last failure on the calling thread.
 *
 * Layouts follow the reference:
 *   mesh    V1x..V3y[num_elem] (FP64, counter-clockwise), elem_s1..3[num_elem],
 *           left_elem/right_elem/left_side_number/right_side_number[num_sides]
 *           (src/2d/conservation/conserv.cu:118-192; right_elem < 0 marks a
 *           boundary side of type -1/-2/-3, conserv_kernels.cu:657-679);
 *   state   c[n * num_elem * n_p + i * num_elem + e] for variable n, mode i,
 *           element e (src/2d/conservation/conserv_kernels.cu:21,183), in the
 *           reference's orthonormal Gram-Schmidt monomial basis (src/2d/basis.cu).
 *
 * Handles are not thread-safe: use one host thread per handle.  Device buffers
 * are owned by the handle.
 */
#ifndef DGX_H
#define DGX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DGX_VERSION 1

enum dgx_status {
    DGX_OK = 0,
    DGX_ERR_INVALID = -1,      /* bad argument or inconsistent mesh            */
    DGX_ERR_CUDA = -2,         /* a CUDA call failed                           */
    DGX_ERR_NOMEM = -3,        /* device or host allocation failed             */
    DGX_ERR_UNSUPPORTED = -4,  /* valid request outside what this build serves */
    DGX_ERR_NONFINITE = -5,    /* the state holds NaN/Inf or negative density  */
    DGX_ERR_BUSY = -6,         /* admission refused (budget or queue full)     */
    DGX_ERR_NOT_FOUND = -7,    /* unknown request id                           */
    DGX_ERR_TIMEOUT = -8       /* a bounded wait ran out                       */
};

enum dgx_equation { DGX_ADVECTION = 0, DGX_EULER = 1 };
enum dgx_flux { DGX_FLUX_CENTRAL = 0, DGX_FLUX_LLF = 1 };
/* Precisions:
 *   FP32         FP32 state and arithmetic (the plain path).
 *   FP32_BF16X3  FP32 state, the basis contractions on the tensor cores.
 *   FP64         the reference's precision.
 *   FP32_COMP    FP32 state and arithmetic, RK4 only, with compensated
 *                accumulation: the stage increments k1/6 + k2/3 + k3/3 are
 *                accumulated apart from the state, and the state is carried as
 *                a pair (c, lo) of FP32 arrays whose sum is updated by an
 *                error-free two-sum each step.  Over thousands of steps it
 *                stays within ~1e-6 of FP64, where FP32 storage alone
 *                accumulates 1e-5 .. 1e-4 (the FP32 rounding of the stored
 *                state, not the FP32 arithmetic, sets that error).  One more
 *                state vector on the device and 19 state passes per RK4 step
 *                instead of 13.  dgx_get_state returns c + lo, dgx_set_state
 *                splits an FP64 state into the pair, dgx_set_state_f32 clears
 *                lo, dgx_state_device_ptr gives c.  No counterpart in the
 *                reference (FP64 throughout). */
enum dgx_precision { DGX_FP32 = 0, DGX_FP32_BF16X3 = 1, DGX_FP64 = 2, DGX_FP32_COMP = 3 };
/* Time integrators (src/2d/conservation/time_integrator.cu):
 *   RK4  classic four-stage Runge-Kutta (time_integrate_rk4, :221-434)
 *   RK2  explicit midpoint: c += k(c + k(c)/2) (time_integrate_rk2, :466-614)
 *   FE   forward Euler: c += k(c) (time_integrate_fe, :622-749) */
enum dgx_integrator { DGX_RK4 = 0, DGX_RK2 = 1, DGX_FE = 2 };
enum dgx_dt_mode { DGX_DT_FIXED = 0, DGX_DT_CFL = 1 };

/* Built-in initial conditions (projected with the degree-2p rule, as the
 * reference's init_conditions, conserv_kernels.cu:167-187).  params[8]:
 *   GAUSSIAN      u = exp(-((x-x0)^2+(y-y0)^2)/w)        {x0, y0, w, Lx, Ly}
 *   POLY          u = (x-y)^alpha                         {alpha}
 *   DENSITY_WAVE  rho = 1 + A sin(2 pi k (x+y)), u, v, p  {A, u, v, p, k}
 *   VORTEX        isentropic vortex on a free stream      {x0, y0, beta, u, v, Lx, Ly}
 *   CONSTANT      constant state                          {rho, u, v, p} (advection: {u})
 *   CYLINDER      free stream rho = gamma, u = M, v = 0, p = 1  {M}
 *                 (the cylinder problem's U0, euler/cylinder/cylinder.cu:26-31)
 *   SUPERSONIC_VORTEX  supersonic vortex between two arcs about the origin:
 *                 rho = (1 + A (1 - 1/r^2))^2.5, speed M/r   {M, A}
 *                 (euler/supersonic/supersonic.cu:26-37; the reference's
 *                 A = 1.0125 for M = 2.25; A = 0 means (gamma-1)/2 M^2)
 *   THREEPOINT    oblique shock state for atan(x/y) < theta, gas at rest
 *                 beyond                                 {M, theta in degrees}
 *                 (euler/threepoint/threepoint.cu:27-54; PI = 3.14159 as there)
 *   LINEAR        u = c0 + cx x + cy y (advection)       {c0, cx, cy}
 *                 (the reference's advection problem is u0 = x + y,
 *                 2dadvec/2dadvec_kernels.cu:176-178, with the exact
 *                 Dirichlet data x - 2t + y at its boundary sides, :184-186:
 *                 DGX_BC_EXACT with {0, 1, 1} and a = (1, 1))
 * Lx, Ly > 0 take distances to the nearest periodic image. */
enum dgx_ic {
    DGX_IC_GAUSSIAN = 0,
    DGX_IC_POLY = 1,
    DGX_IC_DENSITY_WAVE = 2,
    DGX_IC_VORTEX = 3,
    DGX_IC_CONSTANT = 4,
    DGX_IC_CYLINDER = 5,
    DGX_IC_SUPERSONIC_VORTEX = 6,
    DGX_IC_THREEPOINT = 7,
    DGX_IC_LINEAR = 8
};

typedef struct dgx_mesh dgx_mesh;
typedef struct dgx_solver dgx_solver;

typedef struct dgx_solver_desc {
    int order;       /* p, 0..5 (src/2d/conservation/conserv.cu:61-80)            */
    int equation;    /* dgx_equation                                                */
    int flux;        /* dgx_flux: CENTRAL (advection reference), LLF (Euler)        */
    int precision;   /* dgx_precision                                               */
    int integrator;  /* dgx_integrator                                              */
    double gamma;    /* ratio of specific heats (problem file's get_GAMMA)          */
    double ax, ay;   /* advection velocity (reference: (1,1), 2dadvec_kernels.cu:150-155) */
} dgx_solver_desc;

/* --- library ---------------------------------------------------------------- */
int dgx_version(void);
const char *dgx_status_string(int status);
const char *dgx_last_error(void);

/* Basis and quadrature tables in FP64 for order p (replaces set_quadrature,
 * src/2d/conservation/conserv.cu:37-107, and preval_basis, src/2d/basis.cu:150-226).
 * dims[3] = {n_p, n_quad, n_quad1d}; any output pointer may be NULL.
 * basis/grad_x/grad_y are [i*n_quad + j] (grad_* premultiplied by the weights),
 * side is [side*n_p*n_quad1d + i*n_quad1d + j], vertex is [3*i + v]. */
int dgx_tables(int p, int *dims, double *r1, double *r2, double *w, double *r_oned,
               double *w_oned, double *basis, double *grad_x, double *grad_y,
               double *basis_side, double *basis_vertex);

/* --- mesh ------------------------------------------------------------------- */
/* Upload a mesh and compute its geometric factors in FP64 on the device
 * (replaces read_mesh + init_gpu + the preval_* kernels,
 * src/2d/conservation/conserv.cu:118-321, conserv_kernels.cu:338-514).
 * Host pointers.  The edge normal is oriented out of the left element and the
 * side length is taken from the left element's local side. */
int dgx_mesh_create(int num_elem, int num_sides, const double *V1x, const double *V1y,
                    const double *V2x, const double *V2y, const double *V3x,
                    const double *V3y, const int *elem_s1, const int *elem_s2,
                    const int *elem_s3, const int *left_elem, const int *right_elem,
                    const int *left_side_number, const int *right_side_number,
                    dgx_mesh **out);
/* Structured periodic triangulation of [x0,x0+lx] x [y0,y0+ly]: n x n squares
 * split along their SW-NE diagonal (2n^2 elements, 3n^2 sides), interior
 * vertices jittered by jitter*h*(2u-1) with u from a counter-based generator
 * of `seed`.  The synthetic meshes of the benchmark configurations (the
 * reference reads its meshes from .pmsh files, conserv.cu:118-192).
 * dgx_periodic_square_arrays fills host arrays V[6][E], elem_s[3][E],
 * sides[4][S] (left_elem, right_elem, left_side, right_side) without a GPU. */
int dgx_periodic_square_arrays(int n, double lx, double ly, double x0, double y0, double jitter,
                               unsigned long long seed, double *V, int *elem_s, int *sides);
int dgx_mesh_create_periodic_square(int n, double lx, double ly, double x0, double y0,
                                    double jitter, unsigned long long seed, dgx_mesh **out);
int dgx_mesh_destroy(dgx_mesh *mesh);
/* The reference's .pmsh text format (read_mesh, src/2d/conservation/conserv.cu:
 * 118-192; written by src/2d/genmesh.py:290-308).  dgx_pmsh_info gives the
 * counts, dgx_pmsh_read fills caller arrays V[6][E], elem_s[3][E], sides[4][S]
 * (left_elem, right_elem, left_side, right_side); dgx_pmsh_write writes
 * full-precision coordinates. */
int dgx_pmsh_info(const char *path, int *num_elem, int *num_sides);
int dgx_pmsh_read(const char *path, double *V, int *elem_s, int *sides);
int dgx_pmsh_write(const char *path, int num_elem, int num_sides, const double *V,
                   const int *elem_s, const int *sides);
int dgx_mesh_create_from_pmsh(const char *path, dgx_mesh **out);
/* FP64 geometric factors copied to host arrays (NULL to skip): J, x_r, y_r,
 * x_s, y_s, inscribed diameter per element; length, Nx, Ny per side. */
int dgx_mesh_geometry(const dgx_mesh *mesh, double *J, double *xr, double *yr, double *xs,
                      double *ys, double *diameter, double *s_length, double *Nx,
                      double *Ny);
int dgx_mesh_min_diameter(const dgx_mesh *mesh, double *out);
int dgx_mesh_info(const dgx_mesh *mesh, int *num_elem, int *num_sides, int *num_boundary);

/* --- solver ----------------------------------------------------------------- */
int dgx_solver_create(dgx_mesh *mesh, const dgx_solver_desc *desc, dgx_solver **out);
int dgx_solver_destroy(dgx_solver *solver);
/* num_vars (1 or 4), n_p, bytes of one state vector, total device bytes held */
int dgx_solver_info(const dgx_solver *solver, int *num_vars, int *n_p, size_t *state_bytes,
                    size_t *device_bytes);

/* State in the reference layout, host FP64 (any precision) or host FP32. */
int dgx_set_state(dgx_solver *solver, const double *c);
int dgx_get_state(dgx_solver *solver, double *c);
int dgx_set_state_f32(dgx_solver *solver, const float *c, void *stream);
int dgx_get_state_f32(dgx_solver *solver, float *c, void *stream);
/* Device pointer of the resident state (FP32, or FP64 in DGX_FP64 precision). */
int dgx_state_device_ptr(dgx_solver *solver, void **ptr);
/* L2-project a built-in initial condition onto the state (FP64 on the device). */
int dgx_project_ic(dgx_solver *solver, int ic, const double *params);

/* One RHS evaluation on device buffers in the solver's precision:
 * k = dt / J * (volume + sum of the three lifted edge fluxes), the contract of
 * eval_surface + eval_volume + eval_rhs (src/2d/conservation/time_integrator.cu:
 * 130-188, conserv_kernels.cu:697-811).  u and k must not alias. */
int dgx_rhs_eval(dgx_solver *solver, const void *u, void *k, double dt, double t,
                 void *stream);

/* Time step size: FIXED uses dt; CFL uses dt = cfl * min diameter / max wave
 * speed / (2p+1) from cell averages (time_integrator.cu:252-270,
 * euler.cu:252-278), computed and kept on the device. */
int dgx_set_dt(dgx_solver *solver, int dt_mode, double dt, double cfl);
/* End time: the last step is clipped to land on it (time_integrator.cu:263-270);
 * t_end <= 0 disables clipping. */
int dgx_set_end_time(dgx_solver *solver, double t_end);
/* One stage of the solver's integrator on the resident state: s = 0..3 for RK4
 * (rk_tempstorage / rk4, time_integrator.cu:194-218), 0..1 for RK2
 * (rk2_tempstorage / rk2, :445-464), 0 for FE (eval_rhs_fe, :622-700); stage 0
 * also fixes dt.  Other stage numbers return DGX_ERR_INVALID. */
int dgx_rk_stage(dgx_solver *solver, int stage, void *stream);
/* One full time step (CFL + every stage), asynchronous on `stream`. */
int dgx_step(dgx_solver *solver, void *stream);
/* Advance until t_end or max_steps steps (time_integrate_rk4 / _rk2 / _fe,
 * time_integrator.cu:221-749); synchronous. */
int dgx_run(dgx_solver *solver, double t_end, int max_steps, int *steps, double *t,
            void *stream);
/* Current simulation time and last dt (synchronises the stream). */
int dgx_time(dgx_solver *solver, double *t, double *dt, void *stream);
int dgx_reset_time(dgx_solver *solver, double t);
/* Conserved totals  int u_n dx  in FP64 (deterministic device reduction; in
 * DGX_FP32_COMP of the state's two parts, c + lo).
 * The first call on a solver allocates its scratch (8 bytes per element plus
 * 32 KiB), kept until the solver is destroyed; later calls allocate nothing.
 * Synchronous (the totals are host doubles). */
int dgx_conserved_totals(dgx_solver *solver, double *out, void *stream);
/* Conserved totals without allocating.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc: a serving loop held to a fixed
 * device-memory budget, an application whose own allocator owns the device
 * memory, or a latency-critical loop that cannot take the device-wide
 * synchronisation of cudaFree.  dgx_conserved_totals allocates scratch on
 * its first call on a solver; this variant keeps its scratch in one static device array of
 * 256 KiB (4 variables x 8192 partial sums), held on every device that loads
 * the library until the process exits.  It allocates nothing and frees nothing.
 *   state  the solver's state layout and precision, device memory
 *          (e.g. dgx_state_device_ptr)
 *   out    num_vars doubles, device-accessible, written by the GPU
 * Meshes above DGX_TOTALS_STATIC_MAX_ELEMS elements are refused with
 * DGX_ERR_INVALID.  Asynchronous on `stream`.  Every call looks up the
 * array's device address on the current device (so a cudaDeviceReset between
 * calls is harmless); the first lookup on a device may load the library's
 * device code, so make the first call before any stream capture.  Its two
 * kernel launches count in dgx_launch_count.  All calls share the one array:
 * calls that overlap on the GPU (different streams, no ordering between them)
 * race and give wrong totals. */
#define DGX_TOTALS_STATIC_MAX_ELEMS 16777216
int dgx_conserved_totals_static(const dgx_solver *solver, const void *state, double *out,
                                void *stream);
/* Slope limiter for p = 1 on the resident state, in place (the reference's
 * "standard limiter for p = 1", limit_c, src/2d/conservation/conserv_kernels.cu:
 * 522-621, which its integrator leaves disabled and whose bounds it never
 * sets), in Barth-Jespersen form: per element and variable the two linear
 * modes are scaled by the largest phi <= 1 that keeps the traces at the side
 * Gauss points within the range of the cell averages of the element and its
 * three neighbours (a boundary side contributes the element itself).  Cell
 * averages are unchanged.  Asynchronous on `stream`; other orders:
 * DGX_ERR_UNSUPPORTED. */
int dgx_limit(dgx_solver *solver, void *stream);
/* Largest |c - prev| over every coefficient of the resident state, in FP64
 * (prev: a device state in the solver's layout and precision), the quantity
 * of the reference's disabled steady-state test (check_convergence,
 * conserv_kernels.cu:943-947, time_integrator.cu:401-421).  Synchronous. */
int dgx_state_change(dgx_solver *solver, const void *prev, double *max_change, void *stream);
/* Step until the largest coefficient change of one step is <= tol, or
 * max_steps steps (the reference's `while (t < endtime && convergence > TOL)`
 * loop with TOL = 5e-8, time_integrator.cu:247-251).  Keeps one more state
 * vector on the device (allocated on the first call).  Returns the steps taken
 * and the last step's change.  The end time still applies: at it, dt = 0 and
 * the change is 0. */
int dgx_run_steady(dgx_solver *solver, double tol, int max_steps, int *steps, double *change,
                   void *stream);
/* Maximum cell-average wave speed of the resident state. */
int dgx_max_wave_speed(dgx_solver *solver, double *out, void *stream);
/* Vertex values of every variable as the reference's Gmsh "ST" views
 * (src/2d/conservation/main.cu:193-209), one file per variable named by
 * printf(path_pattern, variable), e.g. "output/U%d.msh". */
int dgx_write_vertex_values(dgx_solver *solver, const char *path_pattern);
/* Boundary sides (right_elem < 0, the element being the side's left element):
 *   Euler, -1 reflecting: density and energy kept, momentum reduced to its
 *     tangential part (the reference's reflecting_boundary,
 *     src/2d/conservation/euler/cylinder/cylinder.cu:58-111, with the side normal);
 *   Euler, -2 outflow / -3 inflow: DGX_BC_FREESTREAM params {rho, u, v, p}
 *     (the problem hooks U_outflow / U_inflow, euler.cu:177-241);
 *   advection, any tag: DGX_BC_EXACT, the initial condition `ic` (GAUSSIAN, POLY
 *     or LINEAR) with `params` translated by a*t (the reference's boundary_exact,
 *     2dadvec_kernels.cu:184-186, is LINEAR {0, 1, 1} at a = (1, 1));
 *   Euler, DGX_BC_PROBLEM with ic = CYLINDER / SUPERSONIC_VORTEX / THREEPOINT and
 *     that initial condition's params: the problem file's own hooks for all
 *     three tags --
 *       cylinder: -1 momentum reduced to its part tangential to the circle
 *         about (0.5, 0.5) through the point, -2/-3 the free stream
 *         (cylinder.cu:38-111);
 *       supersonic vortex: -1 the same about the origin, -2/-3 the vortex
 *         state at the point (supersonic.cu:40-113);
 *       three-point: -1 flips the x momentum where m.n > 0, else the y
 *         momentum, -2 the shock state, -3 the shock state left of the front
 *         x = M t cos(theta) + tan(theta), else the initial state
 *         (threepoint.cu:56-109).
 *     The reference's radial reflections take the point with side 1's two
 *     reference coordinates exchanged (cylinder.cu:78-81, supersonic.cu:86-89);
 *     kept alike.
 * Without a setting, outflow/inflow and advection sides take the interior state. */
enum dgx_bc { DGX_BC_NONE = 0, DGX_BC_FREESTREAM = 1, DGX_BC_EXACT = 2, DGX_BC_PROBLEM = 3 };
int dgx_solver_set_boundary(dgx_solver *solver, int kind, int ic, const double *params);
/* Kernel options of a solver (for autotuning and tests):
 *   DGX_OPT_PREFETCH  1 (default): RK stages 2-4 copy the tile's base state and
 *                     accumulator into shared memory with the TMA engine while
 *                     the element work runs; 0: plain loads at the end. */
/*   DGX_OPT_STAGE_TIME  the time at which a stage evaluates time-dependent
 *                     boundary data:
 *                     DGX_STAGE_TIME_EXACT (default) t_n + c_s dt with the
 *                       integrator's nodes c_s (RK4 0, 1/2, 1/2, 1; RK2 0, 1/2);
 *                     DGX_STAGE_TIME_REFERENCE the reference's arguments: Euler
 *                       RK4/RK2 pass t_{n+1} + c_s dt (time_integrator.cu:264-380,
 *                       :509-561), Euler FE and every advection stage pass t_n
 *                       (time_integrator.cu:733, src/2d/time_integrator.cu:145).
 *                     Periodic meshes and time-independent boundary data give
 *                     the same results under both. */
/*   DGX_OPT_LIMITER   1: apply dgx_limit to the state every stage writes (the
 *                     reference's limiter hook after each stage,
 *                     time_integrator.cu:302,332,363); p = 1 only, single
 *                     solves (batches refuse such solvers); 0 (default): off. */
/*   DGX_OPT_HOOK_MATH the arithmetic of the DGX_BC_PROBLEM ghost states:
 *                     DGX_HOOK_MATH_DOUBLE (default) FP64 throughout;
 *                     DGX_HOOK_MATH_REFERENCE the FP32 square roots and powers
 *                       of the reference's problem files (sqrtf of the radius in
 *                       the radial reflections, cylinder.cu:100 and
 *                       supersonic.cu:100; powf in the supersonic vortex's
 *                       state, supersonic.cu:30,35), for callers that need the
 *                       reference's numbers near those boundaries.  The two
 *                       differ by FP32 rounding in the ghost states. */
enum dgx_option { DGX_OPT_PREFETCH = 1, DGX_OPT_STAGE_TIME = 2, DGX_OPT_LIMITER = 3, DGX_OPT_HOOK_MATH = 4 };
enum dgx_stage_time { DGX_STAGE_TIME_EXACT = 0, DGX_STAGE_TIME_REFERENCE = 1 };
enum dgx_hook_math { DGX_HOOK_MATH_DOUBLE = 0, DGX_HOOK_MATH_REFERENCE = 1 };
int dgx_solver_set_option(dgx_solver *solver, int option, int value);
/* Number of CUDA kernels this solver has launched so far. */
int dgx_launch_count(const dgx_solver *solver, long long *count);

/* Tensor-core self-test on the current device.  No reference counterpart.
 * One CTA multiplies a 128x16 by 16x32 matrix of small integers in BF16 with
 * tcgen05.mma (FP32 accumulation), A once from shared and once from tensor
 * memory, and counts the accumulator elements that differ from the exact
 * product: *bad_ss (A in shared memory) and *bad_ts (A in tensor memory); both
 * 0 means the path works.  variant 0 is the operand-descriptor encoding the
 * solvers use, variant 1 the same layout with the two descriptor offsets
 * exchanged (a diagnostic).  `values` (optional, 128 x 64 floats) receives the
 * two accumulators row by row.  DGX_ERR_TIMEOUT if the MMA did not complete. */
int dgx_tc_selftest(int variant, int *bad_ss, int *bad_ts, float *values);

/* --- batches: many independent solves per launch --------------------------- */
/* New, no counterpart in the reference (it runs one solve per process; this
 * generalises its loop, src/2d/conservation/time_integrator.cu:252-429).
 * Solves of equal (precision, order, equation, boundary sides or none) form a
 * class; each RK stage
 * launches one kernel per class over work lists of (solve, element tile), one
 * batched kernel computes every solve's dt, and the whole step is captured as
 * a CUDA graph.  Every solve keeps its own state, time, dt rule and end time
 * (set them before creating the batch); each solve's result equals the same
 * solve run alone with dgx_step, bit for bit.  Batches take RK4 solvers only
 * (others: DGX_ERR_UNSUPPORTED).  Destroy the batch before its solvers. */
typedef struct dgx_batch dgx_batch;
int dgx_batch_create(dgx_solver *const *solvers, int n, dgx_batch **out);
int dgx_batch_destroy(dgx_batch *batch);
/* one RK4 step of every solve (a graph launch, asynchronous on `stream`) */
int dgx_batch_step(dgx_batch *batch, void *stream);
int dgx_batch_run(dgx_batch *batch, int steps, void *stream);
/* Choose per class, by timing `reps` stage launches on the live batch, the
 * kernel options (TMA prefetch of the epilogue operands; flat grid or a
 * persistent grid of 2 or 4 CTAs per SM); then, where the batch allows the
 * fused launch (below), choose between the per-class launches and the fused
 * launch's two variants by timing `reps` whole steps; rebuild the graph.  The
 * solves' states and times are restored afterwards.  Synchronous. */
int dgx_batch_autotune(dgx_batch *batch, int reps, void *stream);
/* The fused launch: one kernel per RK stage for every class of the batch (a
 * step is the dt launch and four stage launches) over one work list of
 * (solve, tile) items, the costliest classes first.  FP32 batches whose meshes
 * have no boundary sides (others: DGX_ERR_UNSUPPORTED).  mode 0: the
 * per-class launches (default); 2 or 3: the fused kernel compiled for 2 or 3
 * CTAs per SM (one register count for every class: 2 keeps order-4 Euler
 * unspilled, 3 caps every class at 168 registers).  Results are the same bits
 * either way.  Rebuilds the graph.  No counterpart in the reference. */
int dgx_batch_set_fused(dgx_batch *batch, int mode);
/* the current mode, and whether the batch allows the fused launch */
int dgx_batch_get_fused(const dgx_batch *batch, int *mode, int *available);
int dgx_batch_info(const dgx_batch *batch, int *num_classes, int *num_items, long long *dofs,
                   long long *launches_per_step);
int dgx_batch_class_options(const dgx_batch *batch, int cls, int *order, int *equation,
                            int *prefetch, int *persistent);
int dgx_batch_launch_count(const dgx_batch *batch, long long *count);
/* Per solve (in creation order): current time, last dt, status flags
 * (nonzero: non-finite or unphysical state) and completed steps, gathered in
 * one copy; any output may be NULL; synchronous. */
int dgx_batch_progress(dgx_batch *batch, double *t, double *dt, unsigned int *status,
                       long long *steps, void *stream);
/* Set the kernel options of one class by hand and rebuild the graph. */
int dgx_batch_set_options(dgx_batch *batch, int cls, int prefetch, int persistent);

/* --- serving: continuous batching of solve requests ------------------------ */
/* New, no counterpart in the reference.  A worker thread admits queued requests
 * while the device-memory budget and slot count allow, keeps their state on the
 * device, repacks the running set into a batch whenever solves join or finish,
 * advances it a few steps at a time and retires finished solves, recording
 * time-to-solution.  A request's result is the same alone and in the mix. */
typedef struct dgx_server dgx_server;
typedef struct dgx_request {
    int n;                       /* periodic square mesh: n x n squares ...            */
    double lx, ly, jitter;       /* ... of [0,lx] x [0,ly], jitter (dgx_mesh_create_periodic_square) */
    unsigned long long seed;     /* equal mesh specs share one device mesh              */
    int order, equation, flux, precision;
    double gamma, ax, ay;
    int ic;                      /* dgx_ic with params                                  */
    double params[8];
    double t_end;                /* end time (the last step is clipped to it)           */
    double cfl;                  /* CFL factor when dt <= 0                             */
    double dt;                   /* > 0: fixed time step                                */
    int keep_state;              /* keep the final state for dgx_server_result          */
} dgx_request;
enum dgx_request_state { DGX_REQ_QUEUED = 0, DGX_REQ_RUNNING = 1, DGX_REQ_DONE = 2,
                         DGX_REQ_FAILED = 3, DGX_REQ_CANCELLED = 4 };
typedef struct dgx_server_stats {
    long long submitted, completed, failed, active, queued, repacks, steps;
    double dof_updates;          /* DOF-updates performed by completed and running solves */
    double busy_seconds;         /* worker time from queueing a round of steps to reading
                                    their progress (the admission work of the round,
                                    which overlaps the steps on the GPU, included)      */
    double p50_latency_s, p99_latency_s, max_latency_s;   /* time-to-solution           */
    size_t device_bytes_in_use;  /* admitted footprint                                  */
    double admit_seconds;        /* worker time spent creating admitted solves (while
                                    the GPU runs the steps queued before them)           */
    double repack_seconds;       /* worker time spent rebuilding the batch              */
    double retire_seconds;       /* worker time spent reading out and freeing finished solves */
    double idle_seconds;         /* worker time spent waiting for requests              */
    long long pool_hits;         /* mesh and solver blocks reused from the server's pool */
    long long pool_misses;       /* blocks the pool had to allocate                     */
    long long cached_meshes;     /* meshes in the cache (running and idle)              */
} dgx_server_stats;
/* budget_bytes: admission limit on the estimated device footprint of running
 * requests; max_active: slot limit. */
int dgx_server_create(size_t budget_bytes, int max_active, dgx_server **out);
/* Queue a request (validated here: DGX_ERR_INVALID / DGX_ERR_UNSUPPORTED; a
 * request larger than the whole budget: DGX_ERR_BUSY). */
int dgx_server_submit(dgx_server *server, const dgx_request *request, long long *id);
/* state (dgx_request_state) and time-to-solution once finished (else -1) */
int dgx_server_status(dgx_server *server, long long id, int *state, double *latency_s);
/* Result of a finished request: final state (if kept, c_len >= its size),
 * conserved totals (4 doubles), steps and final time; any output may be NULL. */
int dgx_server_result(dgx_server *server, long long id, double *c, size_t c_len, double *totals,
                      int *steps, double *t_final);
int dgx_server_cancel(dgx_server *server, long long id);
/* forget a finished, failed or cancelled request */
int dgx_server_release(dgx_server *server, long long id);
/* wait until nothing is queued or running; DGX_ERR_TIMEOUT after timeout_s */
int dgx_server_wait_idle(dgx_server *server, double timeout_s);
int dgx_server_get_stats(dgx_server *server, dgx_server_stats *out);
/* steps advanced between two completion checks (default 8) */
int dgx_server_set_steps_per_check(dgx_server *server, int steps);
/* Fault injection on the host: the worker sleeps `seconds` after every check. */
int dgx_server_inject_stall(dgx_server *server, double seconds);
int dgx_server_destroy(dgx_server *server);

#ifdef __cplusplus
}
#endif

#endif /* DGX_H */
