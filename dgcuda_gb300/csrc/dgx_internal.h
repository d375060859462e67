// dgx_internal.h -- handle layouts and helpers shared by the library's sources.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <mutex>
#include <vector>

#include "dgx.h"
#include "dgx_tables.h"

namespace dgx {

void set_error(const char *fmt, ...);

#define DGX_TRY_CUDA(call)                                                                  \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            ::dgx::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                             __LINE__);                                                     \
            return DGX_ERR_CUDA;                                                            \
        }                                                                                   \
    } while (0)

#define DGX_CHECK_LAUNCH()                                                                  \
    do {                                                                                    \
        cudaError_t e_ = cudaGetLastError();                                                \
        if (e_ != cudaSuccess) {                                                            \
            ::dgx::set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_),     \
                             __FILE__, __LINE__);                                           \
            return DGX_ERR_CUDA;                                                            \
        }                                                                                   \
    } while (0)

// Bit flags of the per-solver device status word.
enum StatusBits : unsigned int {
    kStatusNonFinite = 1u,   // NaN/Inf wave speed or state
    kStatusNegative = 2u,    // non-positive density or pressure in a cell average
    kStatusCopyTimeout = 4u, // a bounded wait for an asynchronous copy ran out
    kStatusBadItem = 8u,     // a batched work item outside its solve's tiles (skipped)
};

// Elements are processed in tiles of kTile consecutive elements, one CTA per
// tile.  The side traces a tile needs live in shared memory in "slots": slot
// 3*l + k holds the trace of the tile's element l on its local side k, slots
// 3*kTile + h hold the tile's halo (traces of neighbours outside the tile).
constexpr int kTile = 128;

// Element-side word: (slot of the neighbour's trace) * 2 + is_left, or the
// (negative) boundary tag of a boundary side.
DGX_HD inline int pack_side_word(int slot, int is_left) { return slot * 2 + is_left; }
// Halo entry: neighbour element * 4 + neighbour's local side.
DGX_HD inline int pack_halo(int e, int side) { return e * 4 + side; }

// Mesh geometry, computed in FP64 on the device at creation.
struct MeshDev {
    int num_elem = 0, num_sides = 0, num_boundary = 0;
    // FP64 reference quantities (device)
    double *V = nullptr;        // [6][E] V1x V1y V2x V2y V3x V3y
    int *elem_s = nullptr;      // [3][E]
    int *sides = nullptr;       // [4][S] left_elem right_elem left_side right_side
    double *J = nullptr, *xr = nullptr, *yr = nullptr, *xs = nullptr, *ys = nullptr;
    double *diam = nullptr;     // [E] inscribed diameters
    double *len = nullptr, *nx = nullptr, *ny = nullptr;   // [S]
    double min_diam = 0.0;
    // per-element hot-path arrays
    int *nbr = nullptr;         // [3][E] element-side words (pack_side_word)
    int *halo_off = nullptr;    // [num_tiles + 1] CSR offsets into halo_list
    int *halo_list = nullptr;   // [total halo] pack_halo entries, per tile
    int num_tiles = 0, max_halo = 0, total_halo = 0;
    float *geo32 = nullptr;     // [5][E] 1/J, x_r, y_r, x_s, y_s
    float *fn32 = nullptr;      // [3 sides][3][E] nx, ny, len/2 (normal out of the side's left element)
    double *geo64 = nullptr;    // same in FP64
    double *fn64 = nullptr;
};

// Device memory of meshes and solvers: every mesh and every solver keeps its
// arrays in one block, carved at 256-byte boundaries.  A BlockPool keeps
// released blocks by size class and hands them out again, so a long-running
// owner (the request server) stops allocating and freeing device memory, and
// with it the device-wide synchronisation of cudaFree, once its working set is
// warm.  A block goes back to its pool only after the device work that reads
// it has finished.
class BlockPool {
public:
    static constexpr size_t kSlabBytes = static_cast<size_t>(64) << 20;
    static constexpr size_t kSlabBlock = static_cast<size_t>(8) << 20;   // larger: one allocation each
    explicit BlockPool(size_t keep_bytes) : keep_(keep_bytes) {}
    ~BlockPool();   // frees the slabs: every block must have been returned
    BlockPool(const BlockPool &) = delete;
    BlockPool &operator=(const BlockPool &) = delete;
    // a block of at least `bytes`; *got is its size (the size class)
    int get(size_t bytes, void **p, size_t *got);
    void put(void *p, size_t bytes);
    void trim();                                   // free the cached blocks not carved from slabs
    size_t cached_bytes();
    long long hits() {
        std::lock_guard<std::mutex> lk(mu_);
        return hits_;
    }
    long long misses() {
        std::lock_guard<std::mutex> lk(mu_);
        return misses_;
    }
    // 4 KiB .. 64 KiB: powers of two; above: 8 classes per octave
    static size_t size_class(size_t bytes);
private:
    std::mutex mu_;
    std::multimap<size_t, void *> free_;
    std::vector<void *> slabs_;
    char *slab_next_ = nullptr;
    size_t slab_left_ = 0;
    size_t cached_ = 0, keep_;   // cached bytes of the blocks not carved from slabs
    long long hits_ = 0, misses_ = 0;
};

struct DeviceBlock {
    void *base = nullptr;
    size_t bytes = 0;
    BlockPool *pool = nullptr;   // nullptr: cudaMalloc / cudaFree
};
int block_alloc(DeviceBlock &b, size_t bytes, BlockPool *pool);
void block_free(DeviceBlock &b);

// offsets of consecutive arrays in one block, each at a 256-byte boundary
struct BlockLayout {
    size_t size = 0;
    template <typename T>
    size_t take(size_t count) {
        size = (size + 255) & ~static_cast<size_t>(255);
        const size_t at = size;
        size += (count ? count : 1) * sizeof(T);
        return at;
    }
};
template <typename T>
T *block_at(const DeviceBlock &b, size_t off) {
    return reinterpret_cast<T *>(static_cast<char *>(b.base) + off);
}

}  // namespace dgx

struct dgx_mesh {
    dgx::MeshDev d;
    dgx::DeviceBlock block;
    int device = 0;
    std::atomic<int> refs{1};
};

namespace dgx {

struct SolverDev {
    int order = 0, np = 0, nv = 0, equation = 0, flux = 0, precision = 0;
    double gamma = 1.4, ax = 1.0, ay = 1.0;
    size_t n = 0;                      // values per state vector
    void *c = nullptr;                 // resident state (FP32 or FP64)
    void *acc = nullptr;               // RK4 accumulator (RK4 only)
    void *ua = nullptr, *ub = nullptr; // stage inputs (ub: RK4 only)
    void *lo = nullptr;                // DGX_FP32_COMP: the state's low part (state = c + lo)
    // device scalars: [0] dt of the current step, [1] t at the end of it,
    // [2] t at its start, [3] fixed dt, [4] cfl, [5] t_end, [6] max wave speed
    double *scal = nullptr;
    unsigned long long *lam_bits = nullptr;  // running max of the wave speed (double bits)
    unsigned int *counter = nullptr;   // grid-completion counter of the CFL kernel
    unsigned int *status = nullptr;    // StatusBits
    long long *steps = nullptr;        // completed steps
    double *red = nullptr;             // reduction scratch (partials)
    int red_len = 0;
    int dt_mode = DGX_DT_CFL;
    int integrator = DGX_RK4;          // dgx_integrator
    int stage_time = DGX_STAGE_TIME_EXACT;   // DGX_OPT_STAGE_TIME
    int prefetch = 1;                  // DGX_OPT_PREFETCH
    int limiter = 0;                   // DGX_OPT_LIMITER: limit every stage's output (p = 1)
    int hook_math = DGX_HOOK_MATH_DOUBLE;   // DGX_OPT_HOOK_MATH
    unsigned long long *chg_bits = nullptr;   // largest coefficient change (double bits)
    void *prev = nullptr;              // dgx_run_steady: the state before the step (on demand)
    double *tot_scratch = nullptr;     // dgx_conserved_totals: E terms + kReduceLen + 1 (on demand)
    int bc_kind = 0, bc_ic = 0;        // boundary ghost states (StageArgs)
    double bc_state[4] = {0, 0, 0, 0};
    double bc_params[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

}  // namespace dgx

struct dgx_solver {
    dgx_mesh *mesh = nullptr;
    dgx::SolverDev s;
    dgx::DeviceBlock block;
    size_t device_bytes = 0;
    long long launches = 0;
};

namespace dgx {

// kernels/launchers implemented in the .cu sources
// each stage translation unit (precision x with/without boundary sides) owns
// its constant tables
int upload_tables_f32_nb();
int upload_tables_f32_b();
int upload_tables_f64_nb();
int upload_tables_f64_b();
int upload_tables_misc();

struct StageArgs {
    int E;
    int mode;          // 0 rhs, 1..4 RK4 stages, 5 out = u + alpha k, 6 out = c + alpha k
    int flux;
    double gamma, ax, ay;
    float gammaf, axf, ayf;   // the same in FP32 (FP32 kernels)
    int prefetch;      // > 0: copy the epilogue operands with the TMA engine, this many values per plane
    unsigned int *status;
    const void *u;     // stage input (read-only)
    const void *c;     // base state
    void *acc;         // accumulator
    void *out;         // k (mode 0), next stage input (1..3), state (4)
    // RK4 in 13 state passes per step (rk13 = 1): stage 1 writes only u2, stage
    // 2 only u3, and stage 3 forms the accumulator c + k1/6 + k2/3 + k3/3 from
    // u2 = c + k1/2 (aux, read before `out` overwrites it in place) and its own
    // input u3 = c + k2/2; rk13 = 0: the 16-pass form with the accumulator
    // written by every stage (kept for the per-stage limiter, which changes the
    // stage states after they are written)
    void *aux;         // read in 13-pass mode 3 and compensated mode 1, written in compensated mode 4
    int rk13;
    // compensated RK4 (DGX_FP32_COMP, comp = 1): acc holds the increment
    // accumulator D and aux the state's low part lo (state = c + lo):
    //   1 u2 = c + k1/2, D = lo + k1/6;  2/3 u = c + alpha k, D += k/3;
    //   4 (c, lo) = two-sum(c, D + k4/6)
    int comp;
    const int *nbr;
    const int *halo_off;
    const int *halo_list;
    int nslot;         // 3*kTile + max halo of the mesh
    const void *geo;
    const void *fn;
    const double *scal;   // device dt/t (modes 1..4); may be null for mode 0
    double dt, t;         // host dt/t for mode 0
    double stage_c;       // stage time = step start + stage_c * dt (modes 1..6)
    double alpha;         // stage weight of modes 5 and 6
    // boundary ghost states: bc_kind 0 none (interior state), 1 free-stream
    // state bc_state (Euler), 2 exact initial condition bc_ic / bc_params
    // translated by a*t (advection)
    int bc_kind, bc_ic;
    int hook_float;            // DGX_BC_PROBLEM ghost states with the reference's FP32 sqrtf/powf
    double bc_state[4];
    double bc_params[8];
    const double *V;           // element vertices V1x, V1y, V2x, V2y, V3x, V3y [6][E] (FP64)
    int bnd;                   // the mesh has boundary sides (selects the kernels with ghost states)
    const void *tc_img;        // BF16x3 path: the order's constant tensor-core operands (device)
};

// Batched launch: items[i] = (index into args, tile); grid CTAs walk the list.
struct BatchStageArgs {
    const StageArgs *args;   // device array, one per solve of the class
    const int2 *items;       // device array of (solve, tile)
    int n_items;
    int grid;
    int nslot;               // largest nslot of the class (shared-memory size)
    int prefetch;            // values per prefetched plane, the largest of the class's solves (0: none)
    int bnd;                 // any solve of the class has boundary sides
};

// Batched launch with the solves' arguments in the kernel's parameter space (up
// to 32 KB of parameters per launch, CUDA 12.1 and later): up to kParamSolves
// solves of one class; CTA b takes tile b - tile_start[j] of the solve j with
// tile_start[j] <= b < tile_start[j+1].  The constant bank serves the
// arguments to every CTA without a dependent global load before its work.
// The block is kept below 31 KB, with the small tables first: measured on
// GB300, a runtime-indexed read of the tile offsets placed past the solves'
// arguments, near the end of a 32 KB parameter block, returned 0.
constexpr int kParamSolves = 88;
struct BatchParamArgs {
    int n;          // solves in this launch
    int nslot;      // largest nslot of the class (shared-memory size)
    int prefetch;   // values per prefetched plane of the class (0: none)
    int bnd;
    int tile_start[kParamSolves + 1];
    StageArgs args[kParamSolves];
};
static_assert(sizeof(BatchParamArgs) <= 31 * 1024, "kept below 31 KB of the 32,764-byte parameter limit");

// _nb: kernels without ghost-state code (meshes without boundary sides); _b: with it
int launch_stage_f32_nb(int order, int equation, const StageArgs &a, cudaStream_t st);
int launch_stage_f32_b(int order, int equation, const StageArgs &a, cudaStream_t st);
int launch_stage_f64_nb(int order, int equation, const StageArgs &a, cudaStream_t st);
int launch_stage_f64_b(int order, int equation, const StageArgs &a, cudaStream_t st);
int launch_batch_stage_f32_nb(int order, int equation, const BatchStageArgs &b, cudaStream_t st);
int launch_batch_stage_f32_b(int order, int equation, const BatchStageArgs &b, cudaStream_t st);
int launch_batch_stage_f64_nb(int order, int equation, const BatchStageArgs &b, cudaStream_t st);
int launch_batch_stage_f64_b(int order, int equation, const BatchStageArgs &b, cudaStream_t st);
int launch_batch_param_f32_nb(int order, int equation, const BatchParamArgs &p, int grid, cudaStream_t st);
int launch_batch_param_f32_b(int order, int equation, const BatchParamArgs &p, int grid, cudaStream_t st);
int launch_batch_param_f64_nb(int order, int equation, const BatchParamArgs &p, int grid, cudaStream_t st);
int launch_batch_param_f64_b(int order, int equation, const BatchParamArgs &p, int grid, cudaStream_t st);
inline int launch_batch_param(int precision, int order, int equation, const BatchParamArgs &p, int grid,
                              cudaStream_t st) {
    if (precision == DGX_FP64)
        return p.bnd ? launch_batch_param_f64_b(order, equation, p, grid, st)
                     : launch_batch_param_f64_nb(order, equation, p, grid, st);
    return p.bnd ? launch_batch_param_f32_b(order, equation, p, grid, st)
                 : launch_batch_param_f32_nb(order, equation, p, grid, st);
}
size_t batch_smem_f32(int order, int equation, int nslot, int prefetch_plane);
size_t batch_smem_f64(int order, int equation, int nslot, int prefetch_plane);

// One launch per RK stage for every FP32 solve of a batch whose meshes have no
// boundary sides, whatever its order and equation (dgx_batch_fused.cu): CTA b
// runs item b, items[b] = (index into args, tile, class code 2*order +
// equation, 0); the items of the costliest classes come first.
struct FusedStageArgs {
    const StageArgs *args;   // this stage's arguments of every solve in the launch
    const int4 *items;
    int n_items;
    int min_ctas;            // 2 or 3: the kernel variant (CTAs per SM it is compiled for)
};
constexpr int kFusedMaxOrder = 5;
int launch_batch_fused_f32(const FusedStageArgs &f, size_t smem, cudaStream_t st);
int upload_tables_fused();
// the BF16x3 tensor-core kernels (dgx_stage_tc.cu) and their tables
int launch_stage_tc(int order, int equation, const StageArgs &a, cudaStream_t st);
int upload_tables_tc();
int tc_images_upload();          // the constant B operands, once per device (dgx_tc_tables.cpp)
const void *tc_image(int order); // their device copy for an order (1..4) on the current device
inline int launch_stage(int precision, int order, int equation, const StageArgs &a, cudaStream_t st) {
    if (precision == DGX_FP32_BF16X3) return launch_stage_tc(order, equation, a, st);
    if (precision == DGX_FP64)
        return a.bnd ? launch_stage_f64_b(order, equation, a, st) : launch_stage_f64_nb(order, equation, a, st);
    return a.bnd ? launch_stage_f32_b(order, equation, a, st) : launch_stage_f32_nb(order, equation, a, st);
}
inline int launch_batch_stage(int precision, int order, int equation, const BatchStageArgs &b, cudaStream_t st) {
    if (precision == DGX_FP64)
        return b.bnd ? launch_batch_stage_f64_b(order, equation, b, st)
                     : launch_batch_stage_f64_nb(order, equation, b, st);
    return b.bnd ? launch_batch_stage_f32_b(order, equation, b, st) : launch_batch_stage_f32_nb(order, equation, b, st);
}

// per-solve time-step arguments (dgx_misc.cu)
struct DtArgs {
    const void *c;
    int E, np, is_double, euler, cfl_mode, order;
    double gamma, phi0, amax, min_diam;
    double *scal;
    unsigned long long *lam_bits;
    unsigned int *counter, *status;
    long long *steps;
    int nblocks;      // blocks that reduce this solve's wave speeds
};
DtArgs make_dt_args(const SolverDev &s, const MeshDev &m);
// batched CFL: items[i] = (solve, block of that solve)
int launch_batch_dt(const DtArgs *args, const int2 *items, int n_items, cudaStream_t st);

// per-solve stage arguments (dgx_api.cu)
StageArgs make_stage_args(dgx_solver *sv, int mode, const void *u, const void *c, void *acc,
                          void *out, double dt, double t);
// the arguments of RK4 stage 0..3 on the solver's resident buffers (the
// 13-pass form unless the per-stage limiter is on)
StageArgs rk4_stage_args(dgx_solver *sv, int stage);

// Creation of meshes and solvers with their device memory from `pool`
// (nullptr: cudaMalloc), uploads and initialisation on `st`.  Without `async`,
// mesh_build returns once the geometry is computed.  With it nothing waits: the
// upload goes through async->stage(bytes), pinned host memory that the caller
// keeps until the stream has passed the copy (nullptr: a pageable copy), and the
// minimum diameter lands in *async->min_diam (pinned) for the caller to store in
// the mesh after synchronising the stream.  solver_build returns with its
// initialisation queued on `st`; scal_init, when given, holds the 8 device
// scalars (fixed dt, cfl, t_end ...).
struct MeshBuildAsync {
    std::function<unsigned char *(size_t)> stage;
    double *min_diam = nullptr;
};
int mesh_build(int num_elem, int num_sides, const double *const Vs[6], const int *const es[3],
               const int *const sd[4], BlockPool *pool, cudaStream_t st, const MeshBuildAsync *async,
               dgx_mesh **out);
int solver_build(dgx_mesh *mesh, const dgx_solver_desc *desc, BlockPool *pool, const double *scal_init,
                 cudaStream_t st, dgx_solver **out);
// dgx_project_ic without its closing synchronisation: validated, queued on st
int project_ic_on(dgx_solver *sv, int ic, const double *params, cudaStream_t st);
int periodic_square_arrays(int n, double lx, double ly, double x0, double y0, double jitter,
                           unsigned long long seed, double *V, int *elem_s, int *sides);
constexpr int kReduceLen = 4096;   // partial sums of the fixed-grid reductions

// misc kernels (dgx_misc.cu)
// geometry of an uploaded mesh; scratch holds scratch_len + 1 doubles, with
// scratch_len = min(ceil(E / 256), kReduceLen) (the reduction's grid).  The
// minimum diameter goes to m.min_diam (synchronous) or, with min_diam_dst (pinned
// host memory), is copied there on st for the caller to collect after a sync.
int mesh_geometry(MeshDev &m, double *scratch, int scratch_len, double *min_diam_dst, cudaStream_t st);
// the 96-byte block of a solver's device scalars: scal[8] from scal8, the rest 0
int init_solver_scalars(void *hdr, const double *scal8, cudaStream_t st);
int project_ic(const SolverDev &s, const MeshDev &m, int ic, const double *params, cudaStream_t st);
int launch_dt(SolverDev &s, const MeshDev &m, cudaStream_t st);
// the p = 1 slope limiter on a state vector in place, and the largest
// |c - prev| over the state (FP64, synchronous) (dgx_limit.cu)
int limit_state(const SolverDev &s, const MeshDev &m, void *state, cudaStream_t st);
int state_change(const SolverDev &s, const void *prev, double *out, cudaStream_t st);
// dst = src (whole state vectors) when the current step advanced (dt != 0)
int commit_state(const SolverDev &s, void *dst, const void *src, cudaStream_t st);
// stages per step of an integrator
inline int num_stages(int integrator) { return integrator == DGX_RK4 ? 4 : (integrator == DGX_RK2 ? 2 : 1); }
int conserved_totals(SolverDev &s, const MeshDev &m, double *out, cudaStream_t st);
// The same sums, queued on `st` without host synchronisation: terms holds E
// doubles, scratch kReduceLen + 1; dev_sums[n] receives variable n's sum, to be
// scaled by phi_0 / 2 on the host (bitwise the values conserved_totals returns).
int conserved_sums_async(const SolverDev &s, const MeshDev &m, double *terms, double *scratch,
                         double *dev_sums, cudaStream_t st);
int convert_state(const void *src, int src_is_double, void *dst, int dst_is_double, size_t n,
                  cudaStream_t st);

}  // namespace dgx
