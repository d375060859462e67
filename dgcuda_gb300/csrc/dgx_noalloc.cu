// dgx_noalloc.cu -- conserved totals without any device allocation.
//
// dgx_conserved_totals() allocates its reduction buffers with cudaMalloc on
// every call (and frees them, which synchronises the device).  Some callers
// cannot do that: a serving loop that owns a fixed device-memory budget and
// must not grow it, a host application whose own allocator has reserved the
// device memory, or a latency-critical loop that cannot afford the implicit
// device synchronisation of cudaFree.  dgx_conserved_totals_static() computes
// the same totals with its scratch in a file-scope static device array instead.
#include "dgx_internal.h"

namespace dgx {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocChunk = 2048;        // elements reduced by one block
constexpr int kNoAllocMaxBlocks = 8192;    // partial sums per variable

// Per-block partial sums, [variable][block].  8192 blocks x 2048 elements
// covers meshes of up to 16,777,216 elements; 4 x 8192 doubles = 256 KiB held
// on every device that loads the library, until the process exits.
__device__ __align__(256) double g_totals_scratch[4 * kNoAllocMaxBlocks];

// Host code cannot use g_totals_scratch as an address: look up its device
// address with the calling thread's current device.  The lookup is repeated on
// every call rather than cached, so a host that resets the device
// (cudaDeviceReset, which discards the module and its static arrays) and keeps
// calling gets the array of the new context, not a dangling address.
int scratch_address(double **out) {
    void *p = nullptr;
    DGX_TRY_CUDA(cudaGetSymbolAddress(&p, g_totals_scratch));
    *out = static_cast<double *>(p);
    return DGX_OK;
}

// pass 1: block b sums c_{n,0,e} * J_e over its fixed chunk of elements (fixed
// tree), for every variable, into partial[n * kNoAllocMaxBlocks + b]
template <typename T>
__global__ void totals_partial_kernel(const T *c, const double *J, int E, int np, int nv,
                                      double *partial) {
    __shared__ double sh[kNoAllocThreads];
    const int lo = blockIdx.x * kNoAllocChunk;
    const int hi = min(E, lo + kNoAllocChunk);
    for (int n = 0; n < nv; ++n) {
        const T *cn = c + static_cast<size_t>(n) * np * E;
        double acc = 0.0;
        for (int e = lo + threadIdx.x; e < hi; e += kNoAllocThreads) acc += static_cast<double>(cn[e]) * J[e];
        sh[threadIdx.x] = acc;
        __syncthreads();
        for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) partial[n * kNoAllocMaxBlocks + blockIdx.x] = sh[0];
        __syncthreads();
    }
}

// pass 2: one block sums the partials of each variable in a fixed order
__global__ void totals_final_kernel(const double *partial, int nblocks, int nv, double scale,
                                    double *out) {
    __shared__ double sh[kNoAllocThreads];
    for (int n = 0; n < nv; ++n) {
        double acc = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += kNoAllocThreads) acc += partial[n * kNoAllocMaxBlocks + b];
        sh[threadIdx.x] = acc;
        __syncthreads();
        for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[n] = sh[0] * scale;
        __syncthreads();
    }
}

}  // namespace
}  // namespace dgx

using namespace dgx;

extern "C" int dgx_conserved_totals_static(const dgx_solver *sv, const void *state, double *out,
                                           void *stream) {
    // the handle is const for the caller; its launch counter is bookkeeping
    dgx_solver *counted = const_cast<dgx_solver *>(sv);
    if (!sv || !state || !out) { set_error("NULL argument"); return DGX_ERR_INVALID; }
    const MeshDev &m = sv->mesh->d;
    const SolverDev &s = sv->s;
    const int E = m.num_elem;
    if (E > DGX_TOTALS_STATIC_MAX_ELEMS) {
        set_error("dgx_conserved_totals_static serves meshes of at most %d elements (this one has %d); "
                  "use dgx_conserved_totals", DGX_TOTALS_STATIC_MAX_ELEMS, E);
        return DGX_ERR_INVALID;
    }
    double *partial = nullptr;
    int rc = scratch_address(&partial);
    if (rc) return rc;
    // every partial that pass 2 reads is written by pass 1 of the same call, so
    // nothing in the shared array needs clearing
    const int nblocks = (E + kNoAllocChunk - 1) / kNoAllocChunk;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (s.precision == DGX_FP64)
        totals_partial_kernel<double><<<nblocks, kNoAllocThreads, 0, st>>>(
            static_cast<const double *>(state), m.J, E, s.np, s.nv, partial);
    else
        totals_partial_kernel<float><<<nblocks, kNoAllocThreads, 0, st>>>(
            static_cast<const float *>(state), m.J, E, s.np, s.nv, partial);
    DGX_CHECK_LAUNCH();
    totals_final_kernel<<<1, kNoAllocThreads, 0, st>>>(partial, nblocks, s.nv, tables(s.order).phi[0] * 0.5, out);
    DGX_CHECK_LAUNCH();
    counted->launches += 2;
    return DGX_OK;
}
