// dgx_batch_fused.cu -- one launch per RK stage for a whole batch of FP32
// solves of mixed orders and equations.
//
// The per-class batched launches (dgx_batch.cu) run each (order, equation)
// class at that class's own occupancy: the kernel of each class is compiled
// for its own register count.  This kernel takes every class in one launch
// per stage over one work list, so a step is the CFL launch and four stage
// launches.  A kernel has one register count, the largest of the classes it
// may run (order-4 Euler: ~250), so every class runs at the occupancy that
// count allows.  It is compiled twice: for two CTAs per SM (no spills) and for
// three (registers capped at 168: order-4 and order-5 Euler spill).  The batch
// autotuner times both against the per-class launches on the live batch.
// Each class's tile is the same stage_tile as the per-class and the plain
// kernels, with the same arguments, so a solve's result is the same bits
// either way.  No counterpart in the reference, which runs one solve per
// process (src/2d/conservation/time_integrator.cu:252-429).
#define DGX_REAL float
#define DGX_REAL_F32
#define DGX_STAGE_BND 0
#define DGX_STAGE_NO_LAUNCHERS
#include "dgx_stage.cuh"

namespace dgx {
namespace {

// one class's tile, out of line: the kernel calls one of them per CTA
template <int P, int EQ>
__device__ __noinline__ void fused_tile(const StageArgs &a, int tile, unsigned char *smem_raw) {
    stage_tile<P, EQ, false>(a, tile, smem_raw, 0u);
}

template <int MINB>
__global__ void __launch_bounds__(kTile, MINB) batch_stage_kernel_fused(const FusedStageArgs f) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ StageArgs s_args;
    constexpr int kWords = sizeof(StageArgs) / sizeof(int);
    static_assert(sizeof(StageArgs) % sizeof(int) == 0, "StageArgs is copied word by word");
    const int4 w = f.items[blockIdx.x];
    if (threadIdx.x == 0) mbar_init(reinterpret_cast<unsigned long long *>(smem_raw), 1);
    if (threadIdx.x < kWords)
        reinterpret_cast<int *>(&s_args)[threadIdx.x] = reinterpret_cast<const int *>(f.args + w.x)[threadIdx.x];
    __syncthreads();
    // a work item outside its solve's tiles (a malformed list) is skipped and
    // reported instead of read out of bounds; uniform over the CTA
    if (w.y < 0 || w.y * kTile >= s_args.E) {
        if (threadIdx.x == 0) atomicOr(s_args.status, kStatusBadItem);
        return;
    }
    switch (w.z) {   // uniform over the CTA
    case 0: fused_tile<0, DGX_ADVECTION>(s_args, w.y, smem_raw); break;
    case 1: fused_tile<0, DGX_EULER>(s_args, w.y, smem_raw); break;
    case 2: fused_tile<1, DGX_ADVECTION>(s_args, w.y, smem_raw); break;
    case 3: fused_tile<1, DGX_EULER>(s_args, w.y, smem_raw); break;
    case 4: fused_tile<2, DGX_ADVECTION>(s_args, w.y, smem_raw); break;
    case 5: fused_tile<2, DGX_EULER>(s_args, w.y, smem_raw); break;
    case 6: fused_tile<3, DGX_ADVECTION>(s_args, w.y, smem_raw); break;
    case 7: fused_tile<3, DGX_EULER>(s_args, w.y, smem_raw); break;
    case 8: fused_tile<4, DGX_ADVECTION>(s_args, w.y, smem_raw); break;
    case 9: fused_tile<4, DGX_EULER>(s_args, w.y, smem_raw); break;
    case 10: fused_tile<5, DGX_ADVECTION>(s_args, w.y, smem_raw); break;
    case 11: fused_tile<5, DGX_EULER>(s_args, w.y, smem_raw); break;
    default:
        if (threadIdx.x == 0) atomicOr(s_args.status, kStatusBadItem);
        break;
    }
}

template <int MINB>
int launch_fused_variant(const FusedStageArgs &f, size_t smem, cudaStream_t st) {
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        DGX_TRY_CUDA(cudaFuncSetAttribute(batch_stage_kernel_fused<MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(smem)));
        DGX_TRY_CUDA(cudaFuncSetAttribute(batch_stage_kernel_fused<MINB>,
                                          cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        configured = smem;
    }
    if (f.n_items > 0) batch_stage_kernel_fused<MINB><<<f.n_items, kTile, smem, st>>>(f);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

}  // namespace

// n_items 0: only sets the kernel's shared-memory limit (outside any capture)
int launch_batch_fused_f32(const FusedStageArgs &f, size_t smem, cudaStream_t st) {
    if (smem > 227 * 1024) { set_error("fused batch: %zu bytes of shared memory per CTA", smem); return DGX_ERR_UNSUPPORTED; }
    return f.min_ctas >= 3 ? launch_fused_variant<3>(f, smem, st) : launch_fused_variant<2>(f, smem, st);
}

int upload_tables_fused() { return upload_tables_impl(); }

}  // namespace dgx
