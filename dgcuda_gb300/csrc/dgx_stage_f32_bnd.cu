// FP32 instantiation of the fused stage kernel (the plain FP32 path),
// for meshes with boundary sides (ghost states).
#define DGX_REAL float
#define DGX_REAL_F32
#define DGX_STAGE_BND 1
#include "dgx_stage.cuh"

namespace dgx {
int launch_stage_f32_b(int order, int equation, const StageArgs &a, cudaStream_t st) {
    return launch_stage_impl(order, equation, a, st);
}
int upload_tables_f32_b() { return upload_tables_impl(); }
int launch_batch_stage_f32_b(int order, int equation, const BatchStageArgs &b, cudaStream_t st) {
    return equation == DGX_EULER ? launch_batch_order<DGX_EULER>(order, b, st)
                                 : launch_batch_order<DGX_ADVECTION>(order, b, st);
}
int launch_batch_param_f32_b(int order, int equation, const BatchParamArgs &p, int grid, cudaStream_t st) {
    return launch_batch_param_impl(order, equation, p, grid, st);
}
}  // namespace dgx
