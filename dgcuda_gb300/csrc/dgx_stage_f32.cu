// FP32 instantiation of the fused stage kernel (the plain FP32 path).
#define DGX_REAL float
#include "dgx_stage.cuh"

namespace dgx {
int launch_stage_f32(int order, int equation, const StageArgs &a, cudaStream_t st) {
    return launch_stage_impl(order, equation, a, st);
}
int upload_tables_f32() { return upload_tables_impl(); }
}  // namespace dgx
