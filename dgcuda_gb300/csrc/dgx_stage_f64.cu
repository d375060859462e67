// FP64 instantiation of the fused stage kernel (the reference's precision).
#define DGX_REAL double
#include "dgx_stage.cuh"

namespace dgx {
int launch_stage_f64(int order, int equation, const StageArgs &a, cudaStream_t st) {
    return launch_stage_impl(order, equation, a, st);
}
int upload_tables_f64() { return upload_tables_impl(); }
}  // namespace dgx
