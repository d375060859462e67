// dgx_tc_selftest.cu -- known-answer test of the tensor-core path on this
// device: one CTA multiplies small-integer BF16 matrices (exact in FP32) with
// tcgen05.mma, once with A in shared memory and once with A in tensor memory,
// and compares every accumulator element with the SIMT product.  No reference
// counterpart; the BF16x3 solver path runs it once per process before use.
#include <cuda_bf16.h>

#include "dgx_internal.h"
#include "dgx_tc.cuh"

namespace dgx {
namespace {

constexpr int kM = 128, kN = 32, kK = 16;

__device__ __forceinline__ float a_val(int m, int k) { return static_cast<float>((3 * m + 5 * k) % 7 - 3); }
__device__ __forceinline__ float b_val(int n, int k) { return static_cast<float>((2 * n + k) % 5 - 2); }

// byte offset of element (row, k) in the K-major core-matrix layout with
// K-chunk stride 128 bytes and 8-row-group stride 256 bytes (K = 16)
__device__ __forceinline__ unsigned kmajor_off(int row, int k) {
    return static_cast<unsigned>((row / 8) * 256 + (k / 8) * 128 + (row % 8) * 16 + (k % 8) * 2);
}

// variant 0 encodes the layout as (LBO = 128, SBO = 256); variant 1 as the
// exchanged pair.  Both stay inside the operand buffers.
__global__ void __launch_bounds__(kM, 1) tc_selftest_kernel(float *out, unsigned *status, int variant) {
    __shared__ __align__(1024) unsigned char sA[kM * kK * 2];
    __shared__ __align__(1024) unsigned char sB[kN * kK * 2];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ unsigned taddr_slot;
    const int t = threadIdx.x;

    // operands: thread t writes row t of A (and row t of B for t < 32)
    for (int k = 0; k < kK; ++k) {
        *reinterpret_cast<__nv_bfloat16 *>(sA + kmajor_off(t, k)) = __float2bfloat16_rn(a_val(t, k));
        if (t < kN) *reinterpret_cast<__nv_bfloat16 *>(sB + kmajor_off(t, k)) = __float2bfloat16_rn(b_val(t, k));
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::smem_u32(&bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (t < 32) tc::tmem_alloc(&taddr_slot, 128);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const unsigned taddr = taddr_slot;

    // the same A row into tensor memory, columns 64..71 (two BF16 per column)
    {
        unsigned w[8];
        for (int c = 0; c < 8; ++c) w[c] = tc::pack_bf16(a_val(t, 2 * c), a_val(t, 2 * c + 1));
        tc::tmem_st8(tc::tmem_lane_base(taddr) + 64, w);
        tc::tmem_wait_st();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    if (t == 0) {
        const unsigned lbo = variant ? 256u : 128u, sbo = variant ? 128u : 256u;
        const uint64_t da = tc::smem_desc(tc::smem_u32(sA), lbo, sbo);
        const uint64_t db = tc::smem_desc(tc::smem_u32(sB), lbo, sbo);
        constexpr unsigned idesc = tc::idesc_bf16_f32(kM, kN);
        tc::mma_ss(taddr, da, db, idesc, 0u);            // D1 in columns 0..31
        tc::mma_ts(taddr + 32, taddr + 64, db, idesc, 0u);  // D2 in columns 32..63
        tc::mma_commit(&bar);
    }
    bool done = false;
    for (long long it = 0; it < (1ll << 24) && !done; ++it) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(tc::smem_u32(&bar))
            : "memory");
        done = ok != 0;
    }
    if (!done) {
        if (t == 0) atomicOr(status + 2, 1u);
        // give the tensor core a last, longer chance before the memory is freed
        for (long long it = 0; it < (1ll << 28) && !done; ++it) {
            unsigned ok;
            asm volatile(
                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
                : "=r"(ok)
                : "r"(tc::smem_u32(&bar))
                : "memory");
            done = ok != 0;
        }
    }
    tc::fence_after_sync();
    if (done) {
        float d1[32], d2[32];
        const unsigned lane = tc::tmem_lane_base(taddr);
        tc::tmem_ld16(lane + 0, d1);
        tc::tmem_ld16(lane + 16, d1 + 16);
        tc::tmem_ld16(lane + 32, d2);
        tc::tmem_ld16(lane + 48, d2 + 16);
        tc::tmem_wait_ld();
        unsigned bad1 = 0, bad2 = 0;
        for (int n = 0; n < kN; ++n) {
            float ref = 0.f;
            for (int k = 0; k < kK; ++k) ref += a_val(t, k) * b_val(n, k);
            bad1 += d1[n] != ref;
            bad2 += d2[n] != ref;
            out[t * 2 * kN + n] = d1[n];
            out[t * 2 * kN + kN + n] = d2[n];
        }
        if (bad1) atomicAdd(status + 0, bad1);
        if (bad2) atomicAdd(status + 1, bad2);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (t < 32) tc::tmem_dealloc(taddr, 128);
}

}  // namespace
}  // namespace dgx

using namespace dgx;

extern "C" int dgx_tc_selftest(int variant, int *bad_ss, int *bad_ts, float *values) {
    if (variant != 0 && variant != 1) { set_error("variant must be 0 or 1"); return DGX_ERR_INVALID; }
    float *d_out = nullptr;
    unsigned *d_status = nullptr;
    DGX_TRY_CUDA(cudaMalloc(&d_out, sizeof(float) * kM * 2 * kN));
    cudaError_t ce = cudaMalloc(&d_status, sizeof(unsigned) * 4);
    if (ce == cudaSuccess) ce = cudaMemset(d_status, 0, sizeof(unsigned) * 4);
    if (ce == cudaSuccess) ce = cudaMemset(d_out, 0, sizeof(float) * kM * 2 * kN);
    unsigned st[4] = {0, 0, 0, 0};
    if (ce == cudaSuccess) {
        tc_selftest_kernel<<<1, kM>>>(d_out, d_status, variant);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    if (ce == cudaSuccess) ce = cudaMemcpy(st, d_status, sizeof(st), cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && values)
        ce = cudaMemcpy(values, d_out, sizeof(float) * kM * 2 * kN, cudaMemcpyDeviceToHost);
    cudaFree(d_out);
    cudaFree(d_status);
    if (ce != cudaSuccess) { set_error("tensor-core self-test: %s", cudaGetErrorString(ce)); return DGX_ERR_CUDA; }
    if (bad_ss) *bad_ss = static_cast<int>(st[0]);
    if (bad_ts) *bad_ts = static_cast<int>(st[1]);
    if (st[2]) { set_error("tensor-core self-test: the MMA did not complete in time"); return DGX_ERR_TIMEOUT; }
    return DGX_OK;
}
