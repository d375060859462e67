// dgx_tc.cuh -- fifth-generation tensor-core primitives (tcgen05, sm_100+
// family) in inline PTX: tensor-memory allocation, the shared-memory matrix
// descriptor, the instruction descriptor of kind::f16 (BF16 inputs, FP32
// accumulation), MMA issue and commit, and tensor-memory loads and stores.
//
// Conventions used by this code base:
//   * One CTA, cta_group::1, M = 128: row m of the accumulator is tensor-memory
//     lane m, so with 128 threads thread t (warp t/32) owns row t and moves it
//     with the 32x32b load/store shapes.
//   * Operands in shared memory are K-major without swizzle: 8-row x 16-byte
//     core matrices stored as 128 contiguous bytes; core matrices adjacent in K
//     are LBO bytes apart, 8-row groups SBO bytes apart.
//   * An A operand in tensor memory holds row m in lane m, two BF16 values of
//     consecutive K per 32-bit column (the lower K in the low half).
#pragma once

#include <cstdint>

namespace dgx {
namespace tc {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// ---- tensor memory ----------------------------------------------------------
// Allocate `ncols` columns (a power of two, >= 32) for the CTA; executed by one
// whole warp; the base address is written to shared memory at `dst`.
__device__ __forceinline__ void tmem_alloc(unsigned *dst, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// Free the allocation; executed by the warp that allocated it.
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes of shared memory -> visible to the tensor core
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16 consecutive columns of this thread's lane (warp w reads lanes 32(w%4)..)
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float *v) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld8(unsigned taddr, float *v) {
    unsigned r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld4(unsigned taddr, float *v) {
    unsigned r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 8 consecutive 32-bit columns of this thread's lane
__device__ __forceinline__ void tmem_st8(unsigned taddr, const unsigned *r) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
                 : "memory");
}
__device__ __forceinline__ void tmem_st1(unsigned taddr, unsigned r0) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x1.b32 [%0], {%1};" ::"r"(taddr), "r"(r0) : "memory");
}
__device__ __forceinline__ void tmem_st2(unsigned taddr, unsigned r0, unsigned r1) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1,%2};" ::"r"(taddr), "r"(r0), "r"(r1) : "memory");
}
__device__ __forceinline__ void tmem_st4(unsigned taddr, const unsigned *r) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr), "r"(r[0]), "r"(r[1]),
                 "r"(r[2]), "r"(r[3])
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// lane field of a tensor-memory address for this warp's 32x32b accesses
__device__ __forceinline__ unsigned tmem_lane_base(unsigned taddr) {
    return taddr + ((static_cast<unsigned>(threadIdx.x / 32) % 4u) * 32u << 16);
}

// ---- descriptors ------------------------------------------------------------
// Shared-memory matrix descriptor, K-major, no swizzle: start address, LBO
// (bytes between core matrices adjacent in K), SBO (bytes between 8-row
// groups); bits 46-47 carry the descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    return d;   // base offset 0, absolute LBO mode 0, layout type 0 (no swizzle)
}
// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr unsigned idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<unsigned>(N >> 3) << 17) |
           (static_cast<unsigned>(M >> 4) << 24);
}

// ---- MMA --------------------------------------------------------------------
// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void mma_ss(unsigned d_tmem, uint64_t a_desc, uint64_t b_desc, unsigned idesc,
                                       unsigned accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// D[tmem] (+)= A[tmem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void mma_ts(unsigned d_tmem, unsigned a_tmem, uint64_t b_desc, unsigned idesc,
                                       unsigned accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The mbarrier completes one arrival when every MMA this thread issued before
// has finished.
__device__ __forceinline__ void mma_commit(unsigned long long *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// ---- BF16 hi/lo split ---------------------------------------------------------
// x = hi + lo + O(2^-17 |x|): hi = bf16(x), lo = bf16(x - hi); two values per
// 32-bit word (the first in the low half)
__device__ __forceinline__ unsigned pack_bf16(float a, float b) {
    unsigned r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
    return r;
}
// One value as the BF16 pair (hi, lo) in one 32-bit word, hi in the low half:
// hi = bf16(x), lo = bf16(x - hi)
__device__ __forceinline__ unsigned split_word(float x) {
    unsigned h, w;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(0.0f), "f"(x));
    const float r = x - __uint_as_float(h << 16);
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(w) : "f"(r), "f"(x));
    return w;
}
__device__ __forceinline__ void split_bf16(float a, float b, unsigned &hi, unsigned &lo) {
    hi = pack_bf16(a, b);
    const float ah = __uint_as_float(hi << 16), bh = __uint_as_float(hi & 0xFFFF0000u);
    lo = pack_bf16(a - ah, b - bh);
}

}  // namespace tc
}  // namespace dgx
