// dgx_stage.cuh -- the fused RHS / RK-stage kernel, one thread per element.
//
// Included by dgx_stage_f32.cu and dgx_stage_f64.cu with DGX_REAL defined as
// the arithmetic type.  Each translation unit owns its copy of the constant
// tables (uploaded by upload_tables_f32/_f64).
//
// One CTA per tile of kTile consecutive elements, one thread per element.
// Phase 1 writes each element's traces on its three sides (p+1 Gauss points)
// to shared memory and, one halo entry per thread, the traces of the tile's
// neighbours outside the tile (their gathers issued together); phase 2, after
// one barrier, reads both traces of every side from shared memory.
// Per element e the kernel computes
//   volume   V_i = sum_q gx_iq (Fx ys - Fy xs) + gy_iq (Fy xr - Fx yr)      at U(q)
//            (src/2d/conservation/conserv_kernels.cu:766-811)
//   surface  for each local side k: own trace and neighbour trace at the p+1
//            Gauss points (the neighbour's points in reverse order), the
//            numerical flux Fhat(U_left, U_right, n_left) and the lift
//            -+ len/2 sum_j w_j Fhat_j phi_i(j)  (conserv_kernels.cu:697-758)
//   rhs      k = dt/J (V + sum of the three sides), sides in local order
//            0,1,2 (time_integrator.cu:130-188)
// and fuses the RK4 combination of the stage (time_integrator.cu:194-218).
// The flux of a side is evaluated by both of its elements with the same
// arguments (left trace, right trace, left normal) and the same instruction
// sequence, so the two evaluations agree bit for bit; there are no atomics and
// the result does not depend on scheduling.
#pragma once

#include "dgx_ic.cuh"
#include "dgx_internal.h"

#ifndef DGX_REAL
#error "define DGX_REAL before including dgx_stage.cuh"
#endif
// DGX_STAGE_BND selects the kernels this translation unit instantiates: 0 for
// meshes without boundary sides (no ghost-state code at all), 1 for meshes with
// them
#ifndef DGX_STAGE_BND
#error "define DGX_STAGE_BND (0 or 1) before including dgx_stage.cuh"
#endif

// Loops over quadrature points (and, optionally, sides) are kept rolled: the
// fully unrolled kernel is several times larger than the instruction cache and
// stalls on instruction fetch; with a uniform loop index the table operands
// still come from the constant bank.
#ifndef DGX_ROLLED_VOLUME
#define DGX_ROLLED_VOLUME 1
#endif
#ifndef DGX_ROLLED_SIDES
#define DGX_ROLLED_SIDES 0
#endif
#ifndef DGX_ROLLED_TRACES
#define DGX_ROLLED_TRACES 0
#endif

namespace dgx {

static __constant__ __align__(16) DGX_REAL c_tab[kTableTotal];

// The same tables transposed, mode index fastest and padded to an even count
// (the pad is 0): phi, gx, gy as [q][i], side and lift as [side][j][i].  Modes
// 2m and 2m+1 are adjacent and 8-byte aligned, the operand of one paired FMA.
DGX_HD constexpr int np_even(int p) { return (num_modes(p) + 1) & ~1; }
DGX_HD constexpr int tabt_block(int p) { return ((3 * num_quad(p) + 6 * num_quad1(p)) * np_even(p) + 3) & ~3; }
DGX_HD constexpr int tabt_offset(int p) { return p == 0 ? 0 : tabt_offset(p - 1) + tabt_block(p - 1); }
constexpr int kTabTTotal = tabt_offset(kMaxOrder + 1);
template <int P>
struct LayT {
    static constexpr int NPP = np_even(P), NQ = num_quad(P), NQ1 = num_quad1(P);
    static constexpr int PHI = tabt_offset(P);
    static constexpr int GX = PHI + NQ * NPP;
    static constexpr int GY = GX + NQ * NPP;
    static constexpr int SIDE = GY + NQ * NPP;
    static constexpr int LIFT = SIDE + 3 * NQ1 * NPP;
};
#ifdef DGX_REAL_F32
static __constant__ __align__(16) float c_tabT[kTabTTotal];
#endif
constexpr bool kStageBnd = DGX_STAGE_BND != 0;

template <typename T>
__device__ __forceinline__ T pick3(T a0, T a1, T a2, int k) { return k == 0 ? a0 : (k == 1 ? a1 : a2); }

template <int P>
struct Lay {
    static constexpr int NP = num_modes(P), NQ = num_quad(P), NQ1 = num_quad1(P);
    static constexpr int PHI = table_offset(P);
    static constexpr int GX = PHI + NP * NQ;
    static constexpr int GY = GX + NP * NQ;
    static constexpr int SIDE = GY + NP * NQ;
    static constexpr int LIFT = SIDE + 3 * NP * NQ1;
    static constexpr int W1 = LIFT + 3 * NP * NQ1;
    static constexpr int SRS = W1 + NQ1;
};

using R = DGX_REAL;

// FP32: the SFU reciprocal and reciprocal square root (a few ulp, far inside
// the FP32 path's tolerance); FP64: IEEE division and square root.
__device__ __forceinline__ float rrcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double rrcp(double x) { return 1.0 / x; }
__device__ __forceinline__ float rsqrt_(float x) { return x * rsqrtf(x); }   // x > 0
__device__ __forceinline__ double rsqrt_(double x) { return sqrt(x); }

// ---- bulk asynchronous copies (TMA engine) into shared memory -------------
__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// global -> shared, 16-byte aligned addresses, size a multiple of 16
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes,
                                              unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase with the given parity: false if the limit ran out.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity, long long limit) {
    for (long long it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Physical flux (Fx, Fy) at a point: advection a*u, Euler
// (src/2d/conservation/euler/euler.cu:92-117).
template <int EQ>
__device__ __forceinline__ void phys_flux(const R *U, R g, R ax, R ay, R *fx, R *fy) {
    if constexpr (EQ == DGX_ADVECTION) {
        fx[0] = ax * U[0];
        fy[0] = ay * U[0];
    } else {
        const R ir = rrcp(U[0]);
        const R u = U[1] * ir, v = U[2] * ir;
        const R p = (g - R(1)) * (U[3] - R(0.5) * (U[1] * u + U[2] * v));
        fx[0] = U[1];         fy[0] = U[2];
        fx[1] = U[1] * u + p; fy[1] = U[1] * v;
        fx[2] = U[2] * u;     fy[2] = U[2] * v + p;
        fx[3] = (U[3] + p) * u;
        fy[3] = (U[3] + p) * v;
    }
}

// Numerical flux Fhat . n with n oriented out of the left element:
// 1/2 [ (F(UL) + F(UR)) . n + lambda (UL - UR) ] with the local Lax-Friedrichs
// lambda = max(|u_n| + c) over both sides (euler.cu:127-168), lambda = |a.n| for
// advection; lambda = 0 for the central flux (2dadvec_kernels.cu:162-164).
template <int EQ>
__device__ __forceinline__ void num_flux(const R *UL, const R *UR, R nx, R ny, int llf, R g,
                                         R ax, R ay, R *Fh) {
    if constexpr (EQ == DGX_ADVECTION) {
        const R an = ax * nx + ay * ny;
        const R lam = llf ? fabs(an) : R(0);
        Fh[0] = R(0.5) * (an * (UL[0] + UR[0]) + lam * (UL[0] - UR[0]));
    } else {
        const R irl = rrcp(UL[0]), irr = rrcp(UR[0]);
        const R ul = UL[1] * irl, vl = UL[2] * irl, ur = UR[1] * irr, vr = UR[2] * irr;
        const R pl = (g - R(1)) * (UL[3] - R(0.5) * (UL[1] * ul + UL[2] * vl));
        const R pr = (g - R(1)) * (UR[3] - R(0.5) * (UR[1] * ur + UR[2] * vr));
        const R unl = ul * nx + vl * ny, unr = ur * nx + vr * ny;
        R lam = R(0);
        if (llf) {
            const R ll = fabs(unl) + rsqrt_(g * pl * irl);
            const R lr = fabs(unr) + rsqrt_(g * pr * irr);
            lam = ll > lr ? ll : lr;
        }
        const R fl[4] = {UL[1] * nx + UL[2] * ny, UL[1] * unl + pl * nx, UL[2] * unl + pl * ny,
                         (UL[3] + pl) * unl};
        const R fr[4] = {UR[1] * nx + UR[2] * ny, UR[1] * unr + pr * nx, UR[2] * unr + pr * ny,
                         (UR[3] + pr) * unr};
#pragma unroll
        for (int n = 0; n < 4; ++n) Fh[n] = R(0.5) * ((fl[n] + fr[n]) + lam * (UL[n] - UR[n]));
    }
}

// Physical position of Gauss point j of local side k of element e, in FP64:
// Vk + t_j (Vk+1 - Vk) with t_j = (1 + s_j)/2, the point the reference's
// boundary hooks map from the element (euler.cu:186-205) written along the
// side, so that it lies on the side for any rounding of the table (a point on
// an axis keeps its sign)
template <int P>
__device__ __forceinline__ void side_point_xy(const StageArgs &a, int e, int k, int j, double &x, double &y) {
    const size_t E = static_cast<size_t>(a.E);
    const double *V = a.V;
    const int kb = k == 2 ? 0 : k + 1;
    const double t = static_cast<double>(c_tab[Lay<P>::SRS + 2 * j]);   // side 0: r = (1 + s_j)/2
    const double xa = V[2 * k * E + e], ya = V[(2 * k + 1) * E + e];
    x = xa + t * (V[2 * kb * E + e] - xa);
    y = ya + t * (V[(2 * kb + 1) * E + e] - ya);
}

// Ghost state on a boundary side (the element is the side's left element, n
// points out of the domain), at the side's point j in this element's order:
//   Euler  -1 reflecting: density and energy kept, momentum reduced to its
//             tangential part (the reference's reflecting_boundary,
//             src/2d/conservation/euler/cylinder/cylinder.cu:58-111, with the
//             side's normal);
//          -2 outflow, -3 inflow: the solver's free-stream state (the problem
//             hooks U_outflow / U_inflow, src/2d/conservation/euler/euler.cu:177-241),
//             or the interior state when none is set;
//   advection: the initial condition translated by a*t (the reference's
//             boundary_exact, src/2d/2dadvec/2dadvec_kernels.cu:184-186,492-517),
//             or the interior state when none is set.
template <int P, int EQ>
__device__ __noinline__ void boundary_ghost(const StageArgs &a, int tag, int k, int j, int e, const R *UO,
                                            R nx, R ny, R *UN) {
    using L = Lay<P>;
    constexpr int NQ1 = L::NQ1;
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    if constexpr (EQ == DGX_EULER) {
        if (a.bc_kind == 3) {   // the problem file's own hooks (DGX_BC_PROBLEM)
            const double *prm = a.bc_params;
            const double g = a.gamma;
            double U[4];
            if (a.bc_ic == DGX_IC_THREEPOINT && tag == -1) {
                // flip the x momentum where m.n > 0, else the y momentum
                // (threepoint.cu:86-109; its sqrtf(m.n) > 0 test is m.n > 0 in FP32)
                const bool out = static_cast<float>(UO[1] * nx + UO[2] * ny) > 0.f;
                UN[0] = UO[0];
                UN[1] = out ? -UO[1] : UO[1];
                UN[2] = out ? UO[2] : -UO[2];
                UN[3] = UO[3];
                return;
            }
            // side point (side 1 exchanged for the radial reflections, as the
            // reference's reflecting_boundary maps it, cylinder.cu:78-81)
            const int jj = (tag == -1 && k == 1) ? NQ1 - 1 - j : j;
            double x, y;
            side_point_xy<P>(a, e, k, jj, x, y);
            if (tag == -1) {   // keep the momentum tangential to the circle through the point
                const double c0 = a.bc_ic == DGX_IC_CYLINDER ? 0.5 : 0.0;
                x -= c0;
                y -= c0;
                // the radius in FP64, or as the reference's hooks take it, sqrtf
                // of the FP64 sum (cylinder.cu:100, supersonic.cu:100)
                const double d = a.hook_float ? static_cast<double>(sqrtf(static_cast<float>(x * x + y * y)))
                                              : sqrt(x * x + y * y);
                const R Nx = static_cast<R>(x / d), Ny = static_cast<R>(y / d);
                const R tm = UO[1] * Ny - UO[2] * Nx;
                UN[0] = UO[0];
                UN[1] = tm * Ny;
                UN[2] = -tm * Nx;
                UN[3] = UO[3];
                return;
            }
            if (a.bc_ic == DGX_IC_THREEPOINT) {
                const double ang = prm[1] * kRefPi / 180.0;
                const double t = a.mode == 0 ? a.t : a.scal[2] + a.stage_c * a.scal[0];
                if (tag == -2 || x < prm[0] * t * cos(ang) + tan(ang)) threepoint_shock(prm, g, U);
                else ic_eval(DGX_IC_THREEPOINT, prm, g, x, y, U);
            } else {
                ic_eval(a.bc_ic, prm, g, x, y, U, a.hook_float != 0);
            }
            for (int n = 0; n < 4; ++n) UN[n] = static_cast<R>(U[n]);
            return;
        }
        if (tag == -1) {
            const R mn = UO[1] * nx + UO[2] * ny;
            UN[0] = UO[0];
            UN[1] = UO[1] - mn * nx;
            UN[2] = UO[2] - mn * ny;
            UN[3] = UO[3];
        } else if (a.bc_kind == 1) {
            for (int n = 0; n < 4; ++n) UN[n] = R(a.bc_state[n]);
        } else {
            for (int n = 0; n < 4; ++n) UN[n] = UO[n];
        }
    } else {
        if (a.bc_kind == 2) {
            double x, y;
            side_point_xy<P>(a, e, k, j, x, y);
            const double t = a.mode == 0 ? a.t : a.scal[2] + a.stage_c * a.scal[0];
            double U[4];
            ic_eval(a.bc_ic, a.bc_params, a.gamma, x - a.ax * t, y - a.ay * t, U);
            UN[0] = static_cast<R>(U[0]);
        } else {
            for (int n = 0; n < NV; ++n) UN[n] = UO[n];
        }
    }
}

// Shared memory of one CTA: the side tables (for traces on a runtime side) and
// the trace slots, slot-major: s_tr[slot_off(slot) + j*NV + n], so a thread
// addresses a whole slot from one base register.  The 32 threads of a warp
// write and read their own slots 3*tid + k together, so those slots must start
// in 32 distinct banks.  An odd stride (NV*NQ1 | 1 words) does that.  For a
// slot of 16 floats (Euler, p = 3) the slots are packed at stride 16 with one
// word of padding per 6 slots instead: slot s starts at 16 s + s/6; the 16
// threads whose slots have one parity start at s/6 = 16 w + u (u = 0..15, w
// the warp) and the two parities 16 banks apart.  That takes nslot/6 words of
// padding where the odd stride takes nslot: 1.7 KB less per CTA at 516 slots,
// which keeps three CTAs of the order-3 Euler kernel on an SM with the widened
// (132-value) prefetch planes of a mesh whose element count is not a multiple
// of 4.
template <int P, int NV>
DGX_HD constexpr int side_table_words() { return (3 * ((num_modes(P) + 1) & ~1) * num_quad1(P) + 3) & ~3; }
template <int P, int NV>
DGX_HD constexpr bool slot_pad6() { return sizeof(R) == 4 && NV * num_quad1(P) == 16; }
template <int P, int NV>
DGX_HD constexpr int slot_words() { return slot_pad6<P, NV>() ? 16 : (NV * num_quad1(P)) | 1; }
template <int P, int NV>
DGX_HD __forceinline__ constexpr int slot_off(int slot) {
    return slot * slot_words<P, NV>() + (slot_pad6<P, NV>() ? slot / 6 : 0);
}
// words of the slot area for nslot slots (a multiple of 4: what follows it is
// 16-byte aligned)
template <int P, int NV>
DGX_HD constexpr size_t slot_area_words(int nslot) {
    return (static_cast<size_t>(slot_off<P, NV>(nslot)) + 3) & ~static_cast<size_t>(3);
}

// Prefetched epilogue operands: per plane (variable x mode) of the base state
// and of the accumulator, the tile's slice, widened to 16-byte boundaries (the
// bulk copy needs 16-byte aligned ends, and a plane of E values starts on one
// only when E is a multiple of kPreAlign).  StageArgs::prefetch holds the
// values per plane in shared memory: kTile when E is a multiple of kPreAlign,
// kTile + kPreAlign otherwise (0: no prefetch).
constexpr int kPreAlign = 16 / static_cast<int>(sizeof(R));
template <int P, int NV>
DGX_HD constexpr size_t prefetch_bytes(int plane) {
    return sizeof(R) * 2 * NV * num_modes(P) * static_cast<size_t>(plane);
}

template <int P, int NV>
DGX_HD constexpr size_t stage_smem_bytes(int nslot, int prefetch) {
    return 16 + sizeof(R) * (static_cast<size_t>(side_table_words<P, NV>()) + slot_area_words<P, NV>(nslot)) +
           prefetch_bytes<P, NV>(prefetch);
}

// One tile of one solve.  `bar` is an initialised mbarrier; `parity` the phase
// this tile's prefetch (if any) completes; returns whether a prefetch was
// issued (the caller then advances its phase).  All threads of the CTA call it
// with the same arguments; on return no copy of this tile is in flight.
// Start the TMA bulk copies of the tile's epilogue operands (modes 2..4: the
// base state for 2, 3 and the accumulator for 2, 3, 4) into `s_pre`, completing
// on `bar`; returns whether copies were issued.
template <int P, int NV>
__device__ __forceinline__ bool issue_prefetch(const StageArgs &a, int tile, unsigned long long *bar, R *s_pre,
                                               int tid) {
    constexpr int NP = num_modes(P);
    const int E = a.E;
    const size_t SE = static_cast<unsigned>(E);   // zero-extended: plane offsets k*SE are 32x32-bit products
    const bool pre = a.prefetch && ((a.mode >= 2 && a.mode <= 4) || (a.comp && a.mode == 1));
    if (pre && tid < 32) {
        // order this CTA's earlier generic-proxy accesses of the shared memory
        // (a previous tile) before the bulk copies that overwrite it
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int cnt = min(kTile, E - tile * kTile);
        const int nplanes = NV * NP;
        // mode 2 and 3: the base state, then the accumulator (13-pass RK4: mode
        // 2 the base state alone, mode 3 the base state and u2); mode 4: the
        // accumulator
        // compensated RK4: mode 1 the state's low part, modes 2-4 the base
        // state and the increment accumulator
        const bool base_only = (a.rk13 && a.mode == 2) || (a.comp && a.mode == 1);
        const int ncopy = ((a.mode == 4 && !a.comp) || base_only) ? nplanes : 2 * nplanes;
        // plane pl's slice [g0, g0 + cnt) widened to [g0 & -A, (g0 + cnt + A-1) & -A)
        // (the state buffers carry 16 bytes of slack past their end)
        const size_t A = kPreAlign;
        if (tid == 0) {
            unsigned total = 0;
            for (int pl = 0; pl < nplanes; ++pl) {
                const size_t g0 = pl * SE + static_cast<size_t>(tile) * kTile;
                total += static_cast<unsigned>((((g0 + cnt + A - 1) & ~(A - 1)) - (g0 & ~(A - 1))) * sizeof(R));
            }
            mbar_expect_tx(bar, total * (ncopy / nplanes));
        }
        __syncwarp();
        for (int q = tid; q < ncopy; q += 32) {
            // planes [0, nplanes): base state (modes 2, 3), then the accumulator
            // (13-pass mode 3: u2); mode 4 copies only the accumulator, to
            // planes [0, nplanes)
            const int which = (a.mode == 4 && !a.comp) ? 1 : (q >= nplanes);
            const int pl = q % nplanes;
            const size_t g0 = pl * SE + static_cast<size_t>(tile) * kTile;
            const size_t a0 = g0 & ~(A - 1), a1 = (g0 + cnt + A - 1) & ~(A - 1);
            const void *second = (a.rk13 && a.mode == 3) ? a.aux : a.acc;
            const void *first = (a.comp && a.mode == 1) ? a.aux : a.c;
            const R *src = static_cast<const R *>(which ? second : first) + a0;
            bulk_copy_g2s(s_pre + static_cast<size_t>(q) * a.prefetch, src, static_cast<unsigned>((a1 - a0) * sizeof(R)),
                          bar);
        }
    }

    return pre;
}

template <int K>
struct IntC {
    static constexpr int value = K;
};

// Mass inverse and the RK combination of the stage (time_integrator.cu:194-218,
// 445-464, 622-700): k = dt/J rhs, then per mode of the kernel
//   0 k;  1 u2 = c + k/2, acc = c + k/6;  2/3 u = c + alpha k, acc += k/3;
//   4 c = acc + k/6;  5 out = u + alpha k;  6 out = c + alpha k;
// in the 13-pass RK4 form (a.rk13, see rk4_stage_args) modes 1 and 2 write no
// accumulator and mode 3 forms it, acc = c + ((u2 - c) + 2 (u3 - c) + k3)/3,
// with u3 this stage's input (the `c` argument) and u2 from a.aux.
// Writes the variables V0 .. V0+VC-1 (all of them by default; rhs and c hold
// just those).  Waits (bounded) for the tile's prefetched base state and
// accumulator when `pre`; `row` is the element's index in the tile; returns
// `pre`.
template <int P, int EQ, int V0 = 0, int VC = (EQ == DGX_EULER) ? 4 : 1>
__device__ __forceinline__ bool stage_epilogue(const StageArgs &a, const R (&rhs)[VC][num_modes(P)],
                                               const R (&c)[VC][num_modes(P)], R dt, R invJ,
                                               int e, size_t SE, bool pre, const R *s_pre,
                                               unsigned long long *bar, unsigned parity, int row) {
    constexpr int NP = num_modes(P);
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    const R sc = dt * invJ;
    R *__restrict__ out = static_cast<R *>(a.out);
    R *__restrict__ oe = out + e;   // (array + element) + plane * E: one wide multiply-add per access
    if (pre) {
        if (!mbar_wait_bounded(bar, parity, 1ll << 26)) {
            // the copies did not land in time: report, wait once more for the
            // copies still in flight (they write this CTA's shared memory), skip
            atomicOr(a.status, kStatusCopyTimeout);
            mbar_wait_bounded(bar, parity, 1ll << 28);
            return pre;
        }
    }
    // Modes 2..4 read this element's base state and accumulator, value pi =
    // (variable, mode) of each: kind 0 from global memory; kind 1 from the
    // prefetched planes (a.prefetch values each; plane pi's slice starts
    // (pi * (E mod kPreAlign)) mod kPreAlign values into its copy); kind 2 from
    // kTile-value planes (E a multiple of kPreAlign), at compile-time offsets.
    auto rk_tail = [&](auto kind) {
        constexpr int K = decltype(kind)::value;
        // the second operand: the accumulator, or u2 in mode 3 of the 13-pass form
        const bool from_u2 = a.rk13 && a.mode == 3;
        const R *pc, *pacc;
        if constexpr (K == 0) {
            pc = static_cast<const R *>((a.comp && a.mode == 1) ? a.aux : a.c) + e;
            pacc = static_cast<const R *>(from_u2 ? a.aux : a.acc) + e;
        } else {
            pc = s_pre + row;
            pacc = s_pre + ((a.mode == 4 && !a.comp) ? 0 : NV * NP * a.prefetch) + row;
        }
        const int pstride = a.prefetch, sm = static_cast<int>(SE & (kPreAlign - 1));
        auto at = [&](const R *p, int pi) -> R {
            if constexpr (K == 2) return p[pi * kTile];
            else if constexpr (K == 1) return p[pi * pstride + ((pi * sm) & (kPreAlign - 1))];
            else return p[pi * SE];
        };
        if (a.comp) {
            // compensated RK4 (pc: the state's low part in mode 1, else the
            // base state; pacc: the increment accumulator D)
            R *__restrict__ ae = static_cast<R *>(a.acc) + e;
            if (a.mode == 1) {          // u2 = c + k1/2, D = lo + k1/6
#pragma unroll
                for (int n = 0; n < VC; ++n)
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        const int pi = (V0 + n) * NP + i;
                        const R kk = sc * rhs[n][i];
                        oe[pi * SE] = fma(R(0.5), kk, c[n][i]);
                        ae[pi * SE] = fma(R(1.0 / 6.0), kk, at(pc, pi));
                    }
            } else if (a.mode == 4) {   // (c, lo) = two-sum(c, D + k4/6)
                // c is read and written in place (each thread its own values,
                // no other thread reads them in this stage): plain pointers
                R *oc = static_cast<R *>(a.out) + e;
                R *ol = static_cast<R *>(a.aux) + e;
#pragma unroll
                for (int n = 0; n < VC; ++n)
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        const int pi = (V0 + n) * NP + i;
                        const R y = fma(R(1.0 / 6.0), sc * rhs[n][i], at(pacc, pi));
                        const R b = at(pc, pi);
                        const R t = b + y;   // the two-sum (Knuth): t + err = b + y exactly
                        const R bp = t - b;
                        const R err = (b - (t - bp)) + (y - bp);
                        oc[pi * SE] = t;
                        ol[pi * SE] = err;
                    }
            } else {                    // 2, 3: u = c + alpha k, D += k/3
                const R alpha = a.mode == 2 ? R(0.5) : R(1);
#pragma unroll
                for (int n = 0; n < VC; ++n)
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        const int pi = (V0 + n) * NP + i;
                        const R kk = sc * rhs[n][i];
                        oe[pi * SE] = fma(alpha, kk, at(pc, pi));
                        ae[pi * SE] = fma(R(1.0 / 3.0), kk, at(pacc, pi));
                    }
            }
        } else if (a.mode == 4) {   // c = acc + k4/6
#pragma unroll
            for (int n = 0; n < VC; ++n)
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    const int pi = (V0 + n) * NP + i;
                    oe[pi * SE] = fma(R(1.0 / 6.0), sc * rhs[n][i], at(pacc, pi));
                }
        } else if (a.rk13) {
            // 2: u3 = c + k2/2;  3: u4 = c + k3 (over u2) and
            //    acc = c + ((u2 - c) + 2 (u3 - c) + k3) / 3, u3 the stage's input
            const R alpha = a.mode == 2 ? R(0.5) : R(1);
            R *__restrict__ ae = static_cast<R *>(a.acc) + e;
            if (a.mode == 3) {
                // without the prefetch u2 is read where u4 goes: all of the
                // element's u2 values are read before its first write
                R u2v[VC][NP];
#pragma unroll
                for (int n = 0; n < VC; ++n)
#pragma unroll
                    for (int i = 0; i < NP; ++i) u2v[n][i] = at(pacc, (V0 + n) * NP + i);
                R *o3 = static_cast<R *>(a.out) + e;
#pragma unroll
                for (int n = 0; n < VC; ++n)
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        const R kk = sc * rhs[n][i];
                        const int pi = (V0 + n) * NP + i;
                        const R base = at(pc, pi);
                        const R dsum = fma(R(2), c[n][i] - base, u2v[n][i] - base) + kk;
                        ae[pi * SE] = fma(R(1.0 / 3.0), dsum, base);
                        o3[pi * SE] = fma(alpha, kk, base);
                    }
            } else {
#pragma unroll
                for (int n = 0; n < VC; ++n)
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        const int pi = (V0 + n) * NP + i;
                        oe[pi * SE] = fma(alpha, sc * rhs[n][i], at(pc, pi));
                    }
            }
        } else {             // 2: u3 = c + k2/2, acc += k2/3;  3: u4 = c + k3, acc += k3/3
            R *__restrict__ ae = static_cast<R *>(a.acc) + e;
            const R alpha = a.mode == 2 ? R(0.5) : R(1);
#pragma unroll
            for (int n = 0; n < VC; ++n)
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    const R kk = sc * rhs[n][i];
                    const int pi = (V0 + n) * NP + i;
                    oe[pi * SE] = fma(alpha, kk, at(pc, pi));
                    ae[pi * SE] = fma(R(1.0 / 3.0), kk, at(pacc, pi));
                }
        }
    };
    switch (a.mode) {
    case 0:
#pragma unroll
        for (int n = 0; n < VC; ++n)
#pragma unroll
            for (int i = 0; i < NP; ++i) out[((V0 + n) * NP + i) * SE + e] = sc * rhs[n][i];
        break;
    case 1: {   // u2 = c + k1/2, and in the 16-pass form acc = c + k1/6
        if (a.comp) {   // and D = lo + k1/6 (rk_tail)
            if (!pre) rk_tail(IntC<0>{});
            else if (a.prefetch == kTile) rk_tail(IntC<2>{});
            else rk_tail(IntC<1>{});
            break;
        }
        R *__restrict__ ae = static_cast<R *>(a.acc) + e;
        if (a.rk13) {
#pragma unroll
            for (int n = 0; n < VC; ++n)
#pragma unroll
                for (int i = 0; i < NP; ++i)
                    oe[((V0 + n) * NP + i) * SE] = fma(R(0.5), sc * rhs[n][i], c[n][i]);
            break;
        }
#pragma unroll
        for (int n = 0; n < VC; ++n)
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const R kk = sc * rhs[n][i];
                const size_t o = ((V0 + n) * NP + i) * SE;
                oe[o] = fma(R(0.5), kk, c[n][i]);
                ae[o] = fma(R(1.0 / 6.0), kk, c[n][i]);
            }
        break;
    }
    case 2:
    case 3:
    case 4:
        if (!pre) rk_tail(IntC<0>{});
        else if (a.prefetch == kTile) rk_tail(IntC<2>{});
        else rk_tail(IntC<1>{});
        break;
    case 5: {   // out = u + alpha k (RK2 first stage, forward Euler)
        const R alpha = R(a.alpha);
#pragma unroll
        for (int n = 0; n < VC; ++n)
#pragma unroll
            for (int i = 0; i < NP; ++i) out[((V0 + n) * NP + i) * SE + e] = fma(alpha, sc * rhs[n][i], c[n][i]);
        break;
    }
    default: {  // 6: out = c + alpha k (RK2 second stage).  out may be the base
                // state itself: each thread reads and then writes only its own
                // element's values, and no other thread reads them
        const R alpha = R(a.alpha);
        const R *pb = static_cast<const R *>(a.c) + e;
        R *po = static_cast<R *>(a.out) + e;
#pragma unroll
        for (int n = 0; n < VC; ++n)
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const size_t o = ((V0 + n) * NP + i) * SE;
                const R base = pb[o];
                po[o] = fma(alpha, sc * rhs[n][i], base);
            }
        break;
    }
    }
    return pre;
}

#ifndef DGX_PAIRED
#define DGX_PAIRED 1
#endif

// Pairs of values: for FP32, two fused multiply-adds in one instruction
// (sm_100 and later), each lane bitwise fmaf(a, b, c); FP64 (never paired by
// the kernels) has the scalar form so that the code compiles for both.
template <typename T> struct Pair2;
template <> struct Pair2<float> { using type = float2; };
template <> struct Pair2<double> { using type = double2; };
using R2 = typename Pair2<R>::type;
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ double2 fma2(double2 a, double2 b, double2 c) {
    return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ double2 fmul2(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ double2 fadd2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ R2 mk2(R x, R y) { R2 v; v.x = x; v.y = y; return v; }
__device__ __forceinline__ R2 dup2(R t) { return mk2(t, t); }

// The Euler LLF flux of num_flux with the left and right states as the lanes
// of pairs: Ulr[n] = (UL[n], UR[n]).  Both elements of a side call it with the
// same arguments and get the same bits.
__device__ __forceinline__ void num_flux_euler_pair(const R2 (&Ulr)[4], R nx, R ny, int llf, R g, R *Fh) {
    const R2 ir = mk2(rrcp(Ulr[0].x), rrcp(Ulr[0].y));
    const R2 u = fmul2(Ulr[1], ir), v = fmul2(Ulr[2], ir);
    const R2 kin = fma2(Ulr[2], v, fmul2(Ulr[1], u));
    const R2 p = fmul2(dup2(g - R(1)), fma2(dup2(R(-0.5)), kin, Ulr[3]));
    const R2 nx2 = dup2(nx), ny2 = dup2(ny);
    const R2 un = fma2(u, nx2, fmul2(v, ny2));
    R lam = R(0);
    if (llf) {
        const R2 c2 = fmul2(fmul2(dup2(g), p), ir);
        const R ll = fabs(un.x) + rsqrt_(c2.x), lr = fabs(un.y) + rsqrt_(c2.y);
        lam = ll > lr ? ll : lr;
    }
    const R2 f[4] = {fma2(Ulr[1], nx2, fmul2(Ulr[2], ny2)), fma2(Ulr[1], un, fmul2(p, nx2)),
                     fma2(Ulr[2], un, fmul2(p, ny2)), fmul2(fadd2(Ulr[3], p), un)};
#pragma unroll
    for (int n = 0; n < 4; ++n) Fh[n] = R(0.5) * ((f[n].x + f[n].y) + lam * (Ulr[n].x - Ulr[n].y));
}

// FP32 Euler: stage_tile with the four variables held as the pairs
// (rho, rho u) and (rho v, E), so that every basis contraction (traces, point
// values, volume projection, lift) issues one paired FMA per two variables.
// Each lane performs the scalar kernel's fused multiply-adds with the same
// operands in the same order, and the side flux's own-side form is the
// scalar kernel's left/right form negated exactly where the element is the
// right one, so the results are bitwise stage_tile's; the fluxes and the
// epilogue stay scalar.
template <int P, bool BND>
__device__ __forceinline__ bool stage_tile_pair(const StageArgs &a, const int tile, unsigned char *smem_raw,
                                                const unsigned parity) {
    using L = Lay<P>;
    constexpr int NP = L::NP, NQ = L::NQ, NQ1 = L::NQ1;
    constexpr int EQ = DGX_EULER, NV = 4;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem_raw);
    R *s_side = reinterpret_cast<R *>(smem_raw + 16);
    R *s_tr = s_side + side_table_words<P, NV>();
    const int nslot = a.nslot;
    R *s_pre = s_tr + slot_area_words<P, NV>(nslot);

    R dt;
    if (a.mode == 0) {
        dt = R(a.dt);
    } else {
        dt = R(a.scal[0]);
        if (dt == R(0)) return false;   // the run has reached its end time (uniform over the CTA)
    }
    const int E = a.E;
    const int tid = threadIdx.x;
    const int e = tile * kTile + tid;
    const bool live = e < E;
    const size_t SE = static_cast<unsigned>(E);   // zero-extended: plane offsets k*SE are 32x32-bit products
    const R g = a.gammaf, ax = a.axf, ay = a.ayf;
    const int llf = a.flux == DGX_FLUX_LLF;
    const R *__restrict__ u = static_cast<const R *>(a.u);

    for (int t = tid; t < 3 * NP * NQ1; t += kTile) s_side[t] = c_tab[L::SIDE + t];
    const bool pre = issue_prefetch<P, NV>(a, tile, bar, s_pre, tid);

    // plane-major arrays are addressed as (array + element) + plane * E: one
    // wide multiply-add per access
    const R *__restrict__ ue = u + (live ? e : 0);
    R2 c2[2][NP];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int i = 0; i < NP; ++i)
            c2[h][i] = live ? mk2(__ldg(ue + ((2 * h) * NP + i) * SE), __ldg(ue + ((2 * h + 1) * NP + i) * SE))
                            : mk2(R(0), R(0));

    int sw[3];
    R snx[3], sny[3], shl[3];
    {
        const int *__restrict__ nbr = a.nbr;
        const R *__restrict__ fn = static_cast<const R *>(a.fn);
        const int ee = live ? e : 0;
        const int *__restrict__ nbe = nbr + ee;
        const R *__restrict__ fne = fn + ee;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sw[k] = __ldg(nbe + k * SE);
            snx[k] = __ldg(fne + (3 * k + 0) * SE);
            sny[k] = __ldg(fne + (3 * k + 1) * SE);
            shl[k] = __ldg(fne + (3 * k + 2) * SE);
        }
    }

    const int h0 = __ldg(a.halo_off + tile), H = __ldg(a.halo_off + tile + 1) - h0;
    R2 cn2[2][NP];
    int hw = tid < H ? __ldg(a.halo_list + h0 + tid) : -1;
    if (hw >= 0) {
        const int ne = hw >> 2;
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int i = 0; i < NP; ++i)
                cn2[h][i] = mk2(__ldg(u + ne + ((2 * h) * NP + i) * SE), __ldg(u + ne + ((2 * h + 1) * NP + i) * SE));
    }

    // own traces on the three sides (constant-bank side tables)
#if DGX_ROLLED_TRACES
#pragma unroll 1
#else
#pragma unroll
#endif
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < NQ1; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                R2 s2 = mk2(R(0), R(0));
#pragma unroll
                for (int i = 0; i < NP; ++i) s2 = fma2(c2[h][i], dup2(c_tab[L::SIDE + (k * NP + i) * NQ1 + j]), s2);
                s_tr[slot_off<P, NV>(3 * tid + k) + j * NV + 2 * h] = s2.x;
                s_tr[slot_off<P, NV>(3 * tid + k) + j * NV + 2 * h + 1] = s2.y;
            }
    __syncthreads();   // s_side ready

    for (int hh = tid; hh < H; hh += kTile) {
        if (hh != tid) {
            hw = __ldg(a.halo_list + h0 + hh);
            const int ne = hw >> 2;
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int i = 0; i < NP; ++i)
                    cn2[h][i] = mk2(__ldg(u + ne + ((2 * h) * NP + i) * SE),
                                    __ldg(u + ne + ((2 * h + 1) * NP + i) * SE));
        }
        const R *ts = s_side + (hw & 3) * NP * NQ1;
        R2 tr2[NQ1][2];
#pragma unroll
        for (int j = 0; j < NQ1; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) tr2[j][h] = mk2(R(0), R(0));
#pragma unroll
        for (int i = 0; i < NP; ++i)
#pragma unroll
            for (int j = 0; j < NQ1; ++j) {
                const R2 t2 = dup2(ts[i * NQ1 + j]);
#pragma unroll
                for (int h = 0; h < 2; ++h) tr2[j][h] = fma2(cn2[h][i], t2, tr2[j][h]);
            }
#pragma unroll
        for (int j = 0; j < NQ1; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                s_tr[slot_off<P, NV>(3 * kTile + hh) + j * NV + 2 * h] = tr2[j][h].x;
                s_tr[slot_off<P, NV>(3 * kTile + hh) + j * NV + 2 * h + 1] = tr2[j][h].y;
            }
    }

    R2 rhs2[2][NP];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int i = 0; i < NP; ++i) rhs2[h][i] = mk2(R(0), R(0));

    R invJ = R(0), xr = R(0), yr = R(0), xs = R(0), ys = R(0);
    if (live) {
        const R *__restrict__ geo = static_cast<const R *>(a.geo);
        const R *__restrict__ ge = geo + e;
        invJ = __ldg(ge);
        xr = __ldg(ge + SE);
        yr = __ldg(ge + 2 * SE);
        xs = __ldg(ge + 3 * SE);
        ys = __ldg(ge + 4 * SE);
        const R2 ys2 = dup2(ys), xr2 = dup2(xr), nxs2 = dup2(-xs), nyr2 = dup2(-yr);
        // point values of the pair h at the point whose table values t(i) gives
        // metric terms (fx ys - fy xs, fy xr - fx yr) per variable pair
        auto metric = [&](const R2 (&U2)[2], R2 (&hr2)[2], R2 (&hs2)[2]) {
            const R U[4] = {U2[0].x, U2[0].y, U2[1].x, U2[1].y};
            R fx[NV], fy[NV];
            phys_flux<EQ>(U, g, ax, ay, fx, fy);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const R2 fx2 = mk2(fx[2 * h], fx[2 * h + 1]), fy2 = mk2(fy[2 * h], fy[2 * h + 1]);
                hr2[h] = fma2(fx2, ys2, fmul2(fy2, nxs2));
                hs2[h] = fma2(fy2, xr2, fmul2(fx2, nyr2));
            }
        };
        if constexpr (NQ % 2 == 0 && L::PHI % 2 == 0 && (NP * NQ) % 2 == 0) {
            // two points per iteration: the tables of points q, q+1 are adjacent,
            // one 2-value constant load serves both
#pragma unroll 1
            for (int q = 0; q < NQ; q += 2) {
                R2 Ua[2], Ub[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    R2 sa = mk2(R(0), R(0)), sb = mk2(R(0), R(0));
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        const R2 t = *reinterpret_cast<const R2 *>(&c_tab[L::PHI + i * NQ + q]);
                        sa = fma2(c2[h][i], dup2(t.x), sa);
                        sb = fma2(c2[h][i], dup2(t.y), sb);
                    }
                    Ua[h] = sa;
                    Ub[h] = sb;
                }
                R2 hra[2], hsa[2], hrb[2], hsb[2];
                metric(Ua, hra, hsa);
                metric(Ub, hrb, hsb);
                // mode 0 is constant: its weighted gradients are 0
#pragma unroll
                for (int i = 1; i < NP; ++i) {
                    const R2 tx = *reinterpret_cast<const R2 *>(&c_tab[L::GX + i * NQ + q]);
                    const R2 ty = *reinterpret_cast<const R2 *>(&c_tab[L::GY + i * NQ + q]);
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        rhs2[h][i] = fma2(dup2(tx.x), hra[h], fma2(dup2(ty.x), hsa[h], rhs2[h][i]));
                        rhs2[h][i] = fma2(dup2(tx.y), hrb[h], fma2(dup2(ty.y), hsb[h], rhs2[h][i]));
                    }
                }
            }
        } else {
#if DGX_ROLLED_VOLUME
#pragma unroll 1
#else
#pragma unroll
#endif
            for (int q = 0; q < NQ; ++q) {
                R2 U2[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    R2 s2 = mk2(R(0), R(0));
#pragma unroll
                    for (int i = 0; i < NP; ++i) s2 = fma2(c2[h][i], dup2(c_tab[L::PHI + i * NQ + q]), s2);
                    U2[h] = s2;
                }
                R2 hr2[2], hs2[2];
                metric(U2, hr2, hs2);
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int i = 1; i < NP; ++i)   // mode 0: gradients 0
                        rhs2[h][i] = fma2(dup2(c_tab[L::GX + i * NQ + q]), hr2[h],
                                          fma2(dup2(c_tab[L::GY + i * NQ + q]), hs2[h], rhs2[h][i]));
            }
        }
    }
    __syncthreads();   // all traces of the tile and its halo are in shared memory
    if (!live) return pre;

#if DGX_ROLLED_SIDES
#pragma unroll 1
#else
#pragma unroll
#endif
    for (int k = 0; k < 3; ++k) {
        const int word = pick3(sw[0], sw[1], sw[2], k);
        const R nx = pick3(snx[0], snx[1], snx[2], k), ny = pick3(sny[0], sny[1], sny[2], k);
        const R hl = pick3(shl[0], shl[1], shl[2], k);
        const int own = 3 * tid + k;
        const bool bnd = BND && word < 0;
        const int slot = bnd ? own : (word >> 1);
        const int il = bnd ? 1 : (word & 1);
        const R *s_own = s_tr + slot_off<P, NV>(own);
        const R *s_nbr = s_tr + slot_off<P, NV>(slot);
        // The flux from this element's side: (own, neighbour) states with the
        // normal out of this element.  Swapping the states and negating the
        // normal negates every operation of num_flux_euler_pair exactly
        // (products and sums of negated operands, |un|, the max of the two
        // wave speeds), so this is bitwise the side's flux (left, right, left
        // normal) for the left element and its negation for the right one, and
        // -len/2 times its lift is bitwise the left/right form's contribution.
        const R sgn = il ? R(1) : R(-1);
        const R nxo = sgn * nx, nyo = sgn * ny;
        R2 Fh2[NQ1][2];
#pragma unroll
        for (int j = 0; j < NQ1; ++j) {
            R UO[NV], UN[NV], Fh[NV];
            R2 Ulr[NV];
#pragma unroll
            for (int n = 0; n < NV; ++n) {
                UO[n] = s_own[j * NV + n];
                UN[n] = s_nbr[(NQ1 - 1 - j) * NV + n];
            }
            if constexpr (BND) {
                if (bnd) boundary_ghost<P, EQ>(a, word, k, j, e, UO, nx, ny, UN);
            }
#pragma unroll
            for (int n = 0; n < NV; ++n) Ulr[n] = mk2(UO[n], UN[n]);
            num_flux_euler_pair(Ulr, nxo, nyo, llf, g, Fh);
            Fh2[j][0] = mk2(Fh[0], Fh[1]);
            Fh2[j][1] = mk2(Fh[2], Fh[3]);
        }
        // the fluxes scaled by -len/2 first, then lifted straight into the
        // modes (each element scales its own, exactly negated, flux: the two
        // elements of a side still get contributions of equal magnitude)
        const R2 sg2 = dup2(-hl);
#pragma unroll
        for (int j = 0; j < NQ1; ++j)
#pragma unroll
            for (int h = 0; h < 2; ++h) Fh2[j][h] = fmul2(sg2, Fh2[j][h]);
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int j = 0; j < NQ1; ++j)
                    rhs2[h][i] = fma2(dup2(c_tab[L::LIFT + (k * NP + i) * NQ1 + j]), Fh2[j][h], rhs2[h][i]);
    }

    R rhs[NV][NP], c[NV][NP];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            rhs[2 * h][i] = rhs2[h][i].x;
            rhs[2 * h + 1][i] = rhs2[h][i].y;
            c[2 * h][i] = c2[h][i].x;
            c[2 * h + 1][i] = c2[h][i].y;
        }
    return stage_epilogue<P, EQ>(a, rhs, c, dt, invJ, e, SE, pre, s_pre, bar, parity, tid);
}

#ifdef DGX_REAL_F32
// FP32 advection: stage_tile with the modes held in pairs (2m, 2m+1) and the
// transposed tables, so that every basis contraction issues one paired FMA per
// two modes.  Sums over modes (traces, point values) run as two partial sums,
// even and odd modes, added at the end; sums into a mode (volume projection,
// lift) keep the scalar kernel's operands and order.  An odd mode count is
// padded with a zero mode.
template <int P, bool BND>
__device__ __forceinline__ bool stage_tile_adv_pair(const StageArgs &a, const int tile, unsigned char *smem_raw,
                                                    const unsigned parity) {
    using L = Lay<P>;
    using T = LayT<P>;
    constexpr int NP = L::NP, NQ = L::NQ, NQ1 = L::NQ1, NPP = T::NPP, NH = NPP / 2;
    constexpr int EQ = DGX_ADVECTION, NV = 1;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem_raw);
    float *s_side = reinterpret_cast<float *>(smem_raw + 16);   // [side][j][i], rows of NPP
    float *s_tr = s_side + side_table_words<P, NV>();
    const int nslot = a.nslot;
    float *s_pre = s_tr + slot_area_words<P, NV>(nslot);

    float dt;
    if (a.mode == 0) {
        dt = float(a.dt);
    } else {
        dt = float(a.scal[0]);
        if (dt == 0.0f) return false;   // the run has reached its end time (uniform over the CTA)
    }
    const int E = a.E;
    const int tid = threadIdx.x;
    const int e = tile * kTile + tid;
    const bool live = e < E;
    const size_t SE = static_cast<unsigned>(E);   // zero-extended: plane offsets k*SE are 32x32-bit products
    const float ax = a.axf, ay = a.ayf;
    const int llf = a.flux == DGX_FLUX_LLF;
    const float *__restrict__ u = static_cast<const float *>(a.u);
    auto t2 = [](int off) { return *reinterpret_cast<const float2 *>(&c_tabT[off]); };

    for (int t = tid; t < 3 * NQ1 * NPP; t += kTile) s_side[t] = c_tabT[T::SIDE + t];
    const bool pre = issue_prefetch<P, NV>(a, tile, bar, s_pre, tid);

    const float *__restrict__ ue = u + (live ? e : 0);   // (array + element) + plane * E
    float2 c2[NH];
#pragma unroll
    for (int m = 0; m < NH; ++m) {
        const float lo = live ? __ldg(ue + (2 * m) * SE) : 0.0f;
        const float hi = (live && 2 * m + 1 < NP) ? __ldg(ue + (2 * m + 1) * SE) : 0.0f;
        c2[m] = make_float2(lo, hi);
    }

    int sw[3];
    float snx[3], sny[3], shl[3];
    {
        const int *__restrict__ nbr = a.nbr;
        const float *__restrict__ fn = static_cast<const float *>(a.fn);
        const int ee = live ? e : 0;
        const int *__restrict__ nbe = nbr + ee;
        const float *__restrict__ fne = fn + ee;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sw[k] = __ldg(nbe + k * SE);
            snx[k] = __ldg(fne + (3 * k + 0) * SE);
            sny[k] = __ldg(fne + (3 * k + 1) * SE);
            shl[k] = __ldg(fne + (3 * k + 2) * SE);
        }
    }

    const int h0 = __ldg(a.halo_off + tile), H = __ldg(a.halo_off + tile + 1) - h0;
    float2 cn2[NH];
    int hw = tid < H ? __ldg(a.halo_list + h0 + tid) : -1;
    auto gather = [&](int ne) {
#pragma unroll
        for (int m = 0; m < NH; ++m)
            cn2[m] = make_float2(__ldg(u + ne + (2 * m) * SE), 2 * m + 1 < NP ? __ldg(u + ne + (2 * m + 1) * SE) : 0.0f);
    };
    if (hw >= 0) gather(hw >> 2);

    // own traces on the three sides
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < NQ1; ++j) {
            float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int m = 0; m < NH; ++m) acc = fma2(c2[m], t2(T::SIDE + (k * NQ1 + j) * NPP + 2 * m), acc);
            s_tr[slot_off<P, NV>(3 * tid + k) + j] = acc.x + acc.y;
        }
    __syncthreads();   // s_side ready

    for (int hh = tid; hh < H; hh += kTile) {
        if (hh != tid) {
            hw = __ldg(a.halo_list + h0 + hh);
            gather(hw >> 2);
        }
        const float *ts = s_side + (hw & 3) * NQ1 * NPP;
#pragma unroll
        for (int j = 0; j < NQ1; ++j) {
            float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int m = 0; m < NH; ++m)
                acc = fma2(cn2[m], *reinterpret_cast<const float2 *>(ts + j * NPP + 2 * m), acc);
            s_tr[slot_off<P, NV>(3 * kTile + hh) + j] = acc.x + acc.y;
        }
    }

    float2 rhs2[NH];
#pragma unroll
    for (int m = 0; m < NH; ++m) rhs2[m] = make_float2(0.0f, 0.0f);

    float invJ = 0.0f;
    if (live) {
        const float *__restrict__ geo = static_cast<const float *>(a.geo);
        invJ = __ldg(geo + e);
        const float *__restrict__ ge = geo + e;
        const float xr = __ldg(ge + SE), yr = __ldg(ge + 2 * SE);
        const float xs = __ldg(ge + 3 * SE), ys = __ldg(ge + 4 * SE);
        // p = 4 unrolled (measured 8 % faster), the lower orders rolled (p = 3
        // unrolled was 10 % slower)
#pragma unroll(P == 4 ? NQ : 1)
        for (int q = 0; q < NQ; ++q) {
            float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int m = 0; m < NH; ++m) acc = fma2(c2[m], t2(T::PHI + q * NPP + 2 * m), acc);
            const float U[1] = {acc.x + acc.y};
            float fx[1], fy[1];
            phys_flux<EQ>(U, a.gammaf, ax, ay, fx, fy);
            const float2 hr = dup2(fx[0] * ys - fy[0] * xs), hs = dup2(fy[0] * xr - fx[0] * yr);
#pragma unroll
            for (int m = 0; m < NH; ++m)
                rhs2[m] = fma2(t2(T::GX + q * NPP + 2 * m), hr, fma2(t2(T::GY + q * NPP + 2 * m), hs, rhs2[m]));
        }
    }
    __syncthreads();   // all traces of the tile and its halo are in shared memory
    if (!live) return pre;

#if DGX_ROLLED_SIDES
#pragma unroll 1
#else
#pragma unroll
#endif
    for (int k = 0; k < 3; ++k) {
        const int word = pick3(sw[0], sw[1], sw[2], k);
        const float nx = pick3(snx[0], snx[1], snx[2], k), ny = pick3(sny[0], sny[1], sny[2], k);
        const float hl = pick3(shl[0], shl[1], shl[2], k);
        const int own = 3 * tid + k;
        const bool bnd = BND && word < 0;
        const int slot = bnd ? own : (word >> 1);
        const int il = bnd ? 1 : (word & 1);
        const float *s_own = s_tr + slot_off<P, NV>(own);
        const float *s_nbr = s_tr + slot_off<P, NV>(slot);
        // the flux from this element's side, (own, neighbour) with the normal
        // out of this element: bitwise the left/right form for the left
        // element and its negation for the right one (as in stage_tile_pair)
        const float sgn = il ? 1.0f : -1.0f;
        const float nxo = sgn * nx, nyo = sgn * ny;
        float2 Fh2[NQ1];
#pragma unroll
        for (int j = 0; j < NQ1; ++j) {
            float UO[1] = {s_own[j]}, UN[1] = {s_nbr[NQ1 - 1 - j]};
            if constexpr (BND) {
                if (bnd) boundary_ghost<P, EQ>(a, word, k, j, e, UO, nx, ny, UN);
            }
            float Fh[1];
            num_flux<EQ>(UO, UN, nxo, nyo, llf, a.gammaf, ax, ay, Fh);
            Fh2[j] = dup2(Fh[0]);
        }
        const float2 sg2 = dup2(-hl);
#pragma unroll
        for (int m = 0; m < NH; ++m) {
            float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int j = 0; j < NQ1; ++j) acc = fma2(t2(T::LIFT + (k * NQ1 + j) * NPP + 2 * m), Fh2[j], acc);
            rhs2[m] = fma2(sg2, acc, rhs2[m]);
        }
    }

    float rhs[1][NP], c[1][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        rhs[0][i] = (i & 1) ? rhs2[i / 2].y : rhs2[i / 2].x;
        c[0][i] = (i & 1) ? c2[i / 2].y : c2[i / 2].x;
    }
    return stage_epilogue<P, EQ>(a, rhs, c, dt, invJ, e, SE, pre, s_pre, bar, parity, tid);
}
#endif

template <int P, int EQ, bool BND>
__device__ __forceinline__ bool stage_tile(const StageArgs &a, const int tile, unsigned char *smem_raw,
                                           const unsigned parity) {
    if constexpr (DGX_PAIRED && sizeof(R) == 4 && EQ == DGX_EULER) {
        return stage_tile_pair<P, BND>(a, tile, smem_raw, parity);
    }
#ifdef DGX_REAL_F32
    if constexpr (DGX_PAIRED && EQ == DGX_ADVECTION) {
        return stage_tile_adv_pair<P, BND>(a, tile, smem_raw, parity);
    }
#endif
    using L = Lay<P>;
    constexpr int NP = L::NP, NQ = L::NQ, NQ1 = L::NQ1;
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem_raw);
    R *s_side = reinterpret_cast<R *>(smem_raw + 16);
    R *s_tr = s_side + side_table_words<P, NV>();
    const int nslot = a.nslot;
    // epilogue operands (base state, accumulator) of the tile, prefetched by the
    // TMA engine while the element work runs; 16-byte aligned (the side tables
    // and the slot area are multiples of 4 words)
    R *s_pre = s_tr + slot_area_words<P, NV>(nslot);

    R dt;
    if (a.mode == 0) {
        dt = R(a.dt);
    } else {
        dt = R(a.scal[0]);
        if (dt == R(0)) return false;   // the run has reached its end time (uniform over the CTA)
    }
    const int E = a.E;
    const int tid = threadIdx.x;
    const int e = tile * kTile + tid;
    const bool live = e < E;
    const size_t SE = static_cast<unsigned>(E);   // zero-extended: plane offsets k*SE are 32x32-bit products
    // physics constants in the kernel's precision (FP32 copies avoid FP64 conversions)
    const R g = sizeof(R) == 4 ? R(a.gammaf) : R(a.gamma);
    const R ax = sizeof(R) == 4 ? R(a.axf) : R(a.ax);
    const R ay = sizeof(R) == 4 ? R(a.ayf) : R(a.ay);
    const int llf = a.flux == DGX_FLUX_LLF;
    const R *__restrict__ u = static_cast<const R *>(a.u);

    for (int t = tid; t < 3 * NP * NQ1; t += kTile) s_side[t] = c_tab[L::SIDE + t];

    // modes 2..4 read the base state (2, 3) and the accumulator (2, 3, 4) at the
    // end: start their copies now
    const bool pre = issue_prefetch<P, NV>(a, tile, bar, s_pre, tid);

    // own coefficients (coalesced: 32 consecutive elements per warp and (n,i))
    R c[NV][NP];
#pragma unroll
    for (int n = 0; n < NV; ++n)
#pragma unroll
        for (int i = 0; i < NP; ++i) c[n][i] = live ? __ldg(u + (n * NP + i) * SE + e) : R(0);

    // side data of the three sides
    int sw[3];
    R snx[3], sny[3], shl[3];
    {
        const int *__restrict__ nbr = a.nbr;
        const R *__restrict__ fn = static_cast<const R *>(a.fn);
        const int ee = live ? e : 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sw[k] = __ldg(nbr + k * SE + ee);
            snx[k] = __ldg(fn + (3 * k + 0) * SE + ee);
            sny[k] = __ldg(fn + (3 * k + 1) * SE + ee);
            shl[k] = __ldg(fn + (3 * k + 2) * SE + ee);
        }
    }

    // first halo entry of this thread: issue its gathers before any compute
    const int h0 = __ldg(a.halo_off + tile), H = __ldg(a.halo_off + tile + 1) - h0;
    R cn[NV][NP];
    int hw = tid < H ? __ldg(a.halo_list + h0 + tid) : -1;
    if (hw >= 0) {
        const int ne = hw >> 2;
#pragma unroll
        for (int n = 0; n < NV; ++n)
#pragma unroll
            for (int i = 0; i < NP; ++i) cn[n][i] = __ldg(u + (n * NP + i) * SE + ne);
    }

    // own traces on the three sides (constant-bank side tables)
#if DGX_ROLLED_TRACES
#pragma unroll 1
#else
#pragma unroll
#endif
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int j = 0; j < NQ1; ++j)
#pragma unroll
            for (int n = 0; n < NV; ++n) {
                R s = R(0);
#pragma unroll
                for (int i = 0; i < NP; ++i) s = fma(c[n][i], c_tab[L::SIDE + (k * NP + i) * NQ1 + j], s);
                s_tr[slot_off<P, NV>(3 * tid + k) + j * NV + n] = s;
            }
    __syncthreads();   // s_side ready

    // halo traces: the tile's neighbours outside the tile, on their own side
    // and in their own point order (a runtime side: tables from shared memory)
    for (int h = tid; h < H; h += kTile) {
        if (h != tid) {
            hw = __ldg(a.halo_list + h0 + h);
            const int ne = hw >> 2;
#pragma unroll
            for (int n = 0; n < NV; ++n)
#pragma unroll
                for (int i = 0; i < NP; ++i) cn[n][i] = __ldg(u + (n * NP + i) * SE + ne);
        }
        const R *ts = s_side + (hw & 3) * NP * NQ1;
        R tr[NQ1][NV];
#pragma unroll
        for (int j = 0; j < NQ1; ++j)
#pragma unroll
            for (int n = 0; n < NV; ++n) tr[j][n] = R(0);
#pragma unroll
        for (int i = 0; i < NP; ++i)
#pragma unroll
            for (int j = 0; j < NQ1; ++j) {
                const R t = ts[i * NQ1 + j];
#pragma unroll
                for (int n = 0; n < NV; ++n) tr[j][n] = fma(cn[n][i], t, tr[j][n]);
            }
#pragma unroll
        for (int j = 0; j < NQ1; ++j)
#pragma unroll
            for (int n = 0; n < NV; ++n) s_tr[slot_off<P, NV>(3 * kTile + h) + j * NV + n] = tr[j][n];
    }

    R rhs[NV][NP];
#pragma unroll
    for (int n = 0; n < NV; ++n)
#pragma unroll
        for (int i = 0; i < NP; ++i) rhs[n][i] = R(0);

    R invJ = R(0), xr = R(0), yr = R(0), xs = R(0), ys = R(0);
    if (live) {
        const R *__restrict__ geo = static_cast<const R *>(a.geo);
        invJ = __ldg(geo + e);
        xr = __ldg(geo + SE + e);
        yr = __ldg(geo + 2 * SE + e);
        xs = __ldg(geo + 3 * SE + e);
        ys = __ldg(geo + 4 * SE + e);
        // ---- volume integral ----------------------------------------------------
#if DGX_ROLLED_VOLUME
#pragma unroll 1
#else
#pragma unroll
#endif
        for (int q = 0; q < NQ; ++q) {
            R U[NV], fx[NV], fy[NV];
#pragma unroll
            for (int n = 0; n < NV; ++n) {
                R s = R(0);
#pragma unroll
                for (int i = 0; i < NP; ++i) s = fma(c[n][i], c_tab[L::PHI + i * NQ + q], s);
                U[n] = s;
            }
            phys_flux<EQ>(U, g, ax, ay, fx, fy);
#pragma unroll
            for (int n = 0; n < NV; ++n) {
                const R hr = fx[n] * ys - fy[n] * xs;
                const R hs = fy[n] * xr - fx[n] * yr;
#pragma unroll
                for (int i = 1; i < NP; ++i)   // mode 0 is constant: its weighted gradients are 0
                    rhs[n][i] = fma(c_tab[L::GX + i * NQ + q], hr, fma(c_tab[L::GY + i * NQ + q], hs, rhs[n][i]));
            }
        }
    }
    __syncthreads();   // all traces of the tile and its halo are in shared memory
    if (!live) {
        // this thread has no element; the CTA's copies are waited for by the others
        return pre;
    }

    // ---- the three sides --------------------------------------------------------
#if DGX_ROLLED_SIDES
#pragma unroll 1
#else
#pragma unroll
#endif
    for (int k = 0; k < 3; ++k) {
        const int word = pick3(sw[0], sw[1], sw[2], k);
        const R nx = pick3(snx[0], snx[1], snx[2], k), ny = pick3(sny[0], sny[1], sny[2], k);
        const R hl = pick3(shl[0], shl[1], shl[2], k);
        const int own = 3 * tid + k;
        const bool bnd = BND && word < 0;       // boundary side: this element is its left element
        const int slot = bnd ? own : (word >> 1);
        const int il = bnd ? 1 : (word & 1);
        const R *s_own = s_tr + slot_off<P, NV>(own);
        const R *s_nbr = s_tr + slot_off<P, NV>(slot);
        R Fh[NQ1][NV];
#pragma unroll
        for (int j = 0; j < NQ1; ++j) {
            R UO[NV], UN[NV], UL[NV], UR[NV];
#pragma unroll
            for (int n = 0; n < NV; ++n) {
                UO[n] = s_own[j * NV + n];
                UN[n] = s_nbr[(NQ1 - 1 - j) * NV + n];
            }
            if constexpr (BND) {
                if (bnd) boundary_ghost<P, EQ>(a, word, k, j, e, UO, nx, ny, UN);
            }
#pragma unroll
            for (int n = 0; n < NV; ++n) {
                UL[n] = il ? UO[n] : UN[n];
                UR[n] = il ? UN[n] : UO[n];
            }
            num_flux<EQ>(UL, UR, nx, ny, llf, g, ax, ay, Fh[j]);
        }
        const R sg = il ? -hl : hl;
#pragma unroll
        for (int n = 0; n < NV; ++n)
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                R s = R(0);
#pragma unroll
                for (int j = 0; j < NQ1; ++j) s = fma(c_tab[L::LIFT + (k * NP + i) * NQ1 + j], Fh[j][n], s);
                rhs[n][i] = fma(sg, s, rhs[n][i]);
            }
    }

    return stage_epilogue<P, EQ>(a, rhs, c, dt, invJ, e, SE, pre, s_pre, bar, parity, tid);
}

#ifndef DGX_STAGE_NO_LAUNCHERS   // (a translation unit that needs only the device functions and tables)
#ifndef DGX_MIN_CTAS_P3
#define DGX_MIN_CTAS_P3 3
#endif

template <int P>
constexpr int min_ctas() { return P <= 3 ? DGX_MIN_CTAS_P3 : 2; }

// Plain path: one CTA per tile of one solve.
template <int P, int EQ, bool BND>
__global__ void __launch_bounds__(kTile, min_ctas<P>()) stage_kernel(const StageArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (threadIdx.x == 0) mbar_init(reinterpret_cast<unsigned long long *>(smem_raw), 1);
    __syncthreads();
    stage_tile<P, EQ, BND>(a, blockIdx.x, smem_raw, 0u);
}

// Batched path: the CTAs of one launch walk a work list of (solve, tile) items
// of many solves of the same order and equation (grid-stride, so the launch can
// be persistent); every solve keeps its own state, geometry and dt.
template <int P, int EQ, bool BND>
__global__ void __launch_bounds__(kTile, min_ctas<P>()) batch_stage_kernel(const BatchStageArgs b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (threadIdx.x == 0) mbar_init(reinterpret_cast<unsigned long long *>(smem_raw), 1);
    __syncthreads();
    // the item's solve arguments live in shared memory, not registers
    __shared__ StageArgs s_args;
    unsigned phase = 0;
    for (int it = blockIdx.x; it < b.n_items; it += gridDim.x) {
        const int2 w = b.items[it];
        constexpr int kWords = sizeof(StageArgs) / sizeof(int);
        static_assert(sizeof(StageArgs) % sizeof(int) == 0, "StageArgs is copied word by word");
        if (threadIdx.x < kWords)
            reinterpret_cast<int *>(&s_args)[threadIdx.x] =
                reinterpret_cast<const int *>(b.args + w.x)[threadIdx.x];
        __syncthreads();
        if (stage_tile<P, EQ, BND>(s_args, w.y, smem_raw, phase & 1u)) ++phase;
        __syncthreads();   // shared memory is reused by the next item
    }
}

template <int P, int EQ, bool BND>
static int launch_one(const StageArgs &a_in, cudaStream_t st) {
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    StageArgs a = a_in;
    if (a.prefetch && stage_smem_bytes<P, NV>(a.nslot, a.prefetch) > 200 * 1024) a.prefetch = 0;
    const size_t smem = stage_smem_bytes<P, NV>(a.nslot, a.prefetch);
    static size_t configured = 0;   // dynamic shared memory opted in so far
    if (smem > 48 * 1024 && smem > configured) {
        DGX_TRY_CUDA(cudaFuncSetAttribute(stage_kernel<P, EQ, BND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(smem)));
        // all of the unified L1 / shared storage as shared memory, so that
        // several CTAs with large tiles fit on an SM
        DGX_TRY_CUDA(cudaFuncSetAttribute(stage_kernel<P, EQ, BND>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                          100));
        configured = smem;
    }
    const int grid = (a.E + kTile - 1) / kTile;
    if (grid > 0) stage_kernel<P, EQ, BND><<<grid, kTile, smem, st>>>(a);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

// Batched path, one item per CTA (the flat grid): no loop to keep live state across.
template <int P, int EQ, bool BND>
__global__ void __launch_bounds__(kTile, min_ctas<P>()) batch_stage_kernel_flat(const BatchStageArgs b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ StageArgs s_args;
    constexpr int kWords = sizeof(StageArgs) / sizeof(int);
    const int2 w = b.items[blockIdx.x];
    if (threadIdx.x == 0) mbar_init(reinterpret_cast<unsigned long long *>(smem_raw), 1);
    if (threadIdx.x < kWords)
        reinterpret_cast<int *>(&s_args)[threadIdx.x] = reinterpret_cast<const int *>(b.args + w.x)[threadIdx.x];
    __syncthreads();
    stage_tile<P, EQ, BND>(s_args, w.y, smem_raw, 0u);
}

template <int P, int EQ, bool BND>
static int launch_batch_one(const BatchStageArgs &b, cudaStream_t st) {
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    const size_t smem = stage_smem_bytes<P, NV>(b.nslot, b.prefetch);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        DGX_TRY_CUDA(cudaFuncSetAttribute(batch_stage_kernel<P, EQ, BND>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        DGX_TRY_CUDA(cudaFuncSetAttribute(batch_stage_kernel_flat<P, EQ, BND>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        DGX_TRY_CUDA(cudaFuncSetAttribute(batch_stage_kernel<P, EQ, BND>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        DGX_TRY_CUDA(cudaFuncSetAttribute(batch_stage_kernel_flat<P, EQ, BND>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        configured = smem;
    }
    if (b.grid > 0 && b.grid >= b.n_items) batch_stage_kernel_flat<P, EQ, BND><<<b.n_items, kTile, smem, st>>>(b);
    else if (b.grid > 0) batch_stage_kernel<P, EQ, BND><<<b.grid, kTile, smem, st>>>(b);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

// bytes of dynamic shared memory one CTA of the batched kernel needs
template <int EQ>
static size_t batch_smem_impl(int order, int nslot, int prefetch) {
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    switch (order) {
    case 0: return stage_smem_bytes<0, NV>(nslot, prefetch);
    case 1: return stage_smem_bytes<1, NV>(nslot, prefetch);
    case 2: return stage_smem_bytes<2, NV>(nslot, prefetch);
    case 3: return stage_smem_bytes<3, NV>(nslot, prefetch);
    case 4: return stage_smem_bytes<4, NV>(nslot, prefetch);
    default: return stage_smem_bytes<5, NV>(nslot, prefetch);
    }
}

template <int EQ>
static int launch_batch_order(int order, const BatchStageArgs &b, cudaStream_t st) {
    switch (order) {
    case 0: return launch_batch_one<0, EQ, kStageBnd>(b, st);
    case 1: return launch_batch_one<1, EQ, kStageBnd>(b, st);
    case 2: return launch_batch_one<2, EQ, kStageBnd>(b, st);
    case 3: return launch_batch_one<3, EQ, kStageBnd>(b, st);
    case 4: return launch_batch_one<4, EQ, kStageBnd>(b, st);
    case 5: return launch_batch_one<5, EQ, kStageBnd>(b, st);
    default: set_error("unsupported order %d", order); return DGX_ERR_UNSUPPORTED;
    }
}

// Batched path with the solves' arguments as a kernel parameter: CTA b finds
// its solve by a binary search of the parameter's tile offsets (uniform over
// the CTA, served by the constant cache) and runs its tile with the solve's
// arguments read in place from the parameter space.
template <int P, int EQ, bool BND>
__global__ void __launch_bounds__(kTile, min_ctas<P>())
    batch_stage_kernel_param(const __grid_constant__ BatchParamArgs p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = static_cast<int>(blockIdx.x);
    int lo = 0, hi = p.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (p.tile_start[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const int t0 = p.tile_start[lo];
    const StageArgs &a = p.args[lo];
    const int tile = b - t0;
    // a work item outside its solve's tiles (a malformed launch) is skipped
    // and reported instead of read out of bounds; uniform over the CTA
    if (tile < 0 || tile * kTile >= a.E) {
        if (threadIdx.x == 0) atomicOr(a.status, kStatusBadItem);
        return;
    }
    if (threadIdx.x == 0) mbar_init(reinterpret_cast<unsigned long long *>(smem_raw), 1);
    __syncthreads();
    stage_tile<P, EQ, BND>(a, tile, smem_raw, 0u);
}

template <int P, int EQ, bool BND>
static int launch_batch_param_one(const BatchParamArgs &p, int grid, cudaStream_t st) {
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    const size_t smem = stage_smem_bytes<P, NV>(p.nslot, p.prefetch);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        DGX_TRY_CUDA(cudaFuncSetAttribute(batch_stage_kernel_param<P, EQ, BND>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
        DGX_TRY_CUDA(cudaFuncSetAttribute(batch_stage_kernel_param<P, EQ, BND>,
                                          cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        configured = smem;
    }
    if (grid > 0) batch_stage_kernel_param<P, EQ, BND><<<grid, kTile, smem, st>>>(p);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

template <int EQ>
static int launch_batch_param_order(int order, const BatchParamArgs &p, int grid, cudaStream_t st) {
    switch (order) {
    case 0: return launch_batch_param_one<0, EQ, kStageBnd>(p, grid, st);
    case 1: return launch_batch_param_one<1, EQ, kStageBnd>(p, grid, st);
    case 2: return launch_batch_param_one<2, EQ, kStageBnd>(p, grid, st);
    case 3: return launch_batch_param_one<3, EQ, kStageBnd>(p, grid, st);
    case 4: return launch_batch_param_one<4, EQ, kStageBnd>(p, grid, st);
    case 5: return launch_batch_param_one<5, EQ, kStageBnd>(p, grid, st);
    default: set_error("unsupported order %d", order); return DGX_ERR_UNSUPPORTED;
    }
}

static int launch_batch_param_impl(int order, int equation, const BatchParamArgs &p, int grid, cudaStream_t st) {
    return equation == DGX_EULER ? launch_batch_param_order<DGX_EULER>(order, p, grid, st)
                                 : launch_batch_param_order<DGX_ADVECTION>(order, p, grid, st);
}

template <int EQ>
static int launch_order(int order, const StageArgs &a, cudaStream_t st) {
    switch (order) {
    case 0: return launch_one<0, EQ, kStageBnd>(a, st);
    case 1: return launch_one<1, EQ, kStageBnd>(a, st);
    case 2: return launch_one<2, EQ, kStageBnd>(a, st);
    case 3: return launch_one<3, EQ, kStageBnd>(a, st);
    case 4: return launch_one<4, EQ, kStageBnd>(a, st);
    case 5: return launch_one<5, EQ, kStageBnd>(a, st);
    default: set_error("unsupported order %d", order); return DGX_ERR_UNSUPPORTED;
    }
}

static int launch_stage_impl(int order, int equation, const StageArgs &a, cudaStream_t st) {
    return equation == DGX_EULER ? launch_order<DGX_EULER>(order, a, st)
                                 : launch_order<DGX_ADVECTION>(order, a, st);
}

#endif   // DGX_STAGE_NO_LAUNCHERS

// Fill this translation unit's constant tables from the FP64 host tables.
static int upload_tables_impl() {
    static R host[kTableTotal];
    for (int p = 0; p <= kMaxOrder; ++p) {
        const Tables &T = tables(p);
        const int np = T.np, nq = T.nq, nq1 = T.nq1;
        R *b = host + table_offset(p);
        for (int i = 0; i < np * nq; ++i) {
            b[i] = static_cast<R>(T.phi[i]);
            b[np * nq + i] = static_cast<R>(T.gx[i]);
            b[2 * np * nq + i] = static_cast<R>(T.gy[i]);
        }
        R *sd = b + 3 * np * nq, *lf = sd + 3 * np * nq1, *w1 = lf + 3 * np * nq1;
        for (int sdi = 0; sdi < 3; ++sdi)
            for (int i = 0; i < np; ++i)
                for (int j = 0; j < nq1; ++j) {
                    const int o = (sdi * np + i) * nq1 + j;
                    sd[o] = static_cast<R>(T.side[o]);
                    lf[o] = static_cast<R>(T.w1[j] * T.side[o]);
                }
        for (int j = 0; j < nq1; ++j) w1[j] = static_cast<R>(T.w1[j]);
        // side points in the reference orientation (side 0: V1->V2, 1: V2->V3, 2: V3->V1)
        R *srs = w1 + nq1;
        for (int j = 0; j < nq1; ++j) {
            const double g = T.s1[j], gr = T.s1[nq1 - 1 - j];
            const double rs[3][2] = {{0.5 + 0.5 * g, 0.0}, {(1.0 - g) / 2.0, (1.0 + g) / 2.0}, {0.0, 0.5 + 0.5 * gr}};
            for (int sd = 0; sd < 3; ++sd) {
                srs[(sd * nq1 + j) * 2] = static_cast<R>(rs[sd][0]);
                srs[(sd * nq1 + j) * 2 + 1] = static_cast<R>(rs[sd][1]);
            }
        }
    }
    DGX_TRY_CUDA(cudaMemcpyToSymbol(c_tab, host, sizeof(host)));
#ifdef DGX_REAL_F32
    static float ht[kTabTTotal];
    for (int p = 0; p <= kMaxOrder; ++p) {
        const Tables &T = tables(p);
        const int np = T.np, nq = T.nq, nq1 = T.nq1, npp = np_even(p);
        float *b = ht + tabt_offset(p);
        for (int q = 0; q < nq; ++q)
            for (int i = 0; i < npp; ++i) {
                const bool m = i < np;
                b[q * npp + i] = m ? static_cast<float>(T.phi[i * nq + q]) : 0.0f;
                b[(nq + q) * npp + i] = m ? static_cast<float>(T.gx[i * nq + q]) : 0.0f;
                b[(2 * nq + q) * npp + i] = m ? static_cast<float>(T.gy[i * nq + q]) : 0.0f;
            }
        float *sd = b + 3 * nq * npp, *lf = sd + 3 * nq1 * npp;
        for (int k = 0; k < 3; ++k)
            for (int j = 0; j < nq1; ++j)
                for (int i = 0; i < npp; ++i) {
                    const int o = (k * np + i) * nq1 + j;
                    const bool m = i < np;
                    sd[(k * nq1 + j) * npp + i] = m ? static_cast<float>(T.side[o]) : 0.0f;
                    lf[(k * nq1 + j) * npp + i] = m ? static_cast<float>(T.w1[j] * T.side[o]) : 0.0f;
                }
    }
    DGX_TRY_CUDA(cudaMemcpyToSymbol(c_tabT, ht, sizeof(ht)));
#endif
    return DGX_OK;
}

}  // namespace dgx
