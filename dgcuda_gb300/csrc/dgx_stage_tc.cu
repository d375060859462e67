// dgx_stage_tc.cu -- the fused RK-stage kernel with its basis contractions on
// the tensor cores (DGX_FP32_BF16X3): FP32 state and flux arithmetic, the
// contractions as tcgen05 MMAs of BF16 hi/lo operands with FP32 accumulation.
//
// Same contract and data flow as the FP32 kernel (dgx_stage.cuh): one CTA per
// tile of 128 elements, one thread per element, traces exchanged through
// shared-memory slots, the flux of a side evaluated by both of its elements,
// the RK combination fused.  Per tile:
//   1. each thread writes its element's coefficients of modes 1..np-1, split
//      into BF16 (hi, lo), to its tensor-memory lane (operand A_U);
//   2. one thread issues the MMAs D_U = A_U B_U: the element's values at the
//      volume points and at its three sides' Gauss points; meanwhile the
//      threads evaluate the halo traces (FP32, as the FP32 kernel);
//   3. each thread adds the mean mode c_0 phi_0 exactly in FP32, puts its own
//      traces in shared memory, and after one barrier evaluates the volume
//      fluxes and the three sides' numerical fluxes; it writes, minus the
//      flux of its cell-average state (the reference state), the geometry-
//      weighted volume fluxes and the lifted side fluxes to its lane (A');
//   4. the MMAs D_P = A' B_P project them onto the basis; meanwhile the
//      threads add the reference state's part exactly in FP32 (its projection
//      is a constant times the column sums of the tables);
//   5. the RK combination (stage_epilogue, shared with the FP32 kernel).
// The BF16x3 terms carry only the deviations from the mean mode and from the
// reference state, so their 2^-17 relative error applies to small numbers.
// Tensor memory: up to 256 columns per CTA (two CTAs per SM).  Every wait is
// bounded; on a timeout the CTA reports, waits once more, frees its tensor
// memory and skips its writes.
#define DGX_REAL float
#define DGX_STAGE_BND 0
#define DGX_STAGE_NO_LAUNCHERS
#include "dgx_stage.cuh"
#include "dgx_tc.cuh"
#include "dgx_tc_layout.h"

namespace dgx {
namespace {

// tensor-memory columns of one CTA
template <int P, int NV>
struct TcCols {
    static constexpr TcDims D = tc_dims(P);
    static constexpr int AUW = D.ku / 2;    // A_U columns per variable
    static constexpr int APW = D.kpv / 2;   // A' columns per variable
    static constexpr int AU = 0;            // phase 1-3
    static constexpr int DU = NV * AUW;
    static constexpr int AP = 0;            // phase 3-4 (overwrites A_U, D_U after they are read)
    static constexpr int DP = NV * APW;
    static constexpr int NEED_A = DU + NV * D.nu, NEED_P = DP + NV * kTcNP;
    static constexpr int NEED = NEED_A > NEED_P ? NEED_A : NEED_P;
    static constexpr int COLS = NEED <= 32 ? 32 : NEED <= 64 ? 64 : NEED <= 128 ? 128 : 256;
    static_assert(NEED <= 256, "tensor-memory budget of one CTA");
    static_assert(AUW % 8 == 0, "A_U is stored in groups of 8 columns");
};

constexpr int kSmemHead = 128;   // barriers, tensor-memory address, flags

template <int P, int NV>
DGX_HD constexpr size_t tc_smem_bytes(int nslot, int prefetch) {
    return kSmemHead + tc_dims(P).bytes +
           sizeof(R) * (static_cast<size_t>(side_table_words<P, NV>()) + slot_area_words<P, NV>(nslot)) +
           prefetch_bytes<P, NV>(prefetch);
}

constexpr unsigned kStatusMmaTimeout = kStatusCopyTimeout;
// polls of an MMA-completion barrier before the kernel gives up (an MMA of this
// size completes in microseconds)
constexpr long long kMmaWait = 1ll << 22;

constexpr int kTcThreads = 2 * kTile;   // two threads per element (row)

template <int P, int EQ, bool BND>
__global__ void __launch_bounds__(kTcThreads, 2) stage_kernel_tc(const StageArgs a) {
    using L = Lay<P>;
    constexpr int NP = L::NP, NQ = L::NQ, NQ1 = L::NQ1;
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    using TC = TcCols<P, NV>;
    constexpr TcDims D = tc_dims(P);
    // the two threads of a row split the variables (Euler: 0,1 | 2,3; advection:
    // the first thread), the volume points and the side points
    constexpr int VH = NV == 4 ? 2 : 1;
    constexpr int QH = (NQ + 1) / 2, SP = 3 * NQ1, SH = (SP + 1) / 2;

    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned long long *bar_pre = reinterpret_cast<unsigned long long *>(smem_raw);
    unsigned long long *bar_mma = bar_pre + 1;
    unsigned *s_tslot = reinterpret_cast<unsigned *>(smem_raw + 16);
    int *s_fail = reinterpret_cast<int *>(smem_raw + 20);
    unsigned char *s_img = smem_raw + kSmemHead;
    R *s_side = reinterpret_cast<R *>(s_img + D.bytes);
    R *s_tr = s_side + side_table_words<P, NV>();
    R *s_pre = s_tr + slot_area_words<P, NV>(a.nslot);
    const int tile = blockIdx.x;

    R dt;
    if (a.mode == 0) {
        dt = R(a.dt);
    } else {
        dt = R(a.scal[0]);
        if (dt == R(0)) return;   // the run has reached its end time (uniform over the grid)
    }
    const int E = a.E;
    const int t = threadIdx.x;
    const int r = t & (kTile - 1);    // row: element of the tile and tensor-memory lane
    const int h = t / kTile;          // which of the row's two threads (uniform over a warp)
    const int e = tile * kTile + r;
    const bool live = e < E;
    const size_t SE = static_cast<size_t>(E);
    const R g = R(a.gammaf), ax = R(a.axf), ay = R(a.ayf);
    const int llf = a.flux == DGX_FLUX_LLF;
    const R *__restrict__ u = static_cast<const R *>(a.u);
    const bool has_vars = NV == 4 || h == 0;   // advection: the variable work is the first thread's
    const int v0 = NV == 4 ? h * VH : 0;

    if (t == 0) {
        mbar_init(bar_pre, 1);
        mbar_init(bar_mma, 1);
        *s_fail = 0;
    }
    if (t < 32) {
        tc::tmem_alloc(s_tslot, TC::COLS);
        tc::tmem_relinquish();
    }
    {   // the constant B operands and the side tables (halo traces) into shared memory
        const uint4 *src = static_cast<const uint4 *>(a.tc_img);
        uint4 *dst = reinterpret_cast<uint4 *>(s_img);
        for (int i = t; i < D.bytes / 16; i += kTcThreads) dst[i] = __ldg(src + i);
        for (int i = t; i < 3 * NP * NQ1; i += kTcThreads) s_side[i] = c_tab[L::SIDE + i];
    }
    tc::fence_before_sync();
    __syncthreads();   // barriers initialised, tensor memory allocated
    tc::fence_after_sync();
    const unsigned tbase = *s_tslot;
    const unsigned tlane = tc::tmem_lane_base(tbase);

    const bool pre = issue_prefetch<P, NV>(a, tile, bar_pre, s_pre, t);

    // the row's mean coefficients, this thread's variables, side data, geometry
    R c0[NV], cv[VH][NP];
#pragma unroll
    for (int n = 0; n < NV; ++n) c0[n] = live ? __ldg(u + (n * NP) * SE + e) : R(0);
#pragma unroll
    for (int n = 0; n < VH; ++n)
#pragma unroll
        for (int i = 0; i < NP; ++i) cv[n][i] = live && has_vars ? __ldg(u + ((v0 + n) * NP + i) * SE + e) : R(0);
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
    R invJ = R(0), xr = R(0), yr = R(0), xs = R(0), ys = R(0);
    if (live) {
        const R *__restrict__ geo = static_cast<const R *>(a.geo);
        invJ = __ldg(geo + e);
        xr = __ldg(geo + SE + e);
        yr = __ldg(geo + 2 * SE + e);
        xs = __ldg(geo + 3 * SE + e);
        ys = __ldg(geo + 4 * SE + e);
    }

    // 1. A_U: modes 1..np-1 of this thread's variables as (hi, lo) words, one
    //    column each; zero padding
    if (has_vars) {
#pragma unroll
        for (int n = 0; n < VH; ++n) {
            unsigned w[TC::AUW];
#pragma unroll
            for (int m = 0; m < TC::AUW; ++m) w[m] = (m + 1 < NP) ? tc::split_word(cv[n][m + 1]) : 0u;
#pragma unroll
            for (int b = 0; b < TC::AUW; b += 8) tc::tmem_st8(tlane + TC::AU + (v0 + n) * TC::AUW + b, w + b);
        }
        tc::tmem_wait_st();
    }
    tc::fence_proxy_async();   // the B operands were written by the generic proxy
    tc::fence_before_sync();
    __syncthreads();
    // 2. D_U = A_U (B_U hi, hi) + A_U (B_U lo, lo)
    if (t == 0) {
        tc::fence_after_sync();
        constexpr unsigned idu = tc::idesc_bf16_f32(kTile, D.nu);
        const unsigned sb = tc::smem_u32(s_img);
#pragma unroll
        for (int n = 0; n < NV; ++n)
#pragma unroll
            for (int s = 0; s < D.ku / 16; ++s) {
                const unsigned dcol = tbase + TC::DU + n * D.nu;
                const unsigned acol = tbase + TC::AU + n * TC::AUW + 8 * s;
                tc::mma_ts(dcol, acol, tc::smem_desc(sb + D.off_buh + 256 * s, 128, D.sbo_u), idu, s > 0 ? 1u : 0u);
                tc::mma_ts(dcol, acol, tc::smem_desc(sb + D.off_bul + 256 * s, 128, D.sbo_u), idu, 1u);
            }
        tc::mma_commit(bar_mma);
    }

    // reference state: the physical flux of the cell-average state
    const R phi0 = c_tab[L::PHI];
    R fxr[NV], fyr[NV];
    {
        R ub[NV];
#pragma unroll
        for (int n = 0; n < NV; ++n) ub[n] = c0[n] * phi0;
        phys_flux<EQ>(ub, g, ax, ay, fxr, fyr);
    }

    // halo traces (FP32), overlapping the MMAs: the tile's neighbours outside
    // the tile, on their own side and in their own point order
    {
        const int hb = __ldg(a.halo_off + tile), H = __ldg(a.halo_off + tile + 1) - hb;
        for (int hh = t; hh < H; hh += kTcThreads) {
            const int hw = __ldg(a.halo_list + hb + hh);
            const int ne = hw >> 2;
            R cn[NV][NP];
#pragma unroll
            for (int n = 0; n < NV; ++n)
#pragma unroll
                for (int i = 0; i < NP; ++i) cn[n][i] = __ldg(u + (n * NP + i) * SE + ne);
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
                    const R tv = ts[i * NQ1 + j];
#pragma unroll
                    for (int n = 0; n < NV; ++n) tr[j][n] = fma(cn[n][i], tv, tr[j][n]);
                }
#pragma unroll
            for (int j = 0; j < NQ1; ++j)
#pragma unroll
                for (int n = 0; n < NV; ++n) s_tr[slot_off<P, NV>(3 * kTile + hh) + j * NV + n] = tr[j][n];
        }
    }

    // 3. point values: this thread's volume points to registers, its side
    //    points (own traces) to shared memory
    if (!mbar_wait_bounded(bar_mma, 0, kMmaWait)) *s_fail = 1;
    tc::fence_after_sync();
    const int q0 = h * QH, s0 = h * SH;
    R Uv[NV][QH];
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        float d[D.nu];
#pragma unroll
        for (int b = 0; b < D.nu; b += 16) tc::tmem_ld16(tlane + TC::DU + n * D.nu + b, d + b);
        tc::tmem_wait_ld();
        const R m0 = c0[n] * phi0;
#pragma unroll
        for (int qq = 0; qq < QH; ++qq) {
            // q0 + qq < NQ except for the second thread's last point at odd NQ
            Uv[n][qq] = (h == 0 ? d[qq] : d[(QH + qq) < NQ ? QH + qq : 0]) + m0;
        }
#pragma unroll
        for (int ss = 0; ss < SH; ++ss) {
            const int sp = s0 + ss;
            if (sp < SP) {
                const int k = sp / NQ1, j = sp - k * NQ1;
                s_tr[slot_off<P, NV>(3 * r + k) + j * NV + n] = (h == 0 ? d[NQ + ss] : d[NQ + SH + ss < D.nu ? NQ + SH + ss : 0]) + m0;
            }
        }
    }
    __syncthreads();   // all traces of the tile and its halo are in shared memory
    const bool fail = *s_fail != 0;   // uniform over the CTA

    R hxr[NV], hyr[NV];   // the reference state's geometry-weighted volume flux
#pragma unroll
    for (int n = 0; n < NV; ++n) {
        hxr[n] = fxr[n] * ys - fyr[n] * xs;
        hyr[n] = fyr[n] * xr - fxr[n] * yr;
    }
    R sgk[3];             // per side: lift sign times half length
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int word = sw[k];
        const bool bnd = BND && word < 0;
        const int il = bnd ? 1 : (word & 1);
        sgk[k] = il ? -shl[k] : shl[k];
    }
    if (!fail) {
        // A' volume part: (x part, y part) of the flux at this thread's points,
        // minus the reference
#pragma unroll
        for (int qq = 0; qq < QH; ++qq) {
            const int q = q0 + qq;
            if (q < NQ) {
                R U[NV], fx[NV], fy[NV];
#pragma unroll
                for (int n = 0; n < NV; ++n) U[n] = Uv[n][qq];
                phys_flux<EQ>(U, g, ax, ay, fx, fy);
#pragma unroll
                for (int n = 0; n < NV; ++n) {
                    const R hr = fx[n] * ys - fy[n] * xs - hxr[n];
                    const R hs = fy[n] * xr - fx[n] * yr - hyr[n];
                    tc::tmem_st2(tlane + TC::AP + n * TC::APW + 2 * q, tc::split_word(hr), tc::split_word(hs));
                }
            }
        }
        // A' side part: the lifted numerical flux at this thread's side points,
        // minus the reference
#pragma unroll
        for (int ss = 0; ss < SH; ++ss) {
            const int sp = s0 + ss;
            if (sp < SP) {
                const int k = sp / NQ1, j = sp - k * NQ1;
                const int word = pick3(sw[0], sw[1], sw[2], k);
                const R nx = pick3(snx[0], snx[1], snx[2], k), ny = pick3(sny[0], sny[1], sny[2], k);
                const int own = 3 * r + k;
                const bool bnd = BND && word < 0;
                const int slot = bnd ? own : (word >> 1);
                const int il = bnd ? 1 : (word & 1);
                const R sg = pick3(sgk[0], sgk[1], sgk[2], k);
                R UO[NV], UN[NV], UL[NV], UR[NV], Fh[NV];
#pragma unroll
                for (int n = 0; n < NV; ++n) {
                    UO[n] = s_tr[slot_off<P, NV>(own) + j * NV + n];
                    UN[n] = s_tr[slot_off<P, NV>(slot) + (NQ1 - 1 - j) * NV + n];
                }
                if constexpr (BND) {
                    if (bnd) boundary_ghost<P, EQ>(a, word, k, j, e, UO, nx, ny, UN);
                }
#pragma unroll
                for (int n = 0; n < NV; ++n) {
                    UL[n] = il ? UO[n] : UN[n];
                    UR[n] = il ? UN[n] : UO[n];
                }
                num_flux<EQ>(UL, UR, nx, ny, llf, g, ax, ay, Fh);
#pragma unroll
                for (int n = 0; n < NV; ++n)
                    tc::tmem_st1(tlane + TC::AP + n * TC::APW + 2 * NQ + sp,
                                 tc::split_word(sg * (Fh[n] - (fxr[n] * nx + fyr[n] * ny))));
            }
        }
        // zero padding of A'
        if (h == 0) {
#pragma unroll
            for (int n = 0; n < NV; ++n)
#pragma unroll
                for (int col = D.ka; col < TC::APW; ++col) tc::tmem_st1(tlane + TC::AP + n * TC::APW + col, 0u);
        }
        tc::tmem_wait_st();
    }
    tc::fence_before_sync();
    __syncthreads();
    // 4. D_P = A' (B_P hi, hi) + A' (B_P lo, lo)
    if (t == 0 && !fail) {
        tc::fence_after_sync();
        constexpr unsigned idp = tc::idesc_bf16_f32(kTile, kTcNP);
        const unsigned sb = tc::smem_u32(s_img);
#pragma unroll
        for (int n = 0; n < NV; ++n)
#pragma unroll
            for (int s = 0; s < D.kpv / 16; ++s) {
                const unsigned dcol = tbase + TC::DP + n * kTcNP;
                const unsigned acol = tbase + TC::AP + n * TC::APW + 8 * s;
                tc::mma_ts(dcol, acol, tc::smem_desc(sb + D.off_bph + 256 * s, 128, D.sbo_p), idp, s > 0 ? 1u : 0u);
                tc::mma_ts(dcol, acol, tc::smem_desc(sb + D.off_bpl + 256 * s, 128, D.sbo_p), idp, 1u);
            }
        tc::mma_commit(bar_mma);
    }
    bool ok = !fail;
    R rhs[VH][NP];
    if (ok) {
        // the reference state's part of this thread's variables, exactly: its
        // flux is constant over the element, so its projection is a constant
        // times the tables' column sums
        const float *sums = reinterpret_cast<const float *>(s_img + D.off_sum);
#pragma unroll
        for (int n = 0; n < VH; ++n) {
            const int v = v0 + n;
            R hx = hxr[0], hy = hyr[0], fxv = fxr[0], fyv = fyr[0];
#pragma unroll
            for (int m = 1; m < NV; ++m)
                if (v == m) { hx = hxr[m]; hy = hyr[m]; fxv = fxr[m]; fyv = fyr[m]; }
            R fr[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) fr[k] = sgk[k] * (fxv * snx[k] + fyv * sny[k]);
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                R acc = hx * sums[i] + hy * sums[16 + i];
#pragma unroll
                for (int k = 0; k < 3; ++k) acc = fma(fr[k], sums[32 + 16 * k + i], acc);
                rhs[n][i] = acc;
            }
        }
        if (!mbar_wait_bounded(bar_mma, 1, kMmaWait)) {
            atomicOr(a.status, kStatusMmaTimeout);
            mbar_wait_bounded(bar_mma, 1, 4 * kMmaWait);
            ok = false;
        }
        tc::fence_after_sync();
#pragma unroll
        for (int n = 0; n < VH; ++n) {
            float d[kTcNP];
            tc::tmem_ld16(tlane + TC::DP + (v0 + n) * kTcNP, d);
            tc::tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < NP; ++i) rhs[n][i] += d[i];
        }
    } else {
        // the point-value MMAs did not complete in time: report, give them a
        // last chance before the tensor memory is freed, write nothing
        if (t == 0) atomicOr(a.status, kStatusMmaTimeout);
        mbar_wait_bounded(bar_mma, 0, 4 * kMmaWait);
    }
    // 5. the RK combination of this thread's variables
    if (ok && live && has_vars) {
        if constexpr (NV == 4) {
            if (h == 0) stage_epilogue<P, EQ, 0, VH>(a, rhs, cv, dt, invJ, e, SE, pre, s_pre, bar_pre, 0u, r);
            else stage_epilogue<P, EQ, VH, VH>(a, rhs, cv, dt, invJ, e, SE, pre, s_pre, bar_pre, 0u, r);
        } else {
            stage_epilogue<P, EQ, 0, VH>(a, rhs, cv, dt, invJ, e, SE, pre, s_pre, bar_pre, 0u, r);
        }
    } else if (pre && t < 32) {
        mbar_wait_bounded(bar_pre, 0u, 1ll << 28);   // no copy in flight at exit
    }
    tc::fence_before_sync();
    __syncthreads();
    if (t < 32) tc::tmem_dealloc(tbase, TC::COLS);
}

template <int P, int EQ, bool BND>
int launch_tc_one(const StageArgs &a_in, cudaStream_t st) {
    constexpr int NV = (EQ == DGX_EULER) ? 4 : 1;
    StageArgs a = a_in;
    if (a.prefetch && tc_smem_bytes<P, NV>(a.nslot, a.prefetch) > 200 * 1024) a.prefetch = 0;
    const size_t smem = tc_smem_bytes<P, NV>(a.nslot, a.prefetch);
    if (smem > 227 * 1024) { set_error("tile halo too large for shared memory (%zu bytes)", smem); return DGX_ERR_UNSUPPORTED; }
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        DGX_TRY_CUDA(cudaFuncSetAttribute(stage_kernel_tc<P, EQ, BND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(smem)));
        DGX_TRY_CUDA(cudaFuncSetAttribute(stage_kernel_tc<P, EQ, BND>,
                                          cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        configured = smem;
    }
    const int grid = (a.E + kTile - 1) / kTile;
    if (grid > 0) stage_kernel_tc<P, EQ, BND><<<grid, kTcThreads, smem, st>>>(a);
    DGX_CHECK_LAUNCH();
    return DGX_OK;
}

template <int EQ, bool BND>
int launch_tc_order(int order, const StageArgs &a, cudaStream_t st) {
    switch (order) {
    case 1: return launch_tc_one<1, EQ, BND>(a, st);
    case 2: return launch_tc_one<2, EQ, BND>(a, st);
    case 3: return launch_tc_one<3, EQ, BND>(a, st);
    case 4: return launch_tc_one<4, EQ, BND>(a, st);
    default: set_error("the BF16x3 path serves orders 1..4, not %d", order); return DGX_ERR_UNSUPPORTED;
    }
}

}  // namespace

int launch_stage_tc(int order, int equation, const StageArgs &a, cudaStream_t st) {
    if (!a.tc_img) { set_error("tensor-core tables missing"); return DGX_ERR_INVALID; }
    if (equation == DGX_EULER)
        return a.bnd ? launch_tc_order<DGX_EULER, true>(order, a, st) : launch_tc_order<DGX_EULER, false>(order, a, st);
    return a.bnd ? launch_tc_order<DGX_ADVECTION, true>(order, a, st)
                 : launch_tc_order<DGX_ADVECTION, false>(order, a, st);
}

int upload_tables_tc() { return upload_tables_impl(); }

}  // namespace dgx
