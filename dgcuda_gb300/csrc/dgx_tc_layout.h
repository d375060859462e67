// dgx_tc_layout.h -- operand shapes of the tensor-core (BF16x3) stage kernel
// per order p (1..4), shared by the host code that builds the constant B
// operands and by the kernel.
//
// Two contractions per element and variable run as tcgen05 MMAs (M = 128
// elements of a tile, one per tensor-memory lane):
//   U   point values: D_U[e][n] = sum_m c[e][m] phi_m(n), m = 1..np-1 (the
//       mean mode 0 is added exactly in FP32), n over the nq volume points and
//       then the 3*nq1 side points (side-major);            K = ku, N = nu
//   P   projection: D_P[e][i] = sum_a A'[e][a] b_i(a) over the a = 2q (x part of
//       the volume flux at point q, tested with w dphi_i/dr), a = 2q+1 (y part,
//       w dphi_i/ds) and a = 2nq + k*nq1 + j (lifted side flux, w_j phi_i on
//       side k);                                             K = kpv, N = 16
// Each A value x occupies one 32-bit tensor-memory column as the BF16 pair
// (hi, lo), x = hi + lo + O(2^-17 |x|), so K counts two BF16 per value; the B
// operand comes in two variants, (b_hi, b_hi) and (b_lo, b_lo) per pair, and
// two MMAs give hi b_hi + lo b_hi + hi b_lo + lo b_lo = (hi + lo)(b_hi + b_lo):
// the three-term split product plus its lo*lo term, which this layout gets for
// free.
// B operands live in shared memory, K-major without swizzle: element (row, k)
// at (row/8)*SBO + (k/8)*128 + (row%8)*16 + (k%8)*2 with SBO = (K/8)*128.
#pragma once

#include "dgx_tables.h"

namespace dgx {

DGX_HD constexpr int round16(int x) { return (x + 15) / 16 * 16; }

struct TcDims {
    int np, nq, nq1;
    int ku, nu;         // U: K (BF16 elements) and N
    int ka, kpv;        // P: values per element and variable, K (BF16 elements)
    int sbo_u, sbo_p;   // 8-row-group strides of the B operands (bytes)
    int off_buh, off_bul, off_bph, off_bpl, off_sum, bytes;   // image layout (bytes)
};

constexpr int kTcMinOrder = 1, kTcMaxOrder = 4;
constexpr int kTcNP = 16;                    // N of the projection (modes, padded)
constexpr int kTcSums = 16 + 16 + 3 * 16;    // Sx[i], Sy[i], L[k][i] (floats)

DGX_HD constexpr TcDims tc_dims(int p) {
    TcDims d{};
    d.np = num_modes(p);
    d.nq = num_quad(p);
    d.nq1 = num_quad1(p);
    d.ku = round16(2 * (d.np - 1));
    d.nu = round16(d.nq + 3 * d.nq1);
    d.ka = 2 * d.nq + 3 * d.nq1;
    d.kpv = round16(2 * d.ka);
    d.sbo_u = (d.ku / 8) * 128;
    d.sbo_p = (d.kpv / 8) * 128;
    d.off_buh = 0;
    d.off_bul = d.nu * d.ku * 2;
    d.off_bph = 2 * d.nu * d.ku * 2;
    d.off_bpl = d.off_bph + kTcNP * d.kpv * 2;
    d.off_sum = d.off_bpl + kTcNP * d.kpv * 2;
    d.bytes = round16(d.off_sum + kTcSums * 4);
    return d;
}

// byte offset of element (row, k) of a K-major operand with K columns
DGX_HD constexpr int tc_kmajor_off(int row, int k, int K) {
    return (row / 8) * ((K / 8) * 128) + (k / 8) * 128 + (row % 8) * 16 + (k % 8) * 2;
}

}  // namespace dgx
