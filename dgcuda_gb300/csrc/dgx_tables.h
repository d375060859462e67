// dgx_tables.h -- sizes of the modal basis and quadrature rules per order p,
// and the FP64 host tables (see dgx_tables.cpp).
#pragma once

#ifdef __CUDACC__
#define DGX_HD __host__ __device__
#else
#define DGX_HD
#endif

namespace dgx {

constexpr int kMaxOrder = 5;
constexpr int kMaxModes = 21;
constexpr int kMaxQuad = 25;
constexpr int kMaxQuad1 = 6;

// n_p = (p+1)(p+2)/2 (src/2d/conservation/main.cu:44)
DGX_HD constexpr int num_modes(int p) { return (p + 1) * (p + 2) / 2; }
// degree-2p triangle rule sizes (src/2d/conservation/conserv.cu:61-80)
DGX_HD constexpr int num_quad(int p) {
    return p == 0 ? 1 : p == 1 ? 3 : p == 2 ? 6 : p == 3 ? 12 : p == 4 ? 16 : 25;
}
DGX_HD constexpr int num_quad1(int p) { return p + 1; }

// Per-order block of the device tables: phi[np*nq], gx[np*nq], gy[np*nq],
// side[3*np*nq1], lift[3*np*nq1] (= w1[j] * side), w1[nq1], and the reference
// coordinates of the side points srs[3][nq1][2].
DGX_HD constexpr int table_block(int p) {   // rounded up to 4 values: every order's block starts 16-byte aligned
    return (3 * num_modes(p) * num_quad(p) + 6 * num_modes(p) * num_quad1(p) + num_quad1(p) + 6 * num_quad1(p) + 3) &
           ~3;
}
DGX_HD constexpr int table_offset(int p) { return p == 0 ? 0 : table_offset(p - 1) + table_block(p - 1); }
constexpr int kTableTotal = table_offset(kMaxOrder + 1);

struct Tables {
    int p = 0, np = 0, nq = 0, nq1 = 0;
    double r1[kMaxQuad] = {}, r2[kMaxQuad] = {}, w[kMaxQuad] = {};   // w sums to 1/2
    double s1[kMaxQuad1] = {}, w1[kMaxQuad1] = {};                    // Gauss on [-1,1]
    double phi[kMaxModes * kMaxQuad] = {};                            // [i*nq + q]
    double gx[kMaxModes * kMaxQuad] = {};                             // w_q dphi_i/dr
    double gy[kMaxModes * kMaxQuad] = {};                             // w_q dphi_i/ds
    double side[3 * kMaxModes * kMaxQuad1] = {};                      // [(s*np + i)*nq1 + j]
    double vert[3 * kMaxModes] = {};                                  // [3*i + v]
};

bool build_tables(int p, Tables &T);
const Tables &tables(int p);   // cached, p in [0, kMaxOrder]

}  // namespace dgx
