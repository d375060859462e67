// dgx_tc_tables.cpp -- the constant B operands of the tensor-core stage kernel
// (layout in dgx_tc_layout.h), built on the host from the FP64 basis and
// quadrature tables, split into BF16 hi/lo parts and uploaded once per device.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "dgx_internal.h"
#include "dgx_tc_layout.h"

namespace dgx {
namespace {

uint16_t bf16_rn(float f) {   // round to nearest even
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return static_cast<uint16_t>(u >> 16);   // Inf / NaN
    u += 0x7FFFu + ((u >> 16) & 1u);
    return static_cast<uint16_t>(u >> 16);
}
float bf16_f(uint16_t h) {
    const uint32_t u = static_cast<uint32_t>(h) << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
void split(double v, uint16_t &hi, uint16_t &lo) {
    hi = bf16_rn(static_cast<float>(v));
    lo = bf16_rn(static_cast<float>(v - static_cast<double>(bf16_f(hi))));
}
void put(std::vector<unsigned char> &img, int base, int row, int k, int K, uint16_t v) {
    std::memcpy(img.data() + base + tc_kmajor_off(row, k, K), &v, 2);
}

// value of basis mode m at U point n: volume points, then side points (side-major)
double u_point(const Tables &T, int m, int n) {
    if (n < T.nq) return T.phi[m * T.nq + n];
    const int r = n - T.nq;
    if (r >= 3 * T.nq1) return 0.0;
    const int ks = r / T.nq1, j = r % T.nq1;
    return T.side[(ks * T.np + m) * T.nq1 + j];
}

// projection weight of mode i for A value a
double p_weight(const Tables &T, int i, int a) {
    if (a < 2 * T.nq) return (a % 2 == 0) ? T.gx[i * T.nq + a / 2] : T.gy[i * T.nq + a / 2];
    const int r = a - 2 * T.nq;
    if (r >= 3 * T.nq1) return 0.0;
    const int ks = r / T.nq1, j = r % T.nq1;
    return T.w1[j] * T.side[(ks * T.np + i) * T.nq1 + j];
}

void build_image(int p, std::vector<unsigned char> &img) {
    const Tables &T = tables(p);
    const TcDims d = tc_dims(p);
    img.assign(d.bytes, 0);
    // U: rows n < nu, K pairs c <-> mode c + 1
    for (int n = 0; n < d.nu; ++n)
        for (int c = 0; 2 * c < d.ku; ++c) {
            const int m = c + 1;
            uint16_t hi = 0, lo = 0;
            if (m < T.np) split(u_point(T, m, n), hi, lo);
            put(img, d.off_buh, n, 2 * c, d.ku, hi);
            put(img, d.off_buh, n, 2 * c + 1, d.ku, hi);
            put(img, d.off_bul, n, 2 * c, d.ku, lo);
            put(img, d.off_bul, n, 2 * c + 1, d.ku, lo);
        }
    // P: rows i < 16 (modes), K pairs a
    for (int i = 0; i < kTcNP; ++i)
        for (int a = 0; 2 * a < d.kpv; ++a) {
            uint16_t hi = 0, lo = 0;
            if (i < T.np && a < d.ka) split(p_weight(T, i, a), hi, lo);
            put(img, d.off_bph, i, 2 * a, d.kpv, hi);
            put(img, d.off_bph, i, 2 * a + 1, d.kpv, hi);
            put(img, d.off_bpl, i, 2 * a, d.kpv, lo);
            put(img, d.off_bpl, i, 2 * a + 1, d.kpv, lo);
        }
    // sums for the mean parts: Sx[i] = sum_q gx, Sy[i] = sum_q gy, L[k][i] = sum_j w_j phi_i(k, j)
    float sums[kTcSums] = {};
    for (int i = 0; i < T.np; ++i) {
        double sx = 0.0, sy = 0.0;
        for (int q = 0; q < T.nq; ++q) {
            sx += T.gx[i * T.nq + q];
            sy += T.gy[i * T.nq + q];
        }
        sums[i] = static_cast<float>(sx);
        sums[16 + i] = static_cast<float>(sy);
        for (int ks = 0; ks < 3; ++ks) {
            double l = 0.0;
            for (int j = 0; j < T.nq1; ++j) l += T.w1[j] * T.side[(ks * T.np + i) * T.nq1 + j];
            sums[32 + 16 * ks + i] = static_cast<float>(l);
        }
    }
    std::memcpy(img.data() + d.off_sum, sums, sizeof(sums));
}

constexpr int kMaxDev = 64;
std::mutex g_mu;
unsigned char *g_dev_img[kMaxDev] = {};
int g_off[kTcMaxOrder + 1] = {};

}  // namespace

int tc_images_upload() {
    int dev = 0;
    DGX_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDev) { set_error("device index %d out of range", dev); return DGX_ERR_UNSUPPORTED; }
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_dev_img[dev]) return DGX_OK;
    std::vector<unsigned char> all;
    for (int p = kTcMinOrder; p <= kTcMaxOrder; ++p) {
        std::vector<unsigned char> img;
        build_image(p, img);
        g_off[p] = static_cast<int>(all.size());
        all.insert(all.end(), img.begin(), img.end());
    }
    unsigned char *d = nullptr;
    DGX_TRY_CUDA(cudaMalloc(&d, all.size()));
    const cudaError_t ce = cudaMemcpy(d, all.data(), all.size(), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        cudaFree(d);
        set_error("uploading the tensor-core tables failed: %s", cudaGetErrorString(ce));
        return DGX_ERR_CUDA;
    }
    g_dev_img[dev] = d;
    return DGX_OK;
}

const void *tc_image(int p) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev || p < kTcMinOrder || p > kTcMaxOrder)
        return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    return g_dev_img[dev] ? g_dev_img[dev] + g_off[p] : nullptr;
}

}  // namespace dgx
