// dgx_meshgen.cpp -- structured periodic triangulations, generated on the host.
//
// n x n squares on [x0, x0+lx] x [y0, y0+ly], each split along its SW-NE
// diagonal into a lower (SW, SE, NE) and an upper (SW, NE, NW) triangle;
// element 2q / 2q+1 and sides 3q (bottom), 3q+1 (left), 3q+2 (diagonal) belong
// to square q = j*n + i.  Periodic sides are ordinary interior sides.  Interior
// vertices move by jitter * h * (2u - 1) in x and y, with u from a counter-based
// generator (splitmix64 of the seed and the vertex index), so the mesh does not
// depend on the order of generation and the Python generator
// (dgcuda_gb300/mesh.py) reproduces it bit for bit.
#include <cstdint>
#include <vector>

#include "dgx.h"
#include "dgx_internal.h"

namespace dgx {

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

inline double unit_draw(uint64_t seed, uint64_t k) {
    return static_cast<double>(splitmix64(seed * 0x9E3779B97F4A7C15ull + k) >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace

int periodic_square_arrays(int n, double lx, double ly, double x0, double y0, double jitter,
                           unsigned long long seed, double *V, int *elem_s, int *sides) {
    if (n < 1 || n > 8192 || !(lx > 0) || !(ly > 0) || jitter < 0 || jitter >= 0.5) {
        set_error("periodic square: need 1 <= n <= 8192, lx, ly > 0 and 0 <= jitter < 0.5");
        return DGX_ERR_INVALID;
    }
    const int nv = n + 1;
    const double hx = lx / n, hy = ly / n;
    std::vector<double> X(static_cast<size_t>(nv) * nv), Y(static_cast<size_t>(nv) * nv);
    for (int j = 0; j < nv; ++j)
        for (int i = 0; i < nv; ++i) {
            const size_t v = static_cast<size_t>(j) * nv + i;
            double x = x0 + i * hx, y = y0 + j * hy;
            if (jitter > 0 && i > 0 && i < n && j > 0 && j < n) {
                x += (jitter * hx) * (2.0 * unit_draw(seed, 2 * v) - 1.0);
                y += (jitter * hy) * (2.0 * unit_draw(seed, 2 * v + 1) - 1.0);
            }
            X[v] = x;
            Y[v] = y;
        }
    const size_t E = 2 * static_cast<size_t>(n) * n, S = 3 * static_cast<size_t>(n) * n;
    auto at = [&](int i, int j) { return static_cast<size_t>(j) * nv + i; };
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            const int q = j * n + i;
            const size_t sw = at(i, j), se = at(i + 1, j), ne = at(i + 1, j + 1), nw = at(i, j + 1);
            const size_t lo = 2 * static_cast<size_t>(q), up = lo + 1;
            const double lower[6] = {X[sw], Y[sw], X[se], Y[se], X[ne], Y[ne]};
            const double upper[6] = {X[sw], Y[sw], X[ne], Y[ne], X[nw], Y[nw]};
            for (int c = 0; c < 6; ++c) {
                V[c * E + lo] = lower[c];
                V[c * E + up] = upper[c];
            }
            const int qr = j * n + (i + 1) % n, qu = ((j + 1) % n) * n + i;
            const int ql = j * n + (i + n - 1) % n, qd = ((j + n - 1) % n) * n + i;
            elem_s[lo] = 3 * q;          elem_s[E + lo] = 3 * qr + 1; elem_s[2 * E + lo] = 3 * q + 2;
            elem_s[up] = 3 * q + 2;      elem_s[E + up] = 3 * qu;     elem_s[2 * E + up] = 3 * q + 1;
            const size_t b = 3 * static_cast<size_t>(q);
            // bottom: lower triangle's side 0 | upper triangle of the square below, side 1
            sides[b] = 2 * q;         sides[S + b] = 2 * qd + 1;     sides[2 * S + b] = 0; sides[3 * S + b] = 1;
            // left: upper triangle's side 2 | lower triangle of the square to the left, side 1
            sides[b + 1] = 2 * q + 1; sides[S + b + 1] = 2 * ql;     sides[2 * S + b + 1] = 2; sides[3 * S + b + 1] = 1;
            // diagonal: lower triangle's side 2 | upper triangle's side 0
            sides[b + 2] = 2 * q;     sides[S + b + 2] = 2 * q + 1;  sides[2 * S + b + 2] = 2; sides[3 * S + b + 2] = 0;
        }
    return DGX_OK;
}

}  // namespace dgx

extern "C" {

int dgx_periodic_square_arrays(int n, double lx, double ly, double x0, double y0, double jitter,
                               unsigned long long seed, double *V, int *elem_s, int *sides) {
    if (!V || !elem_s || !sides) { dgx::set_error("NULL output array"); return DGX_ERR_INVALID; }
    return dgx::periodic_square_arrays(n, lx, ly, x0, y0, jitter, seed, V, elem_s, sides);
}

int dgx_mesh_create_periodic_square(int n, double lx, double ly, double x0, double y0,
                                    double jitter, unsigned long long seed, dgx_mesh **out) {
    if (!out) { dgx::set_error("out is NULL"); return DGX_ERR_INVALID; }
    if (n < 1 || n > 8192) { dgx::set_error("n outside 1..8192"); return DGX_ERR_INVALID; }
    const size_t E = 2 * static_cast<size_t>(n) * n, S = 3 * static_cast<size_t>(n) * n;
    std::vector<double> V(6 * E);
    std::vector<int> es(3 * E), sd(4 * S);
    int rc = dgx::periodic_square_arrays(n, lx, ly, x0, y0, jitter, seed, V.data(), es.data(), sd.data());
    if (rc) return rc;
    return dgx_mesh_create(static_cast<int>(E), static_cast<int>(S), V.data(), V.data() + E,
                           V.data() + 2 * E, V.data() + 3 * E, V.data() + 4 * E, V.data() + 5 * E,
                           es.data(), es.data() + E, es.data() + 2 * E, sd.data(), sd.data() + S,
                           sd.data() + 2 * S, sd.data() + 3 * S, out);
}

}  // extern "C"
