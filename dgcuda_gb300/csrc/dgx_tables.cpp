// dgx_tables.cpp -- one-time basis and quadrature tables (host, extended precision).
//
// The reference tabulates a hard-coded Gram-Schmidt coefficient table
// (src/2d/basis.cu:1-71, accurate to ~1e-14 for p <= 3 and ~1e-9 at p = 4) at
// the points of its quadrature rules (src/2d/quadrature.cu, selected by
// set_quadrature, src/2d/conservation/conserv.cu:37-107).  Here the same
// functions -- the Gram-Schmidt orthonormalisation, on the reference triangle
// (0,0),(1,0),(0,1), of the graded-lex monomials r^(d-j) s^j -- are computed
// afresh in long double: classical Gram-Schmidt with re-orthogonalisation on
// centred monomials (same nested spans, hence the same functions), with inner
// products by the degree-2p rule, which integrates every product exactly.
// Derivatives ride along as the same linear combinations.
#include "dgx_tables.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace dgx {

namespace {

struct Orbit {
    int kind;      // 0 centroid, 1 S21 (a,a,1-2a), 2 S111 (a,b,1-a-b)
    double a, b, w;
    int perm;      // listing order of the orbit's points
};

// Dunavant's symmetric rules with the reference's point order.  S21 orbits are
// listed as (1-2a,a),(a,1-2a),(a,a) except the degree-2 rule, which lists
// (a,a),(1-2a,a),(a,1-2a).  S111 orbits use the permutation tables below.
const int kPerm111[4][6][2] = {
    {{2, 1}, {1, 2}, {2, 0}, {1, 0}, {0, 1}, {0, 2}},
    {{0, 2}, {2, 0}, {1, 0}, {0, 1}, {1, 2}, {2, 1}},
    {{0, 1}, {1, 0}, {1, 2}, {2, 1}, {2, 0}, {0, 2}},
    {{0, 1}, {1, 0}, {0, 2}, {2, 0}, {2, 1}, {1, 2}},
};

std::vector<Orbit> rule_orbits(int p) {
    switch (p) {
    case 0: return {{0, 0, 0, 1.0, 0}};
    case 1: return {{1, 1.0 / 6.0, 0, 1.0 / 3.0, 1}};
    case 2: return {{1, 0.091576213509771, 0, 0.109951743655322, 0},
                    {1, 0.445948490915965, 0, 0.223381589678011, 0}};
    case 3: return {{1, 0.063089014491502, 0, 0.050844906370207, 0},
                    {1, 0.249286745170910, 0, 0.116786275726379, 0},
                    {2, 0.053145049844816, 0.310352451033784, 0.082851075618374, 0}};
    case 4: return {{0, 0, 0, 0.144315607677787, 0},
                    {1, 0.459292588292723, 0, 0.095091634267285, 0},
                    {1, 0.170569307751760, 0, 0.103217370534718, 0},
                    {1, 0.050547228317031, 0, 0.032458497623198, 0},
                    {2, 0.008394777409958, 0.263112829634638, 0.027230314174435, 1}};
    case 5: return {{0, 0, 0, 0.090817990382754, 0},
                    {1, 0.485577633383657, 0, 0.036725957756467, 0},
                    {1, 0.109481575485037, 0, 0.045321059435528, 0},
                    {2, 0.141707219414880, 0.307939838764121, 0.072757916845420, 2},
                    {2, 0.025003534762686, 0.246672560639903, 0.028327242531057, 3},
                    {2, 0.009540815400299, 0.066803251012200, 0.009421666963733, 2}};
    default: return {};
    }
}

void expand_rule(int p, std::vector<double> &r, std::vector<double> &s, std::vector<double> &w) {
    for (const Orbit &o : rule_orbits(p)) {
        if (o.kind == 0) {
            r.push_back(1.0 / 3.0); s.push_back(1.0 / 3.0); w.push_back(o.w);
        } else if (o.kind == 1) {
            const double a = o.a, c = 1.0 - 2.0 * a;
            const double pts[2][3][2] = {{{c, a}, {a, c}, {a, a}}, {{a, a}, {c, a}, {a, c}}};
            for (int k = 0; k < 3; ++k) {
                r.push_back(pts[o.perm][k][0]); s.push_back(pts[o.perm][k][1]); w.push_back(o.w);
            }
        } else {
            const double abc[3] = {o.a, o.b, 1.0 - o.a - o.b};
            for (int k = 0; k < 6; ++k) {
                r.push_back(abc[kPerm111[o.perm][k][0]]);
                s.push_back(abc[kPerm111[o.perm][k][1]]);
                w.push_back(o.w);
            }
        }
    }
}

// Legendre P_n and P_{n-1} at x by the three-term recurrence.
void legendre(int n, long double x, long double &pn, long double &pn1) {
    long double a = 1.0L, b = x;
    if (n == 0) { pn = 1.0L; pn1 = 0.0L; return; }
    for (int k = 2; k <= n; ++k) {
        long double c = ((2 * k - 1) * x * b - (k - 1) * a) / k;
        a = b; b = c;
    }
    pn = b; pn1 = a;
}

void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
    const long double pi = 3.141592653589793238462643383279502884L;
    x.resize(n); w.resize(n);
    for (int i = 0; i < n; ++i) {
        long double z = std::cos(pi * (n - i - 0.25L) / (n + 0.5L));
        long double pn = 0, pn1 = 0, d = 1;
        for (int it = 0; it < 64; ++it) {
            legendre(n, z, pn, pn1);
            d = n * (z * pn - pn1) / (z * z - 1.0L);
            long double dz = pn / d;
            z -= dz;
            if (std::fabs(static_cast<double>(dz)) < 1e-300) break;
        }
        legendre(n, z, pn, pn1);
        d = n * (z * pn - pn1) / (z * z - 1.0L);
        x[i] = static_cast<double>(z);
        w[i] = static_cast<double>(2.0L / ((1.0L - z * z) * d * d));
    }
    if (n % 2) x[n / 2] = 0.0;
}

// graded-lex exponent pair of monomial k: r^(d-j) s^j
void lex_exponents(int k, int &a, int &b) {
    int d = 0, first = 0;
    while (first + d + 1 <= k) { first += d + 1; ++d; }
    b = k - first;
    a = d - b;
}

long double ipow(long double x, int n) {
    long double r = 1.0L;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
}

}  // namespace

bool build_tables(int p, Tables &T) {
    if (p < 0 || p > kMaxOrder) return false;
    T = Tables();
    T.p = p;
    T.np = num_modes(p);
    std::vector<double> r, s, w;
    expand_rule(p, r, s, w);
    T.nq = static_cast<int>(r.size());
    T.nq1 = p + 1;
    if (T.nq != num_quad(p)) return false;
    std::vector<double> g, gw;
    gauss_legendre(T.nq1, g, gw);
    for (int q = 0; q < T.nq; ++q) { T.r1[q] = r[q]; T.r2[q] = s[q]; T.w[q] = 0.5 * w[q]; }
    for (int j = 0; j < T.nq1; ++j) { T.s1[j] = g[j]; T.w1[j] = gw[j]; }

    // evaluation points: volume rule, the three sides in the reference's
    // orientation (basis.cu:192-196), then the three vertices
    std::vector<long double> pr, ps;
    for (int q = 0; q < T.nq; ++q) { pr.push_back(r[q]); ps.push_back(s[q]); }
    for (int j = 0; j < T.nq1; ++j) { pr.push_back(0.5L + 0.5L * g[j]); ps.push_back(0.0L); }
    for (int j = 0; j < T.nq1; ++j) { pr.push_back((1.0L - g[j]) / 2.0L); ps.push_back((1.0L + g[j]) / 2.0L); }
    for (int j = 0; j < T.nq1; ++j) { pr.push_back(0.0L); ps.push_back(0.5L + 0.5L * g[T.nq1 - 1 - j]); }
    pr.push_back(0); ps.push_back(0);
    pr.push_back(1); ps.push_back(0);
    pr.push_back(0); ps.push_back(1);
    const int npts = static_cast<int>(pr.size());

    std::vector<std::vector<long double>> F(T.np), Fr(T.np), Fs(T.np);
    auto dot = [&](const std::vector<long double> &a, const std::vector<long double> &b) {
        long double acc = 0.0L;
        for (int q = 0; q < T.nq; ++q) acc += static_cast<long double>(T.w[q]) * a[q] * b[q];
        return acc;
    };
    const long double third = 1.0L / 3.0L;
    for (int k = 0; k < T.np; ++k) {
        int a, b;
        lex_exponents(k, a, b);
        F[k].resize(npts); Fr[k].resize(npts); Fs[k].resize(npts);
        for (int q = 0; q < npts; ++q) {
            const long double x = pr[q] - third, y = ps[q] - third;
            F[k][q] = ipow(x, a) * ipow(y, b);
            Fr[k][q] = a ? a * ipow(x, a - 1) * ipow(y, b) : 0.0L;
            Fs[k][q] = b ? b * ipow(x, a) * ipow(y, b - 1) : 0.0L;
        }
        for (int sweep = 0; sweep < 2; ++sweep) {
            std::vector<long double> coef(k);
            for (int l = 0; l < k; ++l) coef[l] = dot(F[k], F[l]);
            for (int l = 0; l < k; ++l)
                for (int q = 0; q < npts; ++q) {
                    F[k][q] -= coef[l] * F[l][q];
                    Fr[k][q] -= coef[l] * Fr[l][q];
                    Fs[k][q] -= coef[l] * Fs[l][q];
                }
        }
        const long double nrm = std::sqrt(dot(F[k], F[k]));
        for (int q = 0; q < npts; ++q) { F[k][q] /= nrm; Fr[k][q] /= nrm; Fs[k][q] /= nrm; }
    }
    const int nq = T.nq, nq1 = T.nq1, np = T.np;
    for (int i = 0; i < np; ++i) {
        for (int q = 0; q < nq; ++q) {
            T.phi[i * nq + q] = static_cast<double>(F[i][q]);
            T.gx[i * nq + q] = static_cast<double>(static_cast<long double>(T.w[q]) * Fr[i][q]);
            T.gy[i * nq + q] = static_cast<double>(static_cast<long double>(T.w[q]) * Fs[i][q]);
        }
        for (int sd = 0; sd < 3; ++sd)
            for (int j = 0; j < nq1; ++j)
                T.side[(sd * np + i) * nq1 + j] = static_cast<double>(F[i][nq + sd * nq1 + j]);
        for (int v = 0; v < 3; ++v) T.vert[3 * i + v] = static_cast<double>(F[i][nq + 3 * nq1 + v]);
    }
    return true;
}

const Tables &tables(int p) {
    static Tables cache[kMaxOrder + 1];
    static bool built[kMaxOrder + 1] = {false};
    if (!built[p]) {
        build_tables(p, cache[p]);
        built[p] = true;
    }
    return cache[p];
}

}  // namespace dgx
