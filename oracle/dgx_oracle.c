/*
 * dgx_oracle.c -- FP64 CPU oracle of the reference 2D modal DG scheme.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls this
 * file; tests/ and __graft_entry__.smoke() test the CUDA path against it, and
 * the CPU-baseline leg of bench.py times it.
 *
 * It restates, in plain C with OpenMP over edges and elements, the reference
 * (thePerv/DGCUDA) algorithm for one RHS evaluation and the classic RK4 step:
 *
 *   tables      src/2d/basis.cu:49-226 (Gram-Schmidt graded-lex orthonormal basis,
 *               tabulated at quadrature, side and vertex points),
 *               src/2d/quadrature.cu:7-173 + src/2d/conservation/conserv.cu:37-107
 *               (degree-2p triangle rule, (p+1)-point Gauss-Legendre)
 *   geometry    src/2d/conservation/conserv_kernels.cu:338-514
 *   surface     src/2d/conservation/conserv_kernels.cu:628-758 (Euler, LLF),
 *               src/2d/2dadvec/2dadvec_kernels.cu:471-571 (advection, central)
 *   volume      src/2d/conservation/conserv_kernels.cu:766-811,
 *               src/2d/2dadvec/2dadvec_kernels.cu:583-611
 *   eval_rhs    src/2d/conservation/time_integrator.cu:130-188
 *   RK4         src/2d/conservation/time_integrator.cu:194-218,221-434
 *   CFL         src/2d/conservation/euler/euler.cu:252-278 and
 *               src/2d/conservation/time_integrator.cu:252-270
 *   projection  src/2d/conservation/conserv_kernels.cu:167-187, euler.cu:31-59
 *
 * Physics: src/2d/conservation/euler/euler.cu:61-168 (pressure, sound speed,
 * flux, LLF wave speed).  With ref_sqrtf != 0 the oracle reproduces the
 * reference's single-precision square roots (sqrtf/powf on doubles in
 * conserv_kernels.cu:346,364-371,434 and euler.cu:80,272) so that it can be
 * pinned tightly against the reference's own CPU output; with ref_sqrtf == 0 it
 * is a true FP64 restatement of the same scheme.
 *
 * The traces and the numerical flux are evaluated once per Gauss point and then
 * tested against every mode (the reference recomputes them per mode,
 * conserv_kernels.cu:717-749); the arithmetic is otherwise the same.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAXP 5
#define ORC_MAXNP 21
#define ORC_MAXQ 25
#define ORC_MAXQ1 6
#define ORC_MAXV 4

enum { ORC_ADVECTION = 0, ORC_EULER = 1 };
enum { ORC_CENTRAL = 0, ORC_LLF = 1 };

typedef struct {
    int p, np, nq, nq1;
    double r1[ORC_MAXQ], r2[ORC_MAXQ], w[ORC_MAXQ]; /* w sums to 1/2 */
    double s1[ORC_MAXQ1], w1[ORC_MAXQ1];           /* Gauss points on [-1,1] */
    double phi[ORC_MAXNP * ORC_MAXQ];              /* phi_i(q)            [i*nq+q] */
    double gx[ORC_MAXNP * ORC_MAXQ];               /* w_q dphi_i/dr(q)    [i*nq+q] */
    double gy[ORC_MAXNP * ORC_MAXQ];               /* w_q dphi_i/ds(q)    [i*nq+q] */
    double side[3 * ORC_MAXNP * ORC_MAXQ1];        /* [side*np*nq1 + i*nq1 + j] */
    double vert[3 * ORC_MAXNP];                    /* [3*i + v] */
} orc_tables;

/* ------------------------------------------------------------------------- */
/* Quadrature                                                                 */
/* ------------------------------------------------------------------------- */

/* Symmetric triangle rules (Dunavant) written as orbits in barycentric form.
 * The reference stores the expanded point lists (src/2d/quadrature.cu:7-121);
 * the points, weights and point order produced here are the same.  Weights are
 * the reference's (sum 1) and are halved when tabulated (conserv.cu:94). */
typedef struct { int kind; double a, b, w; int order; } orc_orbit;
/* kind 0: centroid; kind 1: S21 (a, a, 1-2a) listed (1-2a,a),(a,1-2a),(a,a)
 * (order 0) or (a,a),(1-2a,a),(a,1-2a) (order 1);
 * kind 2: S111 (a, b, c=1-a-b) listed in the permutation given by `order`. */

static const int orc_perm111[4][6][2] = {
    /* entries index into (a,b,c) for (r,s) */
    {{2, 1}, {1, 2}, {2, 0}, {1, 0}, {0, 1}, {0, 2}}, /* degree-6 rule  */
    {{0, 2}, {2, 0}, {1, 0}, {0, 1}, {1, 2}, {2, 1}}, /* degree-8 rule  */
    {{0, 1}, {1, 0}, {1, 2}, {2, 1}, {2, 0}, {0, 2}}, /* degree-10 a    */
    {{0, 1}, {1, 0}, {0, 2}, {2, 0}, {2, 1}, {1, 2}}, /* degree-10 b    */
};

static int orc_rule2d(int p, double *r1, double *r2, double *w) {
    static const orc_orbit d1[] = {{0, 0, 0, 1.0, 0}};
    static const orc_orbit d2[] = {{1, 1.0 / 6.0, 0, 1.0 / 3.0, 1}};
    static const orc_orbit d4[] = {{1, 0.091576213509771, 0, 0.109951743655322, 0},
                                   {1, 0.445948490915965, 0, 0.223381589678011, 0}};
    static const orc_orbit d6[] = {{1, 0.063089014491502, 0, 0.050844906370207, 0},
                                   {1, 0.249286745170910, 0, 0.116786275726379, 0},
                                   {2, 0.053145049844816, 0.310352451033784, 0.082851075618374, 0}};
    static const orc_orbit d8[] = {{0, 0, 0, 0.144315607677787, 0},
                                   {1, 0.459292588292723, 0, 0.095091634267285, 0},
                                   {1, 0.170569307751760, 0, 0.103217370534718, 0},
                                   {1, 0.050547228317031, 0, 0.032458497623198, 0},
                                   {2, 0.008394777409958, 0.263112829634638, 0.027230314174435, 1}};
    static const orc_orbit d10[] = {{0, 0, 0, 0.090817990382754, 0},
                                    {1, 0.485577633383657, 0, 0.036725957756467, 0},
                                    {1, 0.109481575485037, 0, 0.045321059435528, 0},
                                    {2, 0.141707219414880, 0.307939838764121, 0.072757916845420, 2},
                                    {2, 0.025003534762686, 0.246672560639903, 0.028327242531057, 3},
                                    {2, 0.009540815400299, 0.066803251012200, 0.009421666963733, 2}};
    const orc_orbit *o;
    int no, n = 0, k, m;
    switch (p) {
    case 0: o = d1; no = 1; break;
    case 1: o = d2; no = 1; break;
    case 2: o = d4; no = 2; break;
    case 3: o = d6; no = 3; break;
    case 4: o = d8; no = 5; break;
    case 5: o = d10; no = 6; break;
    default: return -1;
    }
    for (k = 0; k < no; k++) {
        if (o[k].kind == 0) {
            r1[n] = 1.0 / 3.0; r2[n] = 1.0 / 3.0; w[n] = o[k].w; n++;
        } else if (o[k].kind == 1) {
            double a = o[k].a, c = 1.0 - 2.0 * a;
            if (o[k].order == 1) { r1[n] = a; r2[n] = a; w[n] = o[k].w; n++; }
            r1[n] = c; r2[n] = a; w[n] = o[k].w; n++;
            r1[n] = a; r2[n] = c; w[n] = o[k].w; n++;
            if (o[k].order == 0) { r1[n] = a; r2[n] = a; w[n] = o[k].w; n++; }
        } else {
            double abc[3];
            abc[0] = o[k].a; abc[1] = o[k].b; abc[2] = 1.0 - o[k].a - o[k].b;
            for (m = 0; m < 6; m++) {
                r1[n] = abc[orc_perm111[o[k].order][m][0]];
                r2[n] = abc[orc_perm111[o[k].order][m][1]];
                w[n] = o[k].w; n++;
            }
        }
    }
    return n;
}

/* Gauss-Legendre nodes (ascending) and weights by Newton iteration on P_n. */
static void orc_gauss(int n, double *x, double *w) {
    int i, it, k;
    for (i = 0; i < n; i++) {
        long double z = cosl(3.14159265358979323846264338327950288L * (n - i - 0.25L) / (n + 0.5L));
        long double dp = 1.0L;
        for (it = 0; it < 100; it++) {
            long double p0 = 1.0L, p1 = z, pk;
            for (k = 2; k <= n; k++) {
                pk = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
                p0 = p1; p1 = pk;
            }
            if (n == 1) { p1 = z; p0 = 1.0L; }
            dp = n * (z * p1 - p0) / (z * z - 1.0L);
            {
                long double dz = p1 / dp;
                z -= dz;
                if (fabsl(dz) < 1e-30L) break;
            }
        }
        {
            long double p0 = 1.0L, p1 = z, pk;
            for (k = 2; k <= n; k++) {
                pk = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
                p0 = p1; p1 = pk;
            }
            if (n == 1) { p1 = z; p0 = 1.0L; }
            dp = n * (z * p1 - p0) / (z * z - 1.0L);
        }
        x[i] = (double)z;
        w[i] = (double)(2.0L / ((1.0L - z * z) * dp * dp));
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

/* ------------------------------------------------------------------------- */
/* Orthonormal basis: Gram-Schmidt of graded-lex monomials r^(d-j) s^j       */
/* (src/2d/basis.cu:50-71 evaluates the same functions from a coefficient    */
/* table).  Computed here in extended precision by two passes of modified    */
/* Gram-Schmidt on centred monomials, which span the same nested spaces and  */
/* therefore give the same functions, with inner products taken by the       */
/* degree-2p rule (exact for products of degree <= 2p).                       */
/* ------------------------------------------------------------------------- */
static void orc_monomial(int k, long double r, long double s, long double *f, long double *fr,
                         long double *fs) {
    int d = 0, j, cnt = 0;
    while (cnt + d + 1 <= k) { cnt += d + 1; d++; }
    j = k - cnt;
    {
        long double x = r - 1.0L / 3.0L, y = s - 1.0L / 3.0L;
        int a = d - j, b = j;
        long double xa = 1.0L, yb = 1.0L, xa1 = 0.0L, yb1 = 0.0L;
        int t;
        for (t = 0; t < a; t++) xa *= x;
        for (t = 0; t < b; t++) yb *= y;
        if (a > 0) { xa1 = 1.0L; for (t = 0; t < a - 1; t++) xa1 *= x; xa1 *= a; }
        if (b > 0) { yb1 = 1.0L; for (t = 0; t < b - 1; t++) yb1 *= y; yb1 *= b; }
        *f = xa * yb;
        *fr = xa1 * yb;
        *fs = xa * yb1;
    }
}

int orc_tables_build(int p, orc_tables *T) {
    int np, nq, nq1, npts, i, j, l, pass;
    double s1[ORC_MAXQ1], w1[ORC_MAXQ1];
    /* evaluation points: volume (nq), sides (3*nq1), vertices (3) */
    long double pr[ORC_MAXQ + 3 * ORC_MAXQ1 + 3], ps[ORC_MAXQ + 3 * ORC_MAXQ1 + 3];
    long double F[ORC_MAXNP][ORC_MAXQ + 3 * ORC_MAXQ1 + 3];
    long double FR[ORC_MAXNP][ORC_MAXQ + 3 * ORC_MAXQ1 + 3];
    long double FS[ORC_MAXNP][ORC_MAXQ + 3 * ORC_MAXQ1 + 3];
    if (p < 0 || p > ORC_MAXP) return -1;
    memset(T, 0, sizeof(*T));
    np = (p + 1) * (p + 2) / 2;
    nq = orc_rule2d(p, T->r1, T->r2, T->w);
    nq1 = p + 1;
    orc_gauss(nq1, s1, w1);
    for (i = 0; i < nq; i++) T->w[i] *= 0.5;
    for (j = 0; j < nq1; j++) { T->s1[j] = s1[j]; T->w1[j] = w1[j]; }
    T->p = p; T->np = np; T->nq = nq; T->nq1 = nq1;

    npts = 0;
    for (j = 0; j < nq; j++) { pr[npts] = T->r1[j]; ps[npts] = T->r2[j]; npts++; }
    /* side points in the reference's orientation (basis.cu:192-196) */
    for (j = 0; j < nq1; j++) { pr[npts] = 0.5L + 0.5L * s1[j]; ps[npts] = 0.0L; npts++; }
    for (j = 0; j < nq1; j++) { pr[npts] = (1.0L - s1[j]) / 2.0L; ps[npts] = (1.0L + s1[j]) / 2.0L; npts++; }
    for (j = 0; j < nq1; j++) { pr[npts] = 0.0L; ps[npts] = 0.5L + 0.5L * s1[nq1 - 1 - j]; npts++; }
    pr[npts] = 0; ps[npts] = 0; npts++;
    pr[npts] = 1; ps[npts] = 0; npts++;
    pr[npts] = 0; ps[npts] = 1; npts++;

    for (i = 0; i < np; i++) {
        for (j = 0; j < npts; j++) orc_monomial(i, pr[j], ps[j], &F[i][j], &FR[i][j], &FS[i][j]);
        for (pass = 0; pass < 2; pass++) {
            for (l = 0; l < i; l++) {
                long double a = 0.0L;
                for (j = 0; j < nq; j++) a += (long double)T->w[j] * F[i][j] * F[l][j];
                for (j = 0; j < npts; j++) {
                    F[i][j] -= a * F[l][j];
                    FR[i][j] -= a * FR[l][j];
                    FS[i][j] -= a * FS[l][j];
                }
            }
        }
        {
            long double nrm = 0.0L;
            for (j = 0; j < nq; j++) nrm += (long double)T->w[j] * F[i][j] * F[i][j];
            nrm = sqrtl(nrm);
            for (j = 0; j < npts; j++) { F[i][j] /= nrm; FR[i][j] /= nrm; FS[i][j] /= nrm; }
        }
    }
    for (i = 0; i < np; i++) {
        for (j = 0; j < nq; j++) {
            T->phi[i * nq + j] = (double)F[i][j];
            T->gx[i * nq + j] = (double)((long double)T->w[j] * FR[i][j]);
            T->gy[i * nq + j] = (double)((long double)T->w[j] * FS[i][j]);
        }
        for (l = 0; l < 3; l++)
            for (j = 0; j < nq1; j++) T->side[l * np * nq1 + i * nq1 + j] = (double)F[i][nq + l * nq1 + j];
        for (l = 0; l < 3; l++) T->vert[3 * i + l] = (double)F[i][nq + 3 * nq1 + l];
    }
    return 0;
}

/* Flat export for tests. */
int orc_get_tables(int p, int *dims, double *r1, double *r2, double *w, double *s1, double *w1,
               double *phi, double *gx, double *gy, double *side, double *vert) {
    orc_tables T;
    if (orc_tables_build(p, &T)) return -1;
    dims[0] = T.np; dims[1] = T.nq; dims[2] = T.nq1;
    if (r1) memcpy(r1, T.r1, sizeof(double) * T.nq);
    if (r2) memcpy(r2, T.r2, sizeof(double) * T.nq);
    if (w) memcpy(w, T.w, sizeof(double) * T.nq);
    if (s1) memcpy(s1, T.s1, sizeof(double) * T.nq1);
    if (w1) memcpy(w1, T.w1, sizeof(double) * T.nq1);
    if (phi) memcpy(phi, T.phi, sizeof(double) * T.np * T.nq);
    if (gx) memcpy(gx, T.gx, sizeof(double) * T.np * T.nq);
    if (gy) memcpy(gy, T.gy, sizeof(double) * T.np * T.nq);
    if (side) memcpy(side, T.side, sizeof(double) * 3 * T.np * T.nq1);
    if (vert) memcpy(vert, T.vert, sizeof(double) * 3 * T.np);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Solver state                                                               */
/* ------------------------------------------------------------------------- */
typedef struct {
    int num_elem, num_sides, nv, eq, flux, ref_sqrtf;
    double gamma, ax, ay;
    orc_tables T;
    double *V[6];                      /* V1x V1y V2x V2y V3x V3y */
    int *elem_s[3], *left_elem, *right_elem, *left_side, *right_side;
    double *J, *xr, *yr, *xs, *ys, *len, *nx, *ny, *diam;
    double *left_rhs, *right_rhs, *quad_rhs;    /* [n][i][side] / [n][i][elem] */
    double *k[4], *kstar;
    double min_diam;
    /* boundary ghost states: 0 none (interior state), 1 free-stream state
     * (Euler inflow/outflow), 2 exact initial condition translated by a*t
     * (advection), 3 a problem's own ghost states (bc_ic = its IC) */
    int bc_kind, bc_ic;
    int integrator;       /* 0 RK4, 1 RK2 midpoint, 2 forward Euler */
    int ref_time;         /* 1: the reference's stage-time arguments */
    int limiter;          /* 1: orc_limit_p1 on every stage's output state */
    double bc_state[4], bc_params[8];
} orc_solver;

enum {
    ORC_IC_GAUSSIAN = 0,      /* u = exp(-((x-x0)^2 + (y-y0)^2) / w)          params x0 y0 w [Lx Ly] */
    ORC_IC_POLY = 1,          /* u = (x - y)^alpha                             params alpha */
    ORC_IC_DENSITY_WAVE = 2,  /* rho = 1 + A sin(2 pi k (x+y)), u, v, p const  params A u v p k */
    ORC_IC_VORTEX = 3,        /* isentropic vortex                             params x0 y0 beta uinf vinf Lx Ly */
    ORC_IC_CONSTANT = 4,      /* constant state                                params rho u v p (or u) */
    ORC_IC_CYLINDER = 5,      /* free stream rho = gamma, u = M, p = 1         params M */
    ORC_IC_SUPERSONIC = 6,    /* supersonic vortex between two arcs            params M A */
    ORC_IC_THREEPOINT = 7,    /* oblique shock state inside the angle theta    params M theta_deg */
    ORC_IC_LINEAR = 8,        /* u = c0 + cx x + cy y (advection u0 = x + y,   params c0 cx cy
                                 2dadvec/2dadvec_kernels.cu:176-178) */
};

/* the reference's problem files define PI as 3.14159 (threepoint.cu:13) */
#define ORC_REF_PI 3.14159

/* oblique shock state of the three-point problem (U_shock, threepoint.cu:27-32) */
static void orc_threepoint_shock(const double *P, double g, double *U) {
    double a = P[1] * ORC_REF_PI / 180.;
    U[0] = g;
    U[1] = P[0] * cos(a) * U[0];
    U[2] = P[0] * sin(a) * U[0];
    U[3] = 0.5 * U[0] * P[0] * P[0] + 1. / (g - 1.0);
}

void orc_ic_eval(int ic, const double *P, double g, double x, double y, double *U);

static double orc_fsqrt(const orc_solver *S, double x) {
    return S->ref_sqrtf ? (double)sqrtf((float)x) : sqrt(x);
}

/* length of the vector (dx, dy); the reference evaluates it as
 * sqrtf(powf(dx,2) + powf(dy,2)) in single precision. */
static double orc_len(const orc_solver *S, double dx, double dy) {
    if (S->ref_sqrtf) {
        float fx = (float)dx, fy = (float)dy;
        float a = powf(fx, 2.0f), b = powf(fy, 2.0f);
        return (double)sqrtf(a + b);
    }
    return sqrt(dx * dx + dy * dy);
}

static void orc_geometry_compute(orc_solver *S) {
    int e, s;
    double *V1x = S->V[0], *V1y = S->V[1], *V2x = S->V[2], *V2y = S->V[3], *V3x = S->V[4], *V3y = S->V[5];
    double mind = INFINITY;
#pragma omp parallel for schedule(static) reduction(min : mind)
    for (e = 0; e < S->num_elem; e++) {
        double x1 = V1x[e], y1 = V1y[e], x2 = V2x[e], y2 = V2y[e], x3 = V3x[e], y3 = V3y[e];
        double a, b, c, k;
        S->J[e] = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
        S->xr[e] = x2 - x1; S->yr[e] = y2 - y1;
        S->xs[e] = x3 - x1; S->ys[e] = y3 - y1;
        a = orc_len(S, x1 - x2, y1 - y2);
        b = orc_len(S, x2 - x3, y2 - y3);
        c = orc_len(S, x1 - x3, y1 - y3);
        k = 0.5 * (a + b + c);
        S->diam[e] = 2.0 * orc_fsqrt(S, k * (k - a) * (k - b) * (k - c)) / k;
        if (S->diam[e] < mind) mind = S->diam[e];
    }
    S->min_diam = mind;
#pragma omp parallel for schedule(static)
    for (s = 0; s < S->num_sides; s++) {
        int L = S->left_elem[s], ls = S->left_side[s];
        double px[3] = {V1x[L], V2x[L], V3x[L]}, py[3] = {V1y[L], V2y[L], V3y[L]};
        double ax_ = px[ls], ay_ = py[ls], bx = px[(ls + 1) % 3], by = py[(ls + 1) % 3];
        double tx = px[(ls + 2) % 3], ty = py[(ls + 2) % 3];
        double dx = bx - ax_, dy = by - ay_, l, nx, ny;
        l = orc_len(S, dx, dy);
        S->len[s] = l;
        nx = -dy / l; ny = dx / l;
        /* orient away from the left element's opposite vertex (conserv_kernels.cu:442-498) */
        if (nx * (tx - (ax_ + bx) / 2.0) + ny * (ty - (ay_ + by) / 2.0) > 0) { nx = -nx; ny = -ny; }
        S->nx[s] = nx; S->ny[s] = ny;
    }
}

void orc_destroy(orc_solver *S);

orc_solver *orc_create(int num_elem, int num_sides, const double *V1x, const double *V1y,
                       const double *V2x, const double *V2y, const double *V3x, const double *V3y,
                       const int *elem_s1, const int *elem_s2, const int *elem_s3,
                       const int *left_elem, const int *right_elem, const int *left_side,
                       const int *right_side, int p, int eq, int flux, double gamma, double ax,
                       double ay, int ref_sqrtf) {
    orc_solver *S = (orc_solver *)calloc(1, sizeof(orc_solver));
    int i, nv;
    size_t E = (size_t)num_elem, Sd = (size_t)num_sides;
    const double *Vin[6] = {V1x, V1y, V2x, V2y, V3x, V3y};
    const int *es[3] = {elem_s1, elem_s2, elem_s3};
    if (!S) return NULL;
    if (orc_tables_build(p, &S->T)) { free(S); return NULL; }
    nv = (eq == ORC_EULER) ? 4 : 1;
    S->num_elem = num_elem; S->num_sides = num_sides; S->nv = nv; S->eq = eq; S->flux = flux;
    S->gamma = gamma; S->ax = ax; S->ay = ay; S->ref_sqrtf = ref_sqrtf;
    for (i = 0; i < 6; i++) { S->V[i] = (double *)malloc(E * sizeof(double)); memcpy(S->V[i], Vin[i], E * sizeof(double)); }
    for (i = 0; i < 3; i++) { S->elem_s[i] = (int *)malloc(E * sizeof(int)); memcpy(S->elem_s[i], es[i], E * sizeof(int)); }
    S->left_elem = (int *)malloc(Sd * sizeof(int)); memcpy(S->left_elem, left_elem, Sd * sizeof(int));
    S->right_elem = (int *)malloc(Sd * sizeof(int)); memcpy(S->right_elem, right_elem, Sd * sizeof(int));
    S->left_side = (int *)malloc(Sd * sizeof(int)); memcpy(S->left_side, left_side, Sd * sizeof(int));
    S->right_side = (int *)malloc(Sd * sizeof(int)); memcpy(S->right_side, right_side, Sd * sizeof(int));
    S->J = (double *)malloc(E * sizeof(double));
    S->xr = (double *)malloc(E * sizeof(double)); S->yr = (double *)malloc(E * sizeof(double));
    S->xs = (double *)malloc(E * sizeof(double)); S->ys = (double *)malloc(E * sizeof(double));
    S->diam = (double *)malloc(E * sizeof(double));
    S->len = (double *)malloc(Sd * sizeof(double));
    S->nx = (double *)malloc(Sd * sizeof(double)); S->ny = (double *)malloc(Sd * sizeof(double));
    {
        size_t ns = (size_t)nv * S->T.np * Sd, ne = (size_t)nv * S->T.np * E;
        S->left_rhs = (double *)malloc(ns * sizeof(double));
        S->right_rhs = (double *)malloc(ns * sizeof(double));
        S->quad_rhs = (double *)malloc(ne * sizeof(double));
        for (i = 0; i < 4; i++) S->k[i] = (double *)malloc(ne * sizeof(double));
        S->kstar = (double *)malloc(ne * sizeof(double));
        if (!S->left_rhs || !S->right_rhs || !S->quad_rhs || !S->kstar || !S->k[3]) { orc_destroy(S); return NULL; }
    }
    orc_geometry_compute(S);
    return S;
}

void orc_destroy(orc_solver *S) {
    int i;
    if (!S) return;
    for (i = 0; i < 6; i++) free(S->V[i]);
    for (i = 0; i < 3; i++) free(S->elem_s[i]);
    free(S->left_elem); free(S->right_elem); free(S->left_side); free(S->right_side);
    free(S->J); free(S->xr); free(S->yr); free(S->xs); free(S->ys); free(S->diam);
    free(S->len); free(S->nx); free(S->ny);
    free(S->left_rhs); free(S->right_rhs); free(S->quad_rhs);
    for (i = 0; i < 4; i++) free(S->k[i]);
    free(S->kstar);
    free(S);
}

int orc_geometry(const orc_solver *S, double *J, double *xr, double *yr, double *xs, double *ys,
                 double *len, double *nx, double *ny, double *diam) {
    size_t E = (size_t)S->num_elem * sizeof(double), Sd = (size_t)S->num_sides * sizeof(double);
    if (J) memcpy(J, S->J, E);
    if (xr) memcpy(xr, S->xr, E);
    if (yr) memcpy(yr, S->yr, E);
    if (xs) memcpy(xs, S->xs, E);
    if (ys) memcpy(ys, S->ys, E);
    if (diam) memcpy(diam, S->diam, E);
    if (len) memcpy(len, S->len, Sd);
    if (nx) memcpy(nx, S->nx, Sd);
    if (ny) memcpy(ny, S->ny, Sd);
    return 0;
}

double orc_min_diameter(const orc_solver *S) { return S->min_diam; }

/* ------------------------------------------------------------------------- */
/* Physics                                                                    */
/* ------------------------------------------------------------------------- */
static void orc_euler_flux(double g, const double *U, double *fx, double *fy) {
    double rho = U[0], ru = U[1], rv = U[2], E = U[3];
    double p = (g - 1.) * (E - (ru * ru + rv * rv) / 2. / rho);
    fx[0] = ru;                 fy[0] = rv;
    fx[1] = ru * ru / rho + p;  fy[1] = ru * rv / rho;
    fx[2] = ru * rv / rho;      fy[2] = rv * rv / rho + p;
    fx[3] = ru * (E + p) / rho; fy[3] = rv * (E + p) / rho;
}

static double orc_sound(const orc_solver *S, const double *U) {
    double g = S->gamma;
    double p = (g - 1.) * (U[3] - (U[1] * U[1] + U[2] * U[2]) / 2. / U[0]);
    return orc_fsqrt(S, g * p / U[0]);
}

/* numerical flux Fhat . n at one Gauss point, n oriented out of the left element */
static void orc_num_flux(const orc_solver *S, const double *UL, const double *UR, double nx, double ny,
                         double *Fh) {
    if (S->eq == ORC_ADVECTION) {
        double an = S->ax * nx + S->ay * ny;
        if (S->flux == ORC_CENTRAL) Fh[0] = an * 0.5 * (UL[0] + UR[0]);
        else Fh[0] = 0.5 * (an * (UL[0] + UR[0]) + fabs(an) * (UL[0] - UR[0]));
    } else {
        double fxl[4], fyl[4], fxr[4], fyr[4], lam, sl, sr, ll, lr;
        int n;
        orc_euler_flux(S->gamma, UL, fxl, fyl);
        orc_euler_flux(S->gamma, UR, fxr, fyr);
        sl = nx * (UL[1] / UL[0]) + ny * (UL[2] / UL[0]);
        sr = nx * (UR[1] / UR[0]) + ny * (UR[2] / UR[0]);
        ll = fabs(sl) + orc_sound(S, UL);
        lr = fabs(sr) + orc_sound(S, UR);
        lam = (fabs(ll) > fabs(lr)) ? fabs(ll) : fabs(lr);
        if (S->flux == ORC_CENTRAL) lam = 0.0;
        for (n = 0; n < 4; n++)
            Fh[n] = 0.5 * ((fxl[n] + fxr[n]) * nx + (fyl[n] + fyr[n]) * ny + lam * (UL[n] - UR[n]));
    }
}

static void orc_phys_flux(const orc_solver *S, const double *U, double *fx, double *fy) {
    if (S->eq == ORC_ADVECTION) { fx[0] = S->ax * U[0]; fy[0] = S->ay * U[0]; }
    else orc_euler_flux(S->gamma, U, fx, fy);
}

/* Ghost state of a boundary side at its point j (the element is the side's
 * left element, n points out of the domain): Euler -1 reflecting keeps density
 * and energy and keeps the tangential momentum only (reflecting_boundary,
 * src/2d/conservation/euler/cylinder/cylinder.cu:58-111, with the side normal);
 * -2 outflow / -3 inflow take the free-stream state (U_outflow / U_inflow,
 * euler.cu:177-241) or the interior state; advection takes the initial
 * condition translated by a*t (boundary_exact, 2dadvec_kernels.cu:184-186) or
 * the interior state. */
/* point j of local side ls of element L: the point the reference's hooks map
 * from the element, x = V2 r + V3 s + V1 (1 - r - s) (inflow_boundary,
 * euler.cu:186-205), written along the side as Va + t (Vb - Va) with
 * t = (1 + s_j)/2 so that it lies on the side for any rounding */
static void orc_side_xy(const orc_solver *S, int L, int ls, int j, double *x, double *y) {
    int kb = ls == 2 ? 0 : ls + 1;
    double t = 0.5 + 0.5 * S->T.s1[j];
    double xa = S->V[2 * ls][L], ya = S->V[2 * ls + 1][L];
    *x = xa + t * (S->V[2 * kb][L] - xa);
    *y = ya + t * (S->V[2 * kb + 1][L] - ya);
}

/* Problem ghost states (DGX_BC_PROBLEM), the reference's problem hooks:
 *   cylinder    -1 tangential momentum about the radial direction from (0.5, 0.5)
 *                  (reflecting_boundary, cylinder.cu:58-111); -2/-3 the free stream
 *   supersonic  -1 the same about the origin (supersonic.cu:66-113); -2/-3 U0(x, y)
 *   three-point -1 flips the normal-facing momentum component (threepoint.cu:86-109);
 *               -2 the shock state; -3 the shock state left of the moving front
 *                  x < M t cos(theta) + tan(theta), else U0 (threepoint.cu:60-76)
 * The reference's radial reflections take their point from the mapping with
 * side 1's two coordinates exchanged (cylinder.cu:78-81), i.e. point
 * n_quad1d-1-j of side 1; kept alike. */
static void orc_problem_ghost(const orc_solver *S, int tag, int L, int ls, int j, double t,
                              const double *UL, double nx, double ny, double *UR) {
    const double *P = S->bc_params;
    double x, y;
    if (S->bc_ic == ORC_IC_THREEPOINT) {
        if (tag == -1) {
            UR[0] = UL[0]; UR[3] = UL[3];
            if ((float)(UL[1] * nx + UL[2] * ny) > 0.f) { UR[1] = -UL[1]; UR[2] = UL[2]; }
            else { UR[1] = UL[1]; UR[2] = -UL[2]; }
        } else if (tag == -2) {
            orc_threepoint_shock(P, S->gamma, UR);
        } else {
            double a = P[1] * ORC_REF_PI / 180.;
            orc_side_xy(S, L, ls, j, &x, &y);
            if (x < P[0] * t * cos(a) + tan(a)) orc_threepoint_shock(P, S->gamma, UR);
            else orc_ic_eval(ORC_IC_THREEPOINT, P, S->gamma, x, y, UR);
        }
        return;
    }
    if (tag == -1) {
        double cx = S->bc_ic == ORC_IC_CYLINDER ? 0.5 : 0.0, cy = cx, d, Nx, Ny, tm;
        orc_side_xy(S, L, ls, ls == 1 ? S->T.nq1 - 1 - j : j, &x, &y);
        x -= cx; y -= cy;
        d = sqrt(x * x + y * y);
        Nx = x / d; Ny = y / d;
        tm = UL[1] * Ny - UL[2] * Nx;
        UR[0] = UL[0]; UR[3] = UL[3];
        UR[1] = tm * Ny;
        UR[2] = -tm * Nx;
        return;
    }
    orc_side_xy(S, L, ls, j, &x, &y);
    orc_ic_eval(S->bc_ic, P, S->gamma, x, y, UR);
}

static void orc_ghost(const orc_solver *S, int tag, int L, int ls, int j, double t, const double *UL,
                      double nx, double ny, double *UR) {
    int n;
    if (S->eq == ORC_EULER && S->bc_kind == 3) {
        orc_problem_ghost(S, tag, L, ls, j, t, UL, nx, ny, UR);
        return;
    }
    if (S->eq == ORC_EULER) {
        if (tag == -1) {
            double mn = UL[1] * nx + UL[2] * ny;
            UR[0] = UL[0]; UR[1] = UL[1] - mn * nx; UR[2] = UL[2] - mn * ny; UR[3] = UL[3];
        } else if (S->bc_kind == 1) {
            for (n = 0; n < 4; n++) UR[n] = S->bc_state[n];
        } else {
            for (n = 0; n < 4; n++) UR[n] = UL[n];
        }
    } else if (S->bc_kind == 2) {
        double x, y, U[4];
        orc_side_xy(S, L, ls, j, &x, &y);
        orc_ic_eval(S->bc_ic, S->bc_params, S->gamma, x - S->ax * t, y - S->ay * t, U);
        UR[0] = U[0];
    } else {
        UR[0] = UL[0];
    }
}

int orc_set_boundary(orc_solver *S, int kind, int ic, const double *params) {
    int i;
    if (kind == 1) {
        double rho = params[0], u = params[1], v = params[2], p = params[3];
        S->bc_state[0] = rho; S->bc_state[1] = rho * u; S->bc_state[2] = rho * v;
        S->bc_state[3] = p / (S->gamma - 1.0) + 0.5 * rho * (u * u + v * v);
    } else if (kind == 2 || kind == 3) {
        if (kind == 3 && (ic < ORC_IC_CYLINDER || ic > ORC_IC_THREEPOINT)) return -1;
        S->bc_ic = ic;
        for (i = 0; i < 8; i++) S->bc_params[i] = params ? params[i] : 0.0;
    }
    S->bc_kind = kind;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* RHS: k = dt / J * (volume + sum of the three lifted edge fluxes)           */
/* ------------------------------------------------------------------------- */
int orc_rhs(orc_solver *S, const double *u, double *k, double dt, double t) {
    const orc_tables *T = &S->T;
    int np = T->np, nq = T->nq, nq1 = T->nq1, nv = S->nv;
    int E = S->num_elem, Sd = S->num_sides;
    int s, e, bad = 0;
    /* surface pass, one edge at a time (conserv_kernels.cu:697-758) */
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (s = 0; s < Sd; s++) {
        int L = S->left_elem[s], R = S->right_elem[s], ls = S->left_side[s], rs = S->right_side[s];
        double cL[ORC_MAXV][ORC_MAXNP], cR[ORC_MAXV][ORC_MAXNP];
        double Fh[ORC_MAXQ1][ORC_MAXV];
        int i, j, n;
        for (n = 0; n < nv; n++)
            for (i = 0; i < np; i++) {
                cL[n][i] = u[(size_t)E * np * n + (size_t)i * E + L];
                cR[n][i] = R >= 0 ? u[(size_t)E * np * n + (size_t)i * E + R] : 0.0;
            }
        for (j = 0; j < nq1; j++) {
            double UL[ORC_MAXV] = {0}, UR[ORC_MAXV] = {0};
            for (i = 0; i < np; i++)
                for (n = 0; n < nv; n++) {
                    UL[n] += cL[n][i] * T->side[ls * np * nq1 + i * nq1 + j];
                    if (R >= 0) UR[n] += cR[n][i] * T->side[rs * np * nq1 + i * nq1 + nq1 - j - 1];
                }
            if (R < 0) orc_ghost(S, R, L, ls, j, t, UL, S->nx[s], S->ny[s], UR);
            orc_num_flux(S, UL, UR, S->nx[s], S->ny[s], Fh[j]);
        }
        for (i = 0; i < np; i++)
            for (n = 0; n < nv; n++) {
                double sl = 0., sr = 0.;
                for (j = 0; j < nq1; j++) {
                    sl += T->w1[j] * Fh[j][n] * T->side[ls * np * nq1 + i * nq1 + j];
                    sr += T->w1[j] * Fh[j][n] * T->side[rs * np * nq1 + i * nq1 + nq1 - 1 - j];
                }
                S->left_rhs[(size_t)Sd * np * n + (size_t)i * Sd + s] = -S->len[s] / 2. * sl;
                S->right_rhs[(size_t)Sd * np * n + (size_t)i * Sd + s] = S->len[s] / 2. * sr;
            }
    }
    if (bad) return -2;
    /* volume pass, one element at a time (conserv_kernels.cu:766-811) */
#pragma omp parallel for schedule(static)
    for (e = 0; e < E; e++) {
        double c[ORC_MAXV][ORC_MAXNP], fx[ORC_MAXQ][ORC_MAXV], fy[ORC_MAXQ][ORC_MAXV];
        double xr = S->xr[e], yr = S->yr[e], xs = S->xs[e], ys = S->ys[e];
        int i, j, n, kk;
        for (n = 0; n < nv; n++)
            for (i = 0; i < np; i++) c[n][i] = u[(size_t)E * np * n + (size_t)i * E + e];
        for (j = 0; j < nq; j++) {
            double U[ORC_MAXV] = {0};
            for (kk = 0; kk < np; kk++)
                for (n = 0; n < nv; n++) U[n] += c[n][kk] * T->phi[nq * kk + j];
            orc_phys_flux(S, U, fx[j], fy[j]);
        }
        for (i = 0; i < np; i++)
            for (n = 0; n < nv; n++) {
                double sum = 0.;
                for (j = 0; j < nq; j++)
                    sum += fx[j][n] * (T->gx[nq * i + j] * ys - T->gy[nq * i + j] * yr) +
                           fy[j][n] * (-T->gx[nq * i + j] * xs + T->gy[nq * i + j] * xr);
                S->quad_rhs[(size_t)E * np * n + (size_t)i * E + e] = sum;
            }
    }
    /* assembly with the mass inverse 1/J (time_integrator.cu:130-188) */
#pragma omp parallel for schedule(static)
    for (e = 0; e < E; e++) {
        int sid[3] = {S->elem_s[0][e], S->elem_s[1][e], S->elem_s[2][e]};
        double j_ = S->J[e];
        int i, n, q;
        for (i = 0; i < np; i++)
            for (n = 0; n < nv; n++) {
                double sum = S->quad_rhs[(size_t)E * np * n + (size_t)i * E + e];
                double add[3];
                for (q = 0; q < 3; q++) {
                    size_t o = (size_t)Sd * np * n + (size_t)i * Sd + sid[q];
                    add[q] = (e == S->left_elem[sid[q]]) ? S->left_rhs[o] : S->right_rhs[o];
                }
                k[(size_t)E * np * n + (size_t)i * E + e] = 1. / j_ * dt * (sum + add[0] + add[1] + add[2]);
            }
    }
    return 0;
}

/* maximum wave speed from the cell averages (euler.cu:252-278) */
double orc_max_lambda(const orc_solver *S, const double *c) {
    int E = S->num_elem, np = S->T.np, e;
    double phi0 = S->T.phi[0], mx = 0.0;
    if (S->eq == ORC_ADVECTION) return sqrt(S->ax * S->ax + S->ay * S->ay);
#pragma omp parallel for schedule(static) reduction(max : mx)
    for (e = 0; e < E; e++) {
        double U[4], cs, sp, lam;
        int n;
        for (n = 0; n < 4; n++) U[n] = c[(size_t)E * np * n + e] * phi0;
        cs = orc_sound(S, U);
        sp = orc_fsqrt(S, U[1] * U[1] + U[2] * U[2]) / U[0];
        lam = (sp > 0) ? sp + cs : -sp + cs;
        if (lam > mx) mx = lam;
    }
    return mx;
}

/* dt = cfl * min inscribed diameter / max lambda / (2p+1) (time_integrator.cu:263) */
double orc_cfl_dt(const orc_solver *S, const double *c, double cfl) {
    return cfl * S->min_diam / orc_max_lambda(S, c) / (2. * S->T.p + 1.);
}

/* Time integrator and stage-time rule.  Stage s of a step from t_n takes its
 * boundary data at t_n + c_s dt; with ref_time the reference's arguments
 * instead: Euler RK4/RK2 pass t_{n+1} + c_s dt (time_integrator.cu:264-380,
 * :509-561), Euler forward Euler and every advection stage pass t_n
 * (time_integrator.cu:733; src/2d/time_integrator.cu:145). */
int orc_set_integrator(orc_solver *S, int integrator, int ref_time) {
    if (integrator < 0 || integrator > 2) return -1;
    S->integrator = integrator;
    S->ref_time = ref_time ? 1 : 0;
    return 0;
}

static double orc_stage_time(const orc_solver *S, double t, double dt, double node) {
    if (!S->ref_time) return t + node * dt;
    if (S->eq == ORC_EULER && S->integrator != 2) return (t + dt) + node * dt;
    return t;
}

/* p = 1 slope limiter in place, Barth-Jespersen form of the reference's
 * limit_c (conserv_kernels.cu:522-621; its bounds umin/umax are never set and
 * its calls are commented out, time_integrator.cu:302,332,363): per element
 * and variable, the linear modes are scaled by min over the 6 side Gauss
 * points of min(1, (M - u0)/(u_j - u0)) (u_j > u0) or min(1, (m - u0)/(u_j -
 * u0)) (u_j < u0), m/M the extremes of the cell averages of the element and
 * its neighbours (a boundary side: the element itself). */
int orc_limit_p1(const orc_solver *S, double *c) {
    const orc_tables *T = &S->T;
    int E = S->num_elem, e;
    if (T->p != 1) return -1;
#pragma omp parallel for schedule(static)
    for (e = 0; e < E; e++) {
        int nb[3], k, n, j;
        for (k = 0; k < 3; k++) {
            int s = S->elem_s[k][e], le = S->left_elem[s], re = S->right_elem[s];
            int other = le == e ? re : le;
            nb[k] = other >= 0 ? other : e;
        }
        for (n = 0; n < S->nv; n++) {
            double *cn = c + (size_t)n * 3 * E;
            double c0 = cn[e], c1 = cn[E + e], c2 = cn[2 * E + e];
            double u0 = c0 * T->phi[0], lo = u0, hi = u0, phi = 1.0;
            for (k = 0; k < 3; k++) {
                double un = cn[nb[k]] * T->phi[0];
                lo = fmin(lo, un);
                hi = fmax(hi, un);
            }
            for (k = 0; k < 3; k++)
                for (j = 0; j < 2; j++) {
                    double uj = c0 * T->side[(k * 3 + 0) * 2 + j] + c1 * T->side[(k * 3 + 1) * 2 + j] +
                                c2 * T->side[(k * 3 + 2) * 2 + j];
                    double d = uj - u0, pj = 1.0;
                    if (d > 0.0) pj = fmin(1.0, (hi - u0) / d);
                    else if (d < 0.0) pj = fmin(1.0, (lo - u0) / d);
                    phi = fmin(phi, pj);
                }
            if (phi < 1.0) { cn[E + e] = c1 * phi; cn[2 * E + e] = c2 * phi; }
        }
    }
    return 0;
}

int orc_set_limiter(orc_solver *S, int on) {
    if (on && S->T.p != 1) return -1;
    S->limiter = on ? 1 : 0;
    return 0;
}

/* one classic RK4 step in the reference's form (time_integrator.cu:276-398) */
int orc_rk4_step(orc_solver *S, double *c, double dt, double t) {
    size_t N = (size_t)S->nv * S->T.np * S->num_elem, i;
    static const double alpha[3] = {0.5, 0.5, 1.0};
    static const double tfrac[4] = {0.0, 0.5, 0.5, 1.0};
    int st, rc;
    const double *src = c;
    for (st = 0; st < 4; st++) {
        rc = orc_rhs(S, src, S->k[st], dt, orc_stage_time(S, t, dt, tfrac[st]));
        if (rc) return rc;
        if (st < 3) {
            double a = alpha[st];
            double *ks = S->kstar, *kk = S->k[st];
#pragma omp parallel for schedule(static)
            for (i = 0; i < N; i++) ks[i] = c[i] + a * kk[i];
            if (S->limiter) orc_limit_p1(S, S->kstar);
            src = S->kstar;
        }
    }
    {
        double *k1 = S->k[0], *k2 = S->k[1], *k3 = S->k[2], *k4 = S->k[3];
#pragma omp parallel for schedule(static)
        for (i = 0; i < N; i++) c[i] += k1[i] / 6. + k2[i] / 3. + k3[i] / 3. + k4[i] / 6.;
    }
    if (S->limiter) orc_limit_p1(S, c);
    return 0;
}

/* one explicit-midpoint step: k1 = k(c), k* = c + k1/2, c += k(k*)
 * (rk2_tempstorage / rk2 in time_integrate_rk2, time_integrator.cu:445-464,
 * 518-580) */
int orc_rk2_step(orc_solver *S, double *c, double dt, double t) {
    size_t N = (size_t)S->nv * S->T.np * S->num_elem, i;
    int rc = orc_rhs(S, c, S->k[0], dt, orc_stage_time(S, t, dt, 0.0));
    if (rc) return rc;
    {
        double *ks = S->kstar, *k1 = S->k[0];
#pragma omp parallel for schedule(static)
        for (i = 0; i < N; i++) ks[i] = c[i] + 0.5 * k1[i];
    }
    if (S->limiter) orc_limit_p1(S, S->kstar);
    rc = orc_rhs(S, S->kstar, S->k[1], dt, orc_stage_time(S, t, dt, 0.5));
    if (rc) return rc;
    {
        double *k2 = S->k[1];
#pragma omp parallel for schedule(static)
        for (i = 0; i < N; i++) c[i] += k2[i];
    }
    if (S->limiter) orc_limit_p1(S, c);
    return 0;
}

/* one forward-Euler step: c += dt/J (volume + surface) (eval_rhs_fe,
 * time_integrator.cu:622-700) */
int orc_fe_step(orc_solver *S, double *c, double dt, double t) {
    size_t N = (size_t)S->nv * S->T.np * S->num_elem, i;
    int rc = orc_rhs(S, c, S->k[0], dt, orc_stage_time(S, t, dt, 0.0));
    if (rc) return rc;
    {
        double *k1 = S->k[0];
#pragma omp parallel for schedule(static)
        for (i = 0; i < N; i++) c[i] += k1[i];
    }
    if (S->limiter) orc_limit_p1(S, c);
    return 0;
}

/* one step of the solver's integrator from time t */
int orc_step(orc_solver *S, double *c, double dt, double t) {
    if (S->integrator == 1) return orc_rk2_step(S, c, dt, t);
    if (S->integrator == 2) return orc_fe_step(S, c, dt, t);
    return orc_rk4_step(S, c, dt, t);
}

/* Run to t_end (dt_mode 0: fixed dt, 1: reference CFL rule with factor `cfl`),
 * clipping the last step to land on t_end (time_integrator.cu:263-270), or at
 * most max_steps steps when max_steps > 0.  Returns the number of steps. */
int orc_run(orc_solver *S, double *c, int dt_mode, double dt_fixed, double cfl, double t_end,
            int max_steps, double *t_out) {
    double t = 0.0;
    int steps = 0, rc;
    while (t < t_end && (max_steps <= 0 || steps < max_steps)) {
        double dt = dt_mode ? orc_cfl_dt(S, c, cfl) : dt_fixed;
        double t0 = t;
        if (t + dt > t_end) { dt = t_end - t; t = t_end; }
        else t += dt;
        rc = orc_step(S, c, dt, t0);
        if (rc) return rc;
        steps++;
    }
    if (t_out) *t_out = t;
    return steps;
}

/* ------------------------------------------------------------------------- */
/* Initial conditions: L2 projection with the degree-2p rule (no mass solve,  */
/* the basis is orthonormal on the reference triangle)                        */
/* ------------------------------------------------------------------------- */

static double orc_wrap(double d, double L) {
    if (L > 0) { d = fmod(d, L); if (d > 0.5 * L) d -= L; if (d < -0.5 * L) d += L; }
    return d;
}

void orc_ic_eval(int ic, const double *P, double g, double x, double y, double *U) {
    const double pi = 3.14159265358979323846;
    switch (ic) {
    case ORC_IC_GAUSSIAN: {
        double dx = orc_wrap(x - P[0], P[3]), dy = orc_wrap(y - P[1], P[4]);
        U[0] = exp(-(dx * dx + dy * dy) / P[2]);
        break;
    }
    case ORC_IC_POLY: U[0] = pow(x - y, P[0]); break;
    case ORC_IC_LINEAR: U[0] = P[0] + P[1] * x + P[2] * y; break;
    case ORC_IC_DENSITY_WAVE: {
        double rho = 1.0 + P[0] * sin(2.0 * pi * P[4] * (x + y));
        U[0] = rho; U[1] = rho * P[1]; U[2] = rho * P[2];
        U[3] = P[3] / (g - 1.0) + 0.5 * rho * (P[1] * P[1] + P[2] * P[2]);
        break;
    }
    case ORC_IC_VORTEX: {
        double dx = orc_wrap(x - P[0], P[5]), dy = orc_wrap(y - P[1], P[6]);
        double r2 = dx * dx + dy * dy, b = P[2];
        double du = -b / (2.0 * pi) * exp(0.5 * (1.0 - r2)) * dy;
        double dv = b / (2.0 * pi) * exp(0.5 * (1.0 - r2)) * dx;
        double T = 1.0 - (g - 1.0) * b * b / (8.0 * g * pi * pi) * exp(1.0 - r2);
        double rho = pow(T, 1.0 / (g - 1.0)), p = pow(rho, g);
        double u = P[3] + du, v = P[4] + dv;
        U[0] = rho; U[1] = rho * u; U[2] = rho * v; U[3] = p / (g - 1.0) + 0.5 * rho * (u * u + v * v);
        break;
    }
    case ORC_IC_CYLINDER:   /* U0, cylinder.cu:26-31 */
        U[0] = g; U[1] = U[0] * P[0]; U[2] = 0.0;
        U[3] = 0.5 * U[0] * P[0] * P[0] + 1. / (g - 1.0);
        break;
    case ORC_IC_SUPERSONIC: {   /* U0, supersonic.cu:26-37 (powf there, pow here) */
        double r = sqrt(x * x + y * y), th = atan(y / x);
        double A = P[1] != 0.0 ? P[1] : 0.5 * (g - 1.0) * P[0] * P[0];
        double p;
        U[0] = pow(1 + A * (1. - 1. / (r * r)), 2.5);
        U[1] = U[0] * sin(th) * P[0] / r;
        U[2] = U[0] * -cos(th) * P[0] / r;
        p = (1.0 / g) * pow(U[0], g);
        U[3] = 0.5 * U[0] * (P[0] * P[0] / (r * r)) + p * (1. / (g - 1.));
        break;
    }
    case ORC_IC_THREEPOINT: {   /* U0, threepoint.cu:44-54 */
        double angle = atan(x / y);
        if (angle < P[1] * ORC_REF_PI / 180) {
            orc_threepoint_shock(P, g, U);
        } else {
            U[0] = 0.5 * g; U[1] = 0.; U[2] = 0.;
            U[3] = 0.5 * U[0] * P[0] * P[0] + 1. / (g - 1.0);
        }
        break;
    }
    case ORC_IC_CONSTANT:
    default:
        U[0] = P[0]; U[1] = P[0] * P[1]; U[2] = P[0] * P[2];
        U[3] = P[3] / (g - 1.0) + 0.5 * P[0] * (P[1] * P[1] + P[2] * P[2]);
        break;
    }
}

int orc_project(const orc_solver *S, int ic, const double *params, double *c) {
    const orc_tables *T = &S->T;
    int E = S->num_elem, np = T->np, nq = T->nq, nv = S->nv, e;
    double P[8] = {0};
    int i;
    for (i = 0; i < 8; i++) P[i] = params ? params[i] : 0.0;
#pragma omp parallel for schedule(static)
    for (e = 0; e < E; e++) {
        double v1x = S->V[0][e], v1y = S->V[1][e], v2x = S->V[2][e], v2y = S->V[3][e];
        double v3x = S->V[4][e], v3y = S->V[5][e];
        double U0[ORC_MAXQ][ORC_MAXV];
        int j, ii, n;
        for (j = 0; j < nq; j++) {
            double r = T->r1[j], s = T->r2[j];
            double x = r * v2x + s * v3x + (1 - r - s) * v1x;
            double y = r * v2y + s * v3y + (1 - r - s) * v1y;
            orc_ic_eval(ic, P, S->gamma, x, y, U0[j]);
        }
        for (ii = 0; ii < np; ii++)
            for (n = 0; n < nv; n++) {
                double acc = 0.;
                for (j = 0; j < nq; j++) acc += T->w[j] * U0[j][n] * T->phi[ii * nq + j];
                c[(size_t)E * np * n + (size_t)ii * E + e] = acc;
            }
    }
    return 0;
}

/* conserved totals  int u dx = sum_e c_{n,0,e} * phi_0 * |J_e| / 2 */
int orc_totals(const orc_solver *S, const double *c, double *out) {
    int E = S->num_elem, np = S->T.np, n;
    for (n = 0; n < S->nv; n++) {
        double acc = 0.0;
        int e;
#pragma omp parallel for schedule(static) reduction(+ : acc)
        for (e = 0; e < E; e++) acc += c[(size_t)E * np * n + e] * S->J[e];
        out[n] = acc * S->T.phi[0] * 0.5;
    }
    return 0;
}

int orc_num_vars(const orc_solver *S) { return S->nv; }
int orc_num_modes(const orc_solver *S) { return S->T.np; }

int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}
