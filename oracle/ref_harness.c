/*
 * ref_harness.c -- drives the reference's own CPU Euler loops on our inputs.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile (target `ref`) directly
 * from the reference sources where they lie (src/2d/conservation/euler/cpu/,
 * which `#include`s its own kernels, integrator, quadrature and basis); the
 * binary goes to oracle/_ref/ and is used only to generate and check golden
 * vectors (tests/golden/make_golden.py).  No reference source is copied here.
 *
 * The reference's own read_mesh (euler.c:93-287) expects an older mesh format
 * and its driver hard-codes the initial condition (euler_kernels.c:162-184), so
 * this harness fills the reference's host globals directly, as
 * src/2d/conservation/euler/cpu/main.c does after reading a mesh, and then
 * calls the reference's precompute (euler_kernels.c:367-555), basis
 * (basis.c:150-237), surface (euler_kernels.c:823-984), volume (:986-1104),
 * eval_rhs_rk4 (time_integrator_euler.c:68-136), rk4_tempstorage and rk4
 * (time_integrator_euler.c:19-41) in the order of time_integrate_rk4
 * (time_integrator_euler.c:138-287) with a fixed dt; then, from the same
 * initial state, forward-Euler steps through eval_rhs_fe
 * (time_integrator_euler.c:289-356) in the order of time_integrate_fe
 * (:359-406), also with a fixed dt.
 *
 * Input file (little-endian): int32[8] {num_elem, num_sides, p, nsteps, fe_steps, timed, 0...},
 * float64 dt, float64 V1x..V3y[E] (6 arrays), int32 elem_s1..3[E],
 * int32 left_elem, right_elem, left_side, right_side [S], float64 c0[4*Np*E].
 * Output file: see write order in main() below; with `timed` set, the wall
 * time of the RK4 steps (double, seconds) closes it.
 */
#include <time.h>
#include "euler.c"

static void *xread(FILE *f, size_t n) {
    void *p = malloc(n ? n : 1);
    if (fread(p, 1, n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
    return p;
}

static void xwrite(FILE *f, const void *p, size_t n) {
    if (fwrite(p, 1, n, f) != n) { fprintf(stderr, "short write\n"); exit(3); }
}

int main(int argc, char *argv[]) {
    FILE *in, *out;
    int hdr[8], E, S, n, n_p, nsteps, fe_steps, timed, i, step;
    struct timespec ts0, ts1;
    double rk4_seconds;
    double dt;
    double *V[6];
    int *es[3], *le, *re, *lsn, *rsn;
    double *sx1, *sy1, *sx2, *sy2, *c0, *radii;
    double *r1_local, *r2_local, *w_local, *s_r, *oned_w_local;
    int n_quad, n_quad1d;
    size_t NV;

    if (argc != 3) { fprintf(stderr, "usage: ref_euler in.bin out.bin\n"); return 1; }
    in = fopen(argv[1], "rb");
    if (!in) return 1;
    if (fread(hdr, sizeof(int), 8, in) != 8) return 2;
    E = hdr[0]; S = hdr[1]; n = hdr[2]; nsteps = hdr[3]; fe_steps = hdr[4]; timed = hdr[5];
    n_p = (n + 1) * (n + 2) / 2;
    if (fread(&dt, sizeof(double), 1, in) != 1) return 2;
    for (i = 0; i < 6; i++) V[i] = (double *)xread(in, sizeof(double) * E);
    for (i = 0; i < 3; i++) es[i] = (int *)xread(in, sizeof(int) * E);
    le = (int *)xread(in, sizeof(int) * S);
    re = (int *)xread(in, sizeof(int) * S);
    lsn = (int *)xread(in, sizeof(int) * S);
    rsn = (int *)xread(in, sizeof(int) * S);
    NV = (size_t)4 * n_p * E;
    c0 = (double *)xread(in, sizeof(double) * NV);
    fclose(in);

    /* side end points from the left element's local side (genmesh.py:290-308) */
    sx1 = malloc(sizeof(double) * S); sy1 = malloc(sizeof(double) * S);
    sx2 = malloc(sizeof(double) * S); sy2 = malloc(sizeof(double) * S);
    for (i = 0; i < S; i++) {
        int L = le[i], a = lsn[i], b = (lsn[i] + 1) % 3;
        double px[3] = {V[0][L], V[2][L], V[4][L]}, py[3] = {V[1][L], V[3][L], V[5][L]};
        sx1[i] = px[a]; sy1[i] = py[a]; sx2[i] = px[b]; sy2[i] = py[b];
    }

    set_quadrature(n, &r1_local, &r2_local, &w_local, &s_r, &oned_w_local, &n_quad, &n_quad1d);
    preval_basis(r1_local, r2_local, s_r, w_local, oned_w_local, n_quad, n_quad1d, n_p);
    init_gpu(E, S, n_p, V[0], V[1], V[2], V[3], V[4], V[5], lsn, rsn, sx1, sy1, sx2, sy2,
             es[0], es[1], es[2], le, re);

    preval_side_length(d_s_length, d_s_V1x, d_s_V1y, d_s_V2x, d_s_V2y, S);
    preval_inscribed_circles(d_J, d_V1x, d_V1y, d_V2x, d_V2y, d_V3x, d_V3y, E);
    radii = malloc(sizeof(double) * E);
    memcpy(radii, d_J, sizeof(double) * E);
    preval_jacobian(d_J, d_V1x, d_V1y, d_V2x, d_V2y, d_V3x, d_V3y, E);
    preval_normals(d_Nx, d_Ny, d_s_V1x, d_s_V1y, d_s_V2x, d_s_V2y, d_V1x, d_V1y, d_V2x, d_V2y,
                   d_V3x, d_V3y, d_left_side_number, S);
    preval_normals_direction(d_Nx, d_Ny, d_V1x, d_V1y, d_V2x, d_V2y, d_V3x, d_V3y, d_left_elem,
                             d_left_side_number, S);
    preval_partials(d_V1x, d_V1y, d_V2x, d_V2y, d_V3x, d_V3y, d_xr, d_yr, d_xs, d_ys, E);

    memcpy(d_c, c0, sizeof(double) * NV);

    out = fopen(argv[2], "wb");
    if (!out) return 1;
    {
        int dims[4] = {n_p, n_quad, n_quad1d, 0};
        xwrite(out, dims, sizeof(dims));
    }
    xwrite(out, r1_local, sizeof(double) * n_quad);
    xwrite(out, r2_local, sizeof(double) * n_quad);
    xwrite(out, w_local, sizeof(double) * n_quad);
    xwrite(out, s_r, sizeof(double) * n_quad1d);
    xwrite(out, oned_w_local, sizeof(double) * n_quad1d);
    xwrite(out, basis, sizeof(double) * n_p * n_quad);
    xwrite(out, basis_grad_x, sizeof(double) * n_p * n_quad);
    xwrite(out, basis_grad_y, sizeof(double) * n_p * n_quad);
    xwrite(out, basis_side, sizeof(double) * 3 * n_p * n_quad1d);
    xwrite(out, basis_vertex, sizeof(double) * 3 * n_p);
    xwrite(out, d_J, sizeof(double) * E);
    xwrite(out, d_xr, sizeof(double) * E);
    xwrite(out, d_yr, sizeof(double) * E);
    xwrite(out, d_xs, sizeof(double) * E);
    xwrite(out, d_ys, sizeof(double) * E);
    xwrite(out, radii, sizeof(double) * E);
    xwrite(out, d_s_length, sizeof(double) * S);
    xwrite(out, d_Nx, sizeof(double) * S);
    xwrite(out, d_Ny, sizeof(double) * S);

    eval_global_lambda(d_c, d_lambda, n_quad, n_p, E);
    xwrite(out, d_lambda, sizeof(double) * E);

    /* one RHS evaluation with dt = 1 */
    eval_surface(d_c, d_left_riemann_rhs, d_right_riemann_rhs, d_s_length, d_V1x, d_V1y, d_V2x,
                 d_V2y, d_V3x, d_V3y, d_left_elem, d_right_elem, d_left_side_number,
                 d_right_side_number, d_Nx, d_Ny, n_quad1d, n_quad, n_p, S, E, 0.0);
    eval_volume(d_c, d_quad_rhs, d_xr, d_yr, d_xs, d_ys, n_quad, n_p, E);
    eval_rhs_rk4(d_k1, d_quad_rhs, d_left_riemann_rhs, d_right_riemann_rhs, d_elem_s1, d_elem_s2,
                 d_elem_s3, d_left_elem, d_J, 1.0, n_p, S, E);
    xwrite(out, d_k1, sizeof(double) * NV);

    /* nsteps classic RK4 steps with a fixed dt, stage order of time_integrate_rk4 */
    clock_gettime(CLOCK_MONOTONIC, &ts0);
    for (step = 0; step < nsteps; step++) {
        double *ks[4] = {d_k1, d_k2, d_k3, d_k4};
        double alpha[3] = {0.5, 0.5, 1.0};
        int st;
        for (st = 0; st < 4; st++) {
            double *src = (st == 0) ? d_c : d_kstar;
            eval_surface(src, d_left_riemann_rhs, d_right_riemann_rhs, d_s_length, d_V1x, d_V1y,
                         d_V2x, d_V2y, d_V3x, d_V3y, d_left_elem, d_right_elem, d_left_side_number,
                         d_right_side_number, d_Nx, d_Ny, n_quad1d, n_quad, n_p, S, E, 0.0);
            eval_volume(src, d_quad_rhs, d_xr, d_yr, d_xs, d_ys, n_quad, n_p, E);
            eval_rhs_rk4(ks[st], d_quad_rhs, d_left_riemann_rhs, d_right_riemann_rhs, d_elem_s1,
                         d_elem_s2, d_elem_s3, d_left_elem, d_J, dt, n_p, S, E);
            if (st < 3) rk4_tempstorage(d_c, d_kstar, ks[st], alpha[st], n_p, E);
        }
        rk4(d_c, d_k1, d_k2, d_k3, d_k4, n_p, E);
    }
    clock_gettime(CLOCK_MONOTONIC, &ts1);
    rk4_seconds = (double)(ts1.tv_sec - ts0.tv_sec) + 1e-9 * (double)(ts1.tv_nsec - ts0.tv_nsec);
    xwrite(out, d_c, sizeof(double) * NV);

    /* fe_steps forward-Euler steps from the initial state */
    if (fe_steps > 0) {
        memcpy(d_c, c0, sizeof(double) * NV);
        for (step = 0; step < fe_steps; step++) {
            eval_surface(d_c, d_left_riemann_rhs, d_right_riemann_rhs, d_s_length, d_V1x, d_V1y,
                         d_V2x, d_V2y, d_V3x, d_V3y, d_left_elem, d_right_elem, d_left_side_number,
                         d_right_side_number, d_Nx, d_Ny, n_quad1d, n_quad, n_p, S, E, 0.0);
            eval_volume(d_c, d_quad_rhs, d_xr, d_yr, d_xs, d_ys, n_quad, n_p, E);
            eval_rhs_fe(d_c, d_quad_rhs, d_left_riemann_rhs, d_right_riemann_rhs, d_elem_s1,
                        d_elem_s2, d_elem_s3, d_left_elem, d_J, dt, n_p, S, E);
        }
        xwrite(out, d_c, sizeof(double) * NV);
    }
    if (timed) xwrite(out, &rk4_seconds, sizeof(rk4_seconds));
    fclose(out);
    return 0;
}
