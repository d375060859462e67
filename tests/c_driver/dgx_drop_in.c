/* dgx_drop_in.c -- the reference-side binding of the library, as a driver of
 * the reference would add it, written as a plain C program (test
 * infrastructure: built and run by tests/test_gpu_c_driver.py).
 *
 * It does what the reference's run_dgcuda does around its time loop
 * (src/2d/conservation/main.cu:54-209) with the library in place of init_gpu's
 * geometry kernels and time_integrate_rk4/rk2: read a .pmsh mesh, create the
 * mesh and the solver, project the initial state, run to the end time with
 * the reference's CFL rule, and write the final coefficients in the
 * reference layout c[n][i][e].
 *
 * usage: dgx_drop_in mesh.pmsh order rk2(0|1) precision(0 FP32, 2 FP64)
 *                    ic(dgx_ic) bc(dgx_bc) t_end out.bin [param ...]
 * out.bin: int32 steps, int32 num_vars, int32 n_p, int32 num_elem, double t,
 *          double c[num_vars][n_p][num_elem]
 */
#include <stdio.h>
#include <stdlib.h>

#include "dgx.h"

#define CHECK(call)                                                              \
    do {                                                                         \
        int rc_ = (call);                                                        \
        if (rc_ != DGX_OK) {                                                     \
            fprintf(stderr, "%s: %s (%s)\n", #call, dgx_status_string(rc_),      \
                    dgx_last_error());                                           \
            return 1;                                                            \
        }                                                                        \
    } while (0)

int main(int argc, char **argv) {
    if (argc < 9) {
        fprintf(stderr, "usage: %s mesh.pmsh order rk2 precision ic bc t_end out.bin [param ...]\n", argv[0]);
        return 2;
    }
    const char *mesh_path = argv[1];
    const int order = atoi(argv[2]), rk2 = atoi(argv[3]), precision = atoi(argv[4]);
    const int ic = atoi(argv[5]), bc = atoi(argv[6]);
    const double t_end = atof(argv[7]);
    const char *out_path = argv[8];
    double params[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 9; i < argc && i - 9 < 8; ++i) params[i - 9] = atof(argv[i]);

    /* read_mesh(...) (conserv.cu:118-192): the mesh arrays in the reference layout */
    int num_elem = 0, num_sides = 0;
    CHECK(dgx_pmsh_info(mesh_path, &num_elem, &num_sides));
    double *V = malloc(sizeof(double) * 6 * (size_t)num_elem);
    int *es = malloc(sizeof(int) * 3 * (size_t)num_elem);
    int *sides = malloc(sizeof(int) * 4 * (size_t)num_sides);
    if (!V || !es || !sides) return 1;
    CHECK(dgx_pmsh_read(mesh_path, V, es, sides));
    const size_t E = (size_t)num_elem, S = (size_t)num_sides;

    /* the binding: mesh, solver, initial state, time loop, state out */
    dgx_mesh *mesh;
    dgx_solver *solver;
    dgx_solver_desc desc = {.order = order, .equation = DGX_EULER, .flux = DGX_FLUX_LLF,
                            .precision = precision, .integrator = rk2 ? DGX_RK2 : DGX_RK4,
                            .gamma = 1.4, .ax = 1.0, .ay = 1.0};
    CHECK(dgx_mesh_create(num_elem, num_sides, V, V + E, V + 2 * E, V + 3 * E, V + 4 * E, V + 5 * E,
                          es, es + E, es + 2 * E, sides, sides + S, sides + 2 * S, sides + 3 * S, &mesh));
    CHECK(dgx_solver_create(mesh, &desc, &solver));
    if (bc != DGX_BC_NONE) CHECK(dgx_solver_set_boundary(solver, bc, ic, params));
    CHECK(dgx_project_ic(solver, ic, params));
    CHECK(dgx_set_dt(solver, DGX_DT_CFL, 0.0, 0.7));
    int steps = 0;
    double t = 0.0;
    CHECK(dgx_run(solver, t_end, 0, &steps, &t, NULL));

    int nv = 0, np = 0;
    size_t state_bytes = 0, device_bytes = 0;
    CHECK(dgx_solver_info(solver, &nv, &np, &state_bytes, &device_bytes));
    double *c = malloc(sizeof(double) * (size_t)nv * (size_t)np * E);
    if (!c) return 1;
    CHECK(dgx_get_state(solver, c));
    CHECK(dgx_solver_destroy(solver));
    CHECK(dgx_mesh_destroy(mesh));

    FILE *f = fopen(out_path, "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", out_path); return 1; }
    const int hdr[4] = {steps, nv, np, num_elem};
    fwrite(hdr, sizeof(int), 4, f);
    fwrite(&t, sizeof(double), 1, f);
    fwrite(c, sizeof(double), (size_t)nv * (size_t)np * E, f);
    fclose(f);
    free(V); free(es); free(sides); free(c);
    printf("steps %d t %.17g\n", steps, t);
    return 0;
}
