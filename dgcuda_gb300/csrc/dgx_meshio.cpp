// dgx_meshio.cpp -- the reference's text formats on the host.
//
// .pmsh (written by src/2d/genmesh.py:290-308, read by read_mesh,
// src/2d/conservation/conserv.cu:118-192):
//   num_elem
//   num_elem lines  "V1x V1y V2x V2y V3x V3y s1 s2 s3"
//   num_sides
//   num_sides lines "x1 y1 x2 y2 left_elem right_elem left_side right_side"
// The side end points are not needed (geometry comes from the elements) and
// are written from the left element's local side.
//
// Gmsh vertex values (src/2d/conservation/main.cu:193-209): one file per
// variable, "View \"U<n> \" {" then per element
// "ST (x1,y1,0,x2,y2,0,x3,y3,0) {u1,u2,u3};" and a closing "};".
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dgx_internal.h"

namespace dgx {
namespace {

struct File {
    FILE *f = nullptr;
    explicit File(const char *path, const char *mode) : f(std::fopen(path, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

int read_counts(FILE *f, int *E, int *S, long *sides_pos) {
    char line[1024];
    if (!std::fgets(line, sizeof(line), f) || std::sscanf(line, "%d", E) != 1 || *E <= 0) {
        set_error(".pmsh: bad element count");
        return DGX_ERR_INVALID;
    }
    for (int e = 0; e < *E; ++e)
        if (!std::fgets(line, sizeof(line), f)) {
            set_error(".pmsh: file ends inside the element list");
            return DGX_ERR_INVALID;
        }
    if (sides_pos) *sides_pos = std::ftell(f);
    if (!std::fgets(line, sizeof(line), f) || std::sscanf(line, "%d", S) != 1 || *S <= 0) {
        set_error(".pmsh: bad side count");
        return DGX_ERR_INVALID;
    }
    return DGX_OK;
}

}  // namespace
}  // namespace dgx

using namespace dgx;

extern "C" {

int dgx_pmsh_info(const char *path, int *num_elem, int *num_sides) {
    if (!path || !num_elem || !num_sides) return DGX_ERR_INVALID;
    File F(path, "r");
    if (!F.f) { set_error("cannot open %s", path); return DGX_ERR_NOT_FOUND; }
    return read_counts(F.f, num_elem, num_sides, nullptr);
}

// V[6][E], elem_s[3][E], sides[4][S] (left, right, left_side, right_side)
int dgx_pmsh_read(const char *path, double *V, int *elem_s, int *sides) {
    if (!path || !V || !elem_s || !sides) return DGX_ERR_INVALID;
    File F(path, "r");
    if (!F.f) { set_error("cannot open %s", path); return DGX_ERR_NOT_FOUND; }
    char line[1024];
    int E = 0, S = 0;
    if (!std::fgets(line, sizeof(line), F.f) || std::sscanf(line, "%d", &E) != 1 || E <= 0) {
        set_error(".pmsh: bad element count");
        return DGX_ERR_INVALID;
    }
    for (int e = 0; e < E; ++e) {
        double v[6];
        int s[3];
        if (!std::fgets(line, sizeof(line), F.f) ||
            std::sscanf(line, "%lf %lf %lf %lf %lf %lf %d %d %d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5],
                        &s[0], &s[1], &s[2]) != 9) {
            set_error(".pmsh: element line %d does not hold 9 items", e);
            return DGX_ERR_INVALID;
        }
        for (int c = 0; c < 6; ++c) V[static_cast<size_t>(c) * E + e] = v[c];
        for (int c = 0; c < 3; ++c) elem_s[static_cast<size_t>(c) * E + e] = s[c];
    }
    if (!std::fgets(line, sizeof(line), F.f) || std::sscanf(line, "%d", &S) != 1 || S <= 0) {
        set_error(".pmsh: bad side count");
        return DGX_ERR_INVALID;
    }
    for (int k = 0; k < S; ++k) {
        double x1, y1, x2, y2;
        int le, re, ls, rs;
        if (!std::fgets(line, sizeof(line), F.f) ||
            std::sscanf(line, "%lf %lf %lf %lf %d %d %d %d", &x1, &y1, &x2, &y2, &le, &re, &ls, &rs) != 8) {
            set_error(".pmsh: side line %d does not hold 8 items", k);
            return DGX_ERR_INVALID;
        }
        sides[k] = le;
        sides[static_cast<size_t>(S) + k] = re;
        sides[2 * static_cast<size_t>(S) + k] = ls;
        sides[3 * static_cast<size_t>(S) + k] = rs;
    }
    return DGX_OK;
}

int dgx_pmsh_write(const char *path, int num_elem, int num_sides, const double *V, const int *elem_s,
                   const int *sides) {
    if (!path || !V || !elem_s || !sides || num_elem <= 0 || num_sides <= 0) return DGX_ERR_INVALID;
    File F(path, "w");
    if (!F.f) { set_error("cannot create %s", path); return DGX_ERR_NOT_FOUND; }
    const size_t E = num_elem, S = num_sides;
    std::fprintf(F.f, "%d\n", num_elem);
    for (size_t e = 0; e < E; ++e)
        std::fprintf(F.f, "%.17g %.17g %.17g %.17g %.17g %.17g %d %d %d\n", V[e], V[E + e], V[2 * E + e],
                     V[3 * E + e], V[4 * E + e], V[5 * E + e], elem_s[e], elem_s[E + e], elem_s[2 * E + e]);
    std::fprintf(F.f, "%d\n", num_sides);
    for (size_t k = 0; k < S; ++k) {
        const int le = sides[k], ls = sides[2 * S + k];
        if (le < 0 || le >= num_elem || ls < 0 || ls > 2) { set_error("side %zu: bad left element", k); return DGX_ERR_INVALID; }
        const double px[3] = {V[le], V[2 * E + le], V[4 * E + le]}, py[3] = {V[E + le], V[3 * E + le], V[5 * E + le]};
        std::fprintf(F.f, "%.17g %.17g %.17g %.17g %d %d %d %d\n", px[ls], py[ls], px[(ls + 1) % 3],
                     py[(ls + 1) % 3], le, sides[S + k], ls, sides[3 * S + k]);
    }
    return std::ferror(F.f) ? DGX_ERR_INVALID : DGX_OK;
}

int dgx_mesh_create_from_pmsh(const char *path, dgx_mesh **out) {
    int E = 0, S = 0;
    int rc = dgx_pmsh_info(path, &E, &S);
    if (rc) return rc;
    std::vector<double> V(6 * static_cast<size_t>(E));
    std::vector<int> es(3 * static_cast<size_t>(E)), sd(4 * static_cast<size_t>(S));
    rc = dgx_pmsh_read(path, V.data(), es.data(), sd.data());
    if (rc) return rc;
    const size_t e = E, s = S;
    return dgx_mesh_create(E, S, V.data(), V.data() + e, V.data() + 2 * e, V.data() + 3 * e, V.data() + 4 * e,
                           V.data() + 5 * e, es.data(), es.data() + e, es.data() + 2 * e, sd.data(), sd.data() + s,
                           sd.data() + 2 * s, sd.data() + 3 * s, out);
}

// Vertex values of every variable, written as the reference's Gmsh "ST" views,
// one file per variable: printf(path_pattern, n) (e.g. "out/U%d.msh").
int dgx_write_vertex_values(dgx_solver *sv, const char *path_pattern) {
    if (!sv || !path_pattern) return DGX_ERR_INVALID;
    const MeshDev &m = sv->mesh->d;
    const SolverDev &s = sv->s;
    const size_t E = m.num_elem;
    std::vector<double> c(s.n), V(6 * E);
    int rc = dgx_get_state(sv, c.data());
    if (rc) return rc;
    DGX_TRY_CUDA(cudaMemcpy(V.data(), m.V, sizeof(double) * 6 * E, cudaMemcpyDeviceToHost));
    const Tables &T = tables(s.order);
    for (int n = 0; n < s.nv; ++n) {
        char path[4096];
        std::snprintf(path, sizeof(path), path_pattern, n);
        File F(path, "w");
        if (!F.f) { set_error("cannot create %s", path); return DGX_ERR_NOT_FOUND; }
        std::fprintf(F.f, "View \"U%i \" {\n", n);
        for (size_t e = 0; e < E; ++e) {
            double u[3] = {0, 0, 0};
            for (int i = 0; i < s.np; ++i) {
                const double ci = c[(static_cast<size_t>(n) * s.np + i) * E + e];
                for (int v = 0; v < 3; ++v) u[v] += ci * T.vert[3 * i + v];
            }
            std::fprintf(F.f, "ST (%lf,%lf,0,%lf,%lf,0,%lf,%lf,0) {%lf,%lf,%lf};\n", V[e], V[E + e], V[2 * E + e],
                         V[3 * E + e], V[4 * E + e], V[5 * E + e], u[0], u[1], u[2]);
        }
        std::fprintf(F.f, "};");
    }
    return DGX_OK;
}

}  // extern "C"
