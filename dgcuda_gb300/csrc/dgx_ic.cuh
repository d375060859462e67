// dgx_ic.cuh -- the built-in initial conditions (FP64, device), shared by the
// projection kernel and the exact-Dirichlet boundary ghost state.
#pragma once

#include "dgx.h"

namespace dgx {

__device__ inline double wrap_dist(double d, double L) {
    if (L > 0) {
        d = fmod(d, L);
        if (d > 0.5 * L) d -= L;
        if (d < -0.5 * L) d += L;
    }
    return d;
}

__device__ inline void ic_eval(int ic, const double *P, double g, double x, double y, double *U) {
    const double pi = 3.14159265358979323846;
    switch (ic) {
    case DGX_IC_GAUSSIAN: {
        const double dx = wrap_dist(x - P[0], P[3]), dy = wrap_dist(y - P[1], P[4]);
        U[0] = exp(-(dx * dx + dy * dy) / P[2]);
        break;
    }
    case DGX_IC_POLY: U[0] = pow(x - y, P[0]); break;
    case DGX_IC_DENSITY_WAVE: {
        const double rho = 1.0 + P[0] * sin(2.0 * pi * P[4] * (x + y));
        U[0] = rho; U[1] = rho * P[1]; U[2] = rho * P[2];
        U[3] = P[3] / (g - 1.0) + 0.5 * rho * (P[1] * P[1] + P[2] * P[2]);
        break;
    }
    case DGX_IC_VORTEX: {
        const double dx = wrap_dist(x - P[0], P[5]), dy = wrap_dist(y - P[1], P[6]);
        const double r2 = dx * dx + dy * dy, b = P[2];
        const double f = exp(0.5 * (1.0 - r2));
        const double u = P[3] - b / (2.0 * pi) * f * dy;
        const double v = P[4] + b / (2.0 * pi) * f * dx;
        const double T = 1.0 - (g - 1.0) * b * b / (8.0 * g * pi * pi) * f * f;
        const double rho = pow(T, 1.0 / (g - 1.0)), p = pow(rho, g);
        U[0] = rho; U[1] = rho * u; U[2] = rho * v;
        U[3] = p / (g - 1.0) + 0.5 * rho * (u * u + v * v);
        break;
    }
    default:
        U[0] = P[0]; U[1] = P[0] * P[1]; U[2] = P[0] * P[2];
        U[3] = P[3] / (g - 1.0) + 0.5 * P[0] * (P[1] * P[1] + P[2] * P[2]);
        break;
    }
}


}  // namespace dgx
