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

// the reference's problem files define PI as 3.14159 (threepoint.cu:13)
constexpr double kRefPi = 3.14159;

// oblique shock state of the three-point problem (U_shock, threepoint.cu:27-32):
// P = {M, theta in degrees}
__device__ inline void threepoint_shock(const double *P, double g, double *U) {
    const double a = P[1] * kRefPi / 180.0;
    U[0] = g;
    U[1] = P[0] * cos(a) * U[0];
    U[2] = P[0] * sin(a) * U[0];
    U[3] = 0.5 * U[0] * P[0] * P[0] + 1.0 / (g - 1.0);
}

// ref_float: the FP32 powers of the reference's problem file where it calls
// powf (the supersonic vortex, supersonic.cu:30,35); FP64 pow otherwise
__device__ inline void ic_eval(int ic, const double *P, double g, double x, double y, double *U,
                               bool ref_float = false) {
    const double pi = 3.14159265358979323846;
    switch (ic) {
    case DGX_IC_GAUSSIAN: {
        const double dx = wrap_dist(x - P[0], P[3]), dy = wrap_dist(y - P[1], P[4]);
        U[0] = exp(-(dx * dx + dy * dy) / P[2]);
        break;
    }
    case DGX_IC_POLY: U[0] = pow(x - y, P[0]); break;
    case DGX_IC_LINEAR: U[0] = P[0] + P[1] * x + P[2] * y; break;
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
    case DGX_IC_CYLINDER:   // free stream of the cylinder problem (cylinder.cu:26-31)
        U[0] = g; U[1] = U[0] * P[0]; U[2] = 0.0;
        U[3] = 0.5 * U[0] * P[0] * P[0] + 1.0 / (g - 1.0);
        break;
    case DGX_IC_SUPERSONIC_VORTEX: {   // supersonic.cu:28-38 (pow, or with ref_float its powf)
        const double r = sqrt(x * x + y * y), th = atan(y / x);
        const double A = P[1] != 0.0 ? P[1] : 0.5 * (g - 1.0) * P[0] * P[0];
        const double base = 1.0 + A * (1.0 - 1.0 / (r * r));
        U[0] = ref_float ? static_cast<double>(powf(static_cast<float>(base), 2.5f)) : pow(base, 2.5);
        U[1] = U[0] * sin(th) * P[0] / r;
        U[2] = U[0] * -cos(th) * P[0] / r;
        const double p = (1.0 / g) * (ref_float ? static_cast<double>(powf(static_cast<float>(U[0]),
                                                                           static_cast<float>(g)))
                                                : pow(U[0], g));
        U[3] = 0.5 * U[0] * (P[0] * P[0] / (r * r)) + p * (1.0 / (g - 1.0));
        break;
    }
    case DGX_IC_THREEPOINT:   // threepoint.cu:44-54
        if (atan(x / y) < P[1] * kRefPi / 180.0) {
            threepoint_shock(P, g, U);
        } else {
            U[0] = 0.5 * g; U[1] = 0.0; U[2] = 0.0;
            U[3] = 0.5 * U[0] * P[0] * P[0] + 1.0 / (g - 1.0);
        }
        break;
    default:
        U[0] = P[0]; U[1] = P[0] * P[1]; U[2] = P[0] * P[2];
        U[3] = P[3] / (g - 1.0) + 0.5 * P[0] * (P[1] * P[1] + P[2] * P[2]);
        break;
    }
}


}  // namespace dgx
