// curve_device.cuh -- the boundary curves and the rectangular-polar changes of variables on
// the device, shared by the translation units that evaluate the geometry (rp_precompute.cu,
// geometry_device.cu).  Curves follow Geometry/Curve.hpp:106-161 (the star curve is an
// extension); the changes of variables follow utils/Quadrature.hpp:70-173.
#pragma once
#include "ifgf2d_kernels.cuh"
#include "hankel.cuh"

namespace ifgf {

__device__ __forceinline__ void curve_eval(const DevCurve& c, double t, double& x, double& y, double& xp, double& yp) {
    const double* p = c.p;
    if (c.type == 0) {            // circle
        double s, co; sincos(t, &s, &co);
        x = p[2] * co + p[0]; y = p[2] * s + p[1]; xp = -p[2] * s; yp = p[2] * co;
    } else if (c.type == 1) {     // kite
        double s, co, s2, c2; sincos(t, &s, &co); sincos(2.0 * t, &s2, &c2);
        x = p[0] * co + p[1] * c2 + p[2]; y = p[3] * s; xp = -p[0] * s - 2.0 * p[1] * s2; yp = p[3] * co;
    } else if (c.type == 2) {     // line on [-1, 1]
        x = (p[2] * (t + 1.0) - p[0] * (t - 1)) / 2.0; y = (p[3] * (t + 1.0) - p[1] * (t - 1)) / 2.0;
        xp = (p[2] - p[0]) / 2.0; yp = (p[3] - p[1]) / 2.0;
    } else {                      // star r(t) = 1 + sum a_m cos mt + b_m sin mt
        const int M = (int)p[2];
        double r = 1.0, dr = 0.0;
        for (int m = 1; m <= M; ++m) {
            double s, co; sincos(m * t, &s, &co);
            r += p[2 + m] * co + p[2 + M + m] * s;
            dr += -m * p[2 + m] * s + m * p[2 + M + m] * co;
        }
        double s, co; sincos(t, &s, &co);
        x = p[0] + r * co; y = p[1] + r * s; xp = dr * co - r * s; yp = dr * s + r * co;
    }
}

// rectangular-polar changes of variables (utils/Quadrature.hpp:70-173)
__device__ __forceinline__ double d_v(double t, double p) { const double a = t / kPi - 1.0; return (0.5 - 1.0 / p) * (a * a * a) + (1.0 / p) * a + 0.5; }
__device__ __forceinline__ double d_vp(double t, double p) { const double a = t / kPi - 1.0; return (3.0 / kPi) * (0.5 - 1.0 / p) * (a * a) + 1.0 / (p * kPi); }
__device__ __forceinline__ double d_w(double t, double p) { const double a = pow(d_v(t, p), p); return 2.0 * kPi * a / (a + pow(d_v(2 * kPi - t, p), p)); }
__device__ __forceinline__ double d_wp(double t, double p) {
    const double a = d_v(t, p), b = d_v(2 * kPi - t, p);
    const double s = pow(a, p) + pow(b, p);
    return 2.0 * kPi * p * d_vp(t, p) * pow(a, p - 1.0) * pow(b, p - 1.0) / (s * s);
}
__device__ __forceinline__ int d_sgn(double v) { return (0.0 < v) - (v < 0.0); }

// second derivatives x'', y'' (for the signed curvature)
__device__ __forceinline__ void curve_eval2(const DevCurve& c, double t, double& xpp, double& ypp) {
    const double* p = c.p;
    if (c.type == 0) {
        double s, co; sincos(t, &s, &co);
        xpp = -p[2] * co; ypp = -p[2] * s;
    } else if (c.type == 1) {
        double s, co, s2, c2; sincos(t, &s, &co); sincos(2.0 * t, &s2, &c2);
        xpp = -p[0] * co - 4.0 * p[1] * c2; ypp = -p[3] * s;
    } else if (c.type == 2) {
        xpp = 0.0; ypp = 0.0;
    } else {
        const int M = (int)p[2];
        double r = 1.0, dr = 0.0, ddr = 0.0;
        for (int m = 1; m <= M; ++m) {
            double s, co; sincos(m * t, &s, &co);
            r += p[2 + m] * co + p[2 + M + m] * s;
            dr += -m * p[2 + m] * s + m * p[2 + M + m] * co;
            ddr += -m * m * (p[2 + m] * co + p[2 + M + m] * s);
        }
        double s, co; sincos(t, &s, &co);
        xpp = ddr * co - 2.0 * dr * s - r * co;
        ypp = ddr * s + 2.0 * dr * co - r * s;
    }
}

}  // namespace ifgf
