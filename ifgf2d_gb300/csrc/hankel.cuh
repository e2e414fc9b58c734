// hankel.cuh -- device Hankel functions H0^(1), H1^(1) of real argument, FP64.
//
// Replaces sp_bessel::hankelH1 (complex_bessel-master/include/complex_bessel_bits/
// besselFunctions.h:313-341 -> AMOS zbesh) on the GPU.  Real wavenumber, real x > 0.
// Three regions (coefficients in hankel_tables.inc, generated by gen_hankel_tables.py):
//   x < HK_XA        ascending series in q = x^2/4 (A&S 9.1.10-11), Horner;
//   HK_XA <= x < XC  piecewise Chebyshev expansions of J_nu and Y_nu (width HK_W), Clenshaw;
//   x >= HK_XC       Hankel asymptotic expansion (A&S 9.2.5-10), P, Q polynomials in 1/x^2.
// |H| never vanishes for real x, so errors are stated relative to |H| (~1e-15, tested
// against scipy.special.hankel1 in tests/test_gpu_parity.py).
#pragma once
#include <cuda_runtime.h>

#define HK_TABLE __device__ const
#include "hankel_tables.inc"

namespace ifgf {

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoOverPi = 0.63661977236758134308;
constexpr double kEulerGamma = 0.57721566490153286061;

template <int NU>
__device__ __forceinline__ double2 hankel1(double x) {
    if (x < HK_XA) {
        const double* a = NU == 0 ? hk_ser_a0 : hk_ser_a1;
        const double* b = NU == 0 ? hk_ser_b0 : hk_ser_b1;
        const double q = 0.25 * x * x;
        double J = __ldg(a + HK_NSER - 1), S = __ldg(b + HK_NSER - 1);
#pragma unroll
        for (int k = HK_NSER - 2; k >= 0; --k) { J = fma(J, q, __ldg(a + k)); S = fma(S, q, __ldg(b + k)); }
        const double L = kTwoOverPi * (log(0.5 * x) + kEulerGamma);
        if (NU == 0) return make_double2(J, fma(L, J, S));
        const double h = 0.5 * x;
        const double J1 = h * J;
        return make_double2(J1, fma(L, J1, h * S) - kTwoOverPi / x);
    } else if (x < HK_XC) {
        int p = (int)((x - HK_XA) * (1.0 / HK_W));
        p = p < 0 ? 0 : (p >= HK_NPIECES ? HK_NPIECES - 1 : p);
        const double t = (x - (HK_XA + p * HK_W)) * (2.0 / HK_W) - 1.0;
        const double* cj = (NU == 0 ? hk_cheb0 : hk_cheb1) + p * 2 * (HK_DEG + 1);
        const double* cy = cj + (HK_DEG + 1);
        double bj1 = 0.0, bj2 = 0.0, by1 = 0.0, by2 = 0.0;
        const double t2 = 2.0 * t;
#pragma unroll
        for (int k = HK_DEG; k >= 1; --k) {
            const double bj = fma(t2, bj1, __ldg(cj + k) - bj2);
            const double by = fma(t2, by1, __ldg(cy + k) - by2);
            bj2 = bj1; bj1 = bj; by2 = by1; by1 = by;
        }
        return make_double2(fma(t, bj1, __ldg(cj) - bj2), fma(t, by1, __ldg(cy) - by2));
    } else {
        const double* P = NU == 0 ? hk_asyP0 : hk_asyP1;
        const double* Q = NU == 0 ? hk_asyQ0 : hk_asyQ1;
        const double w = 1.0 / x, w2 = w * w;
        double pp = __ldg(P + HK_NASY - 1), qq = __ldg(Q + HK_NASY - 1);
#pragma unroll
        for (int k = HK_NASY - 2; k >= 0; --k) { pp = fma(pp, w2, __ldg(P + k)); qq = fma(qq, w2, __ldg(Q + k)); }
        qq *= w;
        double s, c;
        sincos(x, &s, &c);
        // e^{i(x - pi/4)} = (c + s + i(s - c))/sqrt2 ; e^{i(x - 3pi/4)} = (s - c - i(s + c))/sqrt2
        const double er = NU == 0 ? (c + s) : (s - c);
        const double ei = NU == 0 ? (s - c) : -(s + c);
        const double amp = sqrt(w * (1.0 / kPi));   // sqrt(2/(pi x)) / sqrt(2)
        return make_double2(amp * (pp * er - qq * ei), amp * (pp * ei + qq * er));
    }
}

// H0 and H1 of the same argument: the per-argument work of each region (the logarithm, the
// Chebyshev piece, 1/x, the amplitude and the one sincos of the asymptotic region) is done once.
// Each result takes the same operations as hankel1<0> / hankel1<1>.
__device__ __forceinline__ void hankel01(double x, double2& h0, double2& h1) {
    if (x < HK_XA) {
        const double q = 0.25 * x * x;
        double J0 = __ldg(hk_ser_a0 + HK_NSER - 1), S0 = __ldg(hk_ser_b0 + HK_NSER - 1);
        double J1 = __ldg(hk_ser_a1 + HK_NSER - 1), S1 = __ldg(hk_ser_b1 + HK_NSER - 1);
#pragma unroll
        for (int k = HK_NSER - 2; k >= 0; --k) {
            J0 = fma(J0, q, __ldg(hk_ser_a0 + k)); S0 = fma(S0, q, __ldg(hk_ser_b0 + k));
            J1 = fma(J1, q, __ldg(hk_ser_a1 + k)); S1 = fma(S1, q, __ldg(hk_ser_b1 + k));
        }
        const double L = kTwoOverPi * (log(0.5 * x) + kEulerGamma);
        h0 = make_double2(J0, fma(L, J0, S0));
        const double h = 0.5 * x;
        const double j1 = h * J1;
        h1 = make_double2(j1, fma(L, j1, h * S1) - kTwoOverPi / x);
    } else if (x < HK_XC) {
        int p = (int)((x - HK_XA) * (1.0 / HK_W));
        p = p < 0 ? 0 : (p >= HK_NPIECES ? HK_NPIECES - 1 : p);
        const double t = (x - (HK_XA + p * HK_W)) * (2.0 / HK_W) - 1.0;
        const double t2 = 2.0 * t;
#pragma unroll
        for (int nu = 0; nu < 2; ++nu) {
            const double* cj = (nu == 0 ? hk_cheb0 : hk_cheb1) + p * 2 * (HK_DEG + 1);
            const double* cy = cj + (HK_DEG + 1);
            double bj1 = 0.0, bj2 = 0.0, by1 = 0.0, by2 = 0.0;
#pragma unroll
            for (int k = HK_DEG; k >= 1; --k) {
                const double bj = fma(t2, bj1, __ldg(cj + k) - bj2);
                const double by = fma(t2, by1, __ldg(cy + k) - by2);
                bj2 = bj1; bj1 = bj; by2 = by1; by1 = by;
            }
            const double2 v = make_double2(fma(t, bj1, __ldg(cj) - bj2), fma(t, by1, __ldg(cy) - by2));
            if (nu == 0) h0 = v; else h1 = v;
        }
    } else {
        const double w = 1.0 / x, w2 = w * w;
        double p0 = __ldg(hk_asyP0 + HK_NASY - 1), q0 = __ldg(hk_asyQ0 + HK_NASY - 1);
        double p1 = __ldg(hk_asyP1 + HK_NASY - 1), q1 = __ldg(hk_asyQ1 + HK_NASY - 1);
#pragma unroll
        for (int k = HK_NASY - 2; k >= 0; --k) {
            p0 = fma(p0, w2, __ldg(hk_asyP0 + k)); q0 = fma(q0, w2, __ldg(hk_asyQ0 + k));
            p1 = fma(p1, w2, __ldg(hk_asyP1 + k)); q1 = fma(q1, w2, __ldg(hk_asyQ1 + k));
        }
        q0 *= w; q1 *= w;
        double s, c;
        sincos(x, &s, &c);
        const double amp = sqrt(w * (1.0 / kPi));
        const double er0 = c + s, ei0 = s - c, er1 = s - c, ei1 = -(s + c);
        h0 = make_double2(amp * (p0 * er0 - q0 * ei0), amp * (p0 * ei0 + q0 * er0));
        h1 = make_double2(amp * (p1 * er1 - q1 * ei1), amp * (p1 * ei1 + q1 * er1));
    }
}

// Single-layer kernel (i/4) H0(k r), 0 for r < 1e-14 (ForwardMap/GreenFunctions.hpp:87-108)
__device__ __forceinline__ double2 green_sl(double dx, double dy, double k) {
    const double r = sqrt(dx * dx + dy * dy);
    if (r < 1e-14) return make_double2(0.0, 0.0);
    const double2 h = hankel1<0>(k * r);
    return make_double2(-0.25 * h.y, 0.25 * h.x);
}

// Combined-field kernel without the jump term, target minus source d = x - y, unit normal n
// at the source y:  dPhi/dn_y - i eta Phi = (ik/4) H1(kr) (d.n)/r + (eta/4) H0(kr); 0 for r < 1e-14.
__device__ __forceinline__ double2 green_cfie(double dx, double dy, double nx, double ny, double k, double eta) {
    const double r = sqrt(dx * dx + dy * dy);
    if (r < 1e-14) return make_double2(0.0, 0.0);
    double2 h0, h1;
    hankel01(k * r, h0, h1);
    const double c = 0.25 * k * (dx * nx + dy * ny) / r;   // (ik/4)(d.n)/r = i c
    return make_double2(-c * h1.y + 0.25 * eta * h0.x, c * h1.x + 0.25 * eta * h0.y);
}

// kernel of the chosen formulation (eta unused for the single layer)
__device__ __forceinline__ double2 green_form(int form, double dx, double dy, double nx, double ny, double k, double eta) {
    return form == 2 ? green_cfie(dx, dy, nx, ny, k, eta) : green_sl(dx, dy, k);
}

// e^{ikr}/sqrt(r) (GreenFunctions.hpp:125-131)
__device__ __forceinline__ double2 factorization(double r, double k) {
    double s, c;
    sincos(k * r, &s, &c);
    const double a = 1.0 / sqrt(r);
    return make_double2(c * a, s * a);
}

}  // namespace ifgf
