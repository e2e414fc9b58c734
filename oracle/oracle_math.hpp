// oracle_math.hpp -- CPU ORACLE (test infrastructure only; never linked into the product).
//
// Scalar numerics of the IFGF2D forward map restated for the CPU oracle:
//   * Hankel functions H0^(1), H1^(1) of real argument (replaces the AMOS/complex_bessel
//     call sp_bessel::hankelH1, complex_bessel-master/include/complex_bessel_bits/
//     besselFunctions.h:313-341).  Method: ascending power series (A&S 9.1.10-9.1.11)
//     summed in double-double arithmetic for x < 25, Hankel asymptotic expansion
//     (A&S 9.2.5-9.2.10) for x >= 25.  Pinned against scipy.special.hankel1 by the
//     tests (tests/test_oracle.py).
//   * Fejer quadrature and the rectangular-polar changes of variables
//     (utils/Quadrature.hpp:12-173).
//   * 1D Chebyshev transform and root finding (utils/Chebyshev1d.hpp:249-266, 134-163,
//     231-267).  The colleague-matrix eigen-solve of cheb_root_finder is replaced by
//     sign-change sampling + bisection of the same degree N-1 interpolant.
//   * Brent's minimiser (utils/BrentsMethod.hpp:42-156): Brent's published
//     "localmin" algorithm, restated step for step because the near-singular t
//     values it returns feed the rectangular-polar weights.
#pragma once

#include <cmath>
#include <complex>
#include <vector>
#include <array>
#include <functional>
#include <algorithm>

namespace orc {

using cd = std::complex<double>;
static constexpr double PI = 3.14159265358979323846264338327950288;
static constexpr double EULER_GAMMA = 0.57721566490153286060651209008240243;

// ------------------------------------------------------------------------------------
// double-double arithmetic (Dekker / Knuth error-free transformations)
// ------------------------------------------------------------------------------------
struct dd { double hi, lo; };
static inline dd dd_quick_two_sum(double a, double b) { double s = a + b; return {s, b - (s - a)}; }
static inline dd dd_two_sum(double a, double b) {
    double s = a + b; double bb = s - a; return {s, (a - (s - bb)) + (b - bb)};
}
static inline dd dd_add(dd a, dd b) {
    dd s = dd_two_sum(a.hi, b.hi);
    dd t = dd_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = dd_quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return dd_quick_two_sum(s.hi, s.lo);
}
static inline dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
static inline dd dd_mul(dd a, dd b) {
    double p = a.hi * b.hi; double e = std::fma(a.hi, b.hi, -p);
    e += a.hi * b.lo + a.lo * b.hi;
    return dd_quick_two_sum(p, e);
}
static inline dd dd_mul_d(dd a, double b) {
    double p = a.hi * b; double e = std::fma(a.hi, b, -p);
    e += a.lo * b;
    return dd_quick_two_sum(p, e);
}
static inline dd dd_div_d(dd a, double b) {
    double q1 = a.hi / b;
    double p = q1 * b; double pe = std::fma(q1, b, -p);
    dd s = dd_two_sum(a.hi, -p);
    s.lo -= pe; s.lo += a.lo;
    double q2 = (s.hi + s.lo) / b;
    return dd_quick_two_sum(q1, q2);
}
static inline double dd_to_d(dd a) { return a.hi + a.lo; }

// ------------------------------------------------------------------------------------
// Bessel J0, Y0, J1, Y1 and Hankel H0^(1), H1^(1) for real x > 0
// ------------------------------------------------------------------------------------
static constexpr double HANKEL_SERIES_MAX = 25.0;

// Ascending series in double-double.  Returns J0,Y0 (order 0) or J1,Y1 (order 1).
static inline void bessel_series(int order, double x, double& J, double& Y) {
    // q = x^2/4 exactly as a double-double
    double x2 = x * x; double x2e = std::fma(x, x, -x2);
    dd q = {x2 * 0.25, x2e * 0.25};
    dd mq = dd_neg(q);
    const double lnhalf = std::log(0.5 * x);
    if (order == 0) {
        // J0 = sum_k t_k, t_k = (-q)^k/(k!)^2 ; Y0 = (2/pi)[(ln(x/2)+gamma) J0 - sum_k H_k t_k]
        dd t = {1.0, 0.0}, sJ = {1.0, 0.0}, sH = {0.0, 0.0}, H = {0.0, 0.0};
        for (int k = 1; k < 400; ++k) {
            t = dd_div_d(dd_mul(t, mq), double(k) * double(k));
            H = dd_add(H, dd_div_d({1.0, 0.0}, double(k)));
            sJ = dd_add(sJ, t);
            sH = dd_add(sH, dd_mul(H, t));
            if (double(k) > 0.5 * x && std::fabs(t.hi) * (1.0 + std::fabs(H.hi)) < 1e-34) break;
        }
        J = dd_to_d(sJ);
        dd y = dd_add(dd_mul_d(sJ, lnhalf + EULER_GAMMA), dd_neg(sH));
        Y = (2.0 / PI) * dd_to_d(y);
    } else {
        // J1 = sum_k u_k, u_k = (x/2)(-q)^k/(k!(k+1)!)
        // Y1 = (2/pi)(ln(x/2)+gamma) J1 - 2/(pi x) - (1/pi) sum_k (H_k + H_{k+1}) u_k
        dd u = {0.5 * x, 0.0}, sJ = u, H = {0.0, 0.0}, H1 = {1.0, 0.0};
        dd sH = dd_mul(dd_add(H, H1), u);
        for (int k = 1; k < 400; ++k) {
            u = dd_div_d(dd_mul(u, mq), double(k) * double(k + 1));
            H = H1;
            H1 = dd_add(H1, dd_div_d({1.0, 0.0}, double(k + 1)));
            sJ = dd_add(sJ, u);
            sH = dd_add(sH, dd_mul(dd_add(H, H1), u));
            if (double(k) > 0.5 * x && std::fabs(u.hi) * (1.0 + std::fabs(H1.hi)) < 1e-34) break;
        }
        J = dd_to_d(sJ);
        dd y = dd_add(dd_mul_d(sJ, (2.0 / PI) * (lnhalf + EULER_GAMMA)),
                      dd_neg(dd_mul_d(sH, 1.0 / PI)));
        Y = dd_to_d(y) - 2.0 / (PI * x);
    }
}

// Hankel asymptotic expansion: H_nu(x) = sqrt(2/(pi x)) (P + iQ) e^{i(x - (nu/2+1/4) pi)}
static inline cd hankel_asymptotic(int order, double x) {
    const double mu = 4.0 * order * order;
    double c = 1.0;                // (nu, m) / (2x)^m
    double P = 1.0, Q = 0.0;
    double prev = 1e300;
    for (int m = 1; m < 120; ++m) {
        double f = (2.0 * m - 1.0);
        c *= (mu - f * f) / (4.0 * m) / (2.0 * x);
        double a = std::fabs(c);
        if (a > prev) break;       // asymptotic series started to diverge
        prev = a;
        if (m & 1) { Q += ((m / 2) & 1 ? -c : c); }
        else       { P += ((m / 2) & 1 ? -c : c); }
        if (a < 1e-19) break;
    }
    // e^{i(x - (nu/2 + 1/4) pi)} = e^{ix} * e^{-i (nu/2+1/4) pi}
    const double s = std::sin(x), co = std::cos(x);
    const double r2 = std::sqrt(0.5);
    cd phase = cd(co, s) * (order == 0 ? cd(r2, -r2) : cd(-r2, -r2));
    return std::sqrt(2.0 / (PI * x)) * cd(P, Q) * phase;
}

static inline cd hankel1(int order, double x) {
    if (x < HANKEL_SERIES_MAX) {
        double J, Y; bessel_series(order, x, J, Y); return cd(J, Y);
    }
    return hankel_asymptotic(order, x);
}

// ------------------------------------------------------------------------------------
// Quadrature.hpp restated (utils/Quadrature.hpp:12-173)
// ------------------------------------------------------------------------------------
static inline double ab2cd(double x, double a, double b, double c, double d) {
    return ((d - c) / (b - a)) * (x - a) + c;
}
static inline double ab2cdjac(double a, double b, double c, double d) { return (d - c) / (b - a); }

// Fejer's first rule on [-1,1], nodes cos(pi(2i+1)/(2N)) (descending).  Quadrature.hpp:25-43
static inline void fejer1(int N, std::vector<double>& nodes, std::vector<double>& weights) {
    nodes.assign(N, 0.0); weights.assign(N, 0.0);
    for (int i = 0; i < N; ++i) {
        nodes[i] = std::cos(PI * (2.0 * i + 1.0) / (2.0 * N));
        double w = 0.0;
        for (int j = 1; j <= (int)std::floor(N * 0.5); ++j)
            w += std::cos(j * PI * (2.0 * i + 1.0) / N) / (4.0 * j * j - 1.0);
        weights[i] = (2.0 / N) * (1.0 - 2.0 * w);
    }
}

static inline double v_func(double t, double p) {
    double a = t / PI - 1.0;
    return (0.5 - 1.0 / p) * std::pow(a, 3) + (1.0 / p) * a + 0.5;
}
static inline double vp_func(double t, double p) {
    double a = t / PI - 1.0;
    return (3.0 / PI) * (0.5 - 1.0 / p) * std::pow(a, 2.0) + 1.0 / (p * PI);
}
static inline double w_cov_base(double t, double p) {
    double vp = std::pow(v_func(t, p), p);
    return 2.0 * PI * vp / (vp + std::pow(v_func(2 * PI - t, p), p));
}
static inline double wp_cov_base(double t, double p) {
    double num = 2.0 * PI * p * vp_func(t, p) * std::pow(v_func(t, p), p - 1.0) *
                 std::pow(v_func(2 * PI - t, p), p - 1.0);
    double den = std::pow(std::pow(v_func(t, p), p) + std::pow(v_func(2 * PI - t, p), p), 2.0);
    return num / den;
}
static inline int sgn(double v) { return (0.0 < v) - (v < 0.0); }
static inline double xi_cov_center(double t, double alpha, double p) {
    return alpha + ((sgn(t) - alpha) / PI) * w_cov_base(PI * std::fabs(t), p);
}
static inline double xi_cov_right(double t, double p) {
    return 1.0 - (2.0 / PI) * w_cov_base(PI * std::fabs((t - 1.0) / 2.0), p);
}
static inline double xi_cov_left(double t, double p) {
    return -1.0 + (2.0 / PI) * w_cov_base(PI * std::fabs((t + 1.0) / 2.0), p);
}
static inline double dxi_cov_center(double t, double alpha, double p) {
    return (1.0 - alpha * sgn(t)) * wp_cov_base(PI * std::fabs(t), p);
}
static inline double dxi_cov_right(double t, double p) {
    double h = (t - 1.0) / 2.0; return -wp_cov_base(PI * std::fabs(h), p) * sgn(h);
}
static inline double dxi_cov_left(double t, double p) {
    double h = (t + 1.0) / 2.0; return wp_cov_base(PI * std::fabs(h), p) * sgn(h);
}
static inline double both_edge_cov(double t, double p) { return -1.0 + (1.0 / PI) * w_cov_base(PI * (t + 1.0), p); }
static inline double minus1_edge_cov(double t, double p) { return -1.0 + 2.0 * (1.0 / PI) * w_cov_base((PI / 2.0) * (t + 1.0), p); }
static inline double plus1_edge_cov(double t, double p) { return -3.0 + 2.0 * (1.0 / PI) * w_cov_base(PI + (PI / 2.0) * (t + 1), p); }
static inline double der_both_edge_cov(double t, double p) { return wp_cov_base(PI * (t + 1.0), p); }
static inline double der_minus1_edge_cov(double t, double p) { return wp_cov_base(PI * (t + 1.0), p); }
static inline double der_plus1_edge_cov(double t, double p) { return wp_cov_base(PI + (PI / 2.0) * (t + 1), p); }

// ------------------------------------------------------------------------------------
// Chebyshev1d.hpp restated
// ------------------------------------------------------------------------------------
// Chebyshev points cos(pi(2i+1)/(2N)), descending (Chebyshev1d.hpp:252-265)
static inline std::vector<double> cheb1d_points(int N) {
    std::vector<double> x(N);
    for (int i = 0; i < N; ++i) x[i] = std::cos(PI * (2.0 * i + 1.0) / (2.0 * N));
    return x;
}
// T_n(x_i) table [n][i] (Chebyshev1d.hpp:285-310)
static inline std::vector<std::vector<double>> cheb1d_Tn(int N) {
    std::vector<double> x = cheb1d_points(N);
    std::vector<std::vector<double>> T(N, std::vector<double>(N));
    for (int i = 0; i < N; ++i) { T[0][i] = 1.0; if (N > 1) T[1][i] = x[i]; }
    for (int n = 2; n < N; ++n)
        for (int i = 0; i < N; ++i) T[n][i] = 2.0 * x[i] * T[n - 1][i] - T[n - 2][i];
    return T;
}
// values at the descending Chebyshev points -> coefficients (Chebyshev1d.hpp:363-392)
static inline void cheb1d_coeffs(int N, const cd* f, cd* c, const std::vector<std::vector<double>>& T) {
    for (int i = 0; i < N; ++i) c[i] = 0.0;
    for (int k = 0; k < N; ++k) { c[0] += f[k]; c[1] += f[k] * T[1][k]; }
    c[0] *= 1.0 / N; c[1] *= 2.0 / N;
    for (int i = 2; i < N; ++i) {
        for (int k = 0; k < N; ++k) c[i] += f[k] * T[i][k];
        c[i] *= 2.0 / N;
    }
}
// Real coefficients of f on [a,b] from N Chebyshev samples (Chebyshev1d.hpp:446-457, 322-360)
static inline std::vector<double> cheb1d_fit(const std::function<double(double)>& f, int N, double a, double b) {
    std::vector<double> x = cheb1d_points(N), fv(N), c(N, 0.0);
    for (int i = 0; i < N; ++i) fv[i] = f(ab2cd(x[i], -1, 1, a, b));
    std::vector<double> tnm1(N, 1.0), tn(x);
    for (int k = 0; k < N; ++k) { c[0] += fv[k]; c[1] += fv[k] * x[k]; }
    c[0] *= 1.0 / N; c[1] *= 2.0 / N;
    for (int i = 2; i < N; ++i) {
        for (int k = 0; k < N; ++k) {
            double v = 2.0 * x[k] * tn[k] - tnm1[k];
            c[i] += fv[k] * v; tnm1[k] = tn[k]; tn[k] = v;
        }
        c[i] *= 2.0 / N;
    }
    return c;
}
static inline double cheb1d_eval(const std::vector<double>& c, double xi) {
    double b1 = 0.0, b2 = 0.0;
    for (int k = (int)c.size() - 1; k >= 1; --k) { double b = 2.0 * xi * b1 - b2 + c[k]; b2 = b1; b1 = b; }
    return xi * b1 - b2 + c[0];
}
// Real roots in (-1,1) of the degree N-1 Chebyshev interpolant of f on [a,b], mapped to [a,b].
// (Chebyshev1d.hpp:460-496 finds them as colleague-matrix eigenvalues; here: sampling+bisection.)
static inline std::vector<double> cheb1d_roots(const std::function<double(double)>& f, int N, double a, double b) {
    std::vector<double> c = cheb1d_fit(f, N, a, b);
    std::vector<double> roots;
    const int S = 4000;
    double xl = -1.0, fl = cheb1d_eval(c, xl);
    for (int s = 1; s <= S; ++s) {
        double xr = -1.0 + 2.0 * s / S, fr = cheb1d_eval(c, xr);
        if (fl == 0.0 && xl > -1.0) roots.push_back(xl);
        else if ((fl < 0.0 && fr > 0.0) || (fl > 0.0 && fr < 0.0)) {
            double lo = xl, hi = xr, flo = fl;
            for (int it = 0; it < 100; ++it) {
                double mid = 0.5 * (lo + hi), fm = cheb1d_eval(c, mid);
                if ((fm < 0.0) == (flo < 0.0)) { lo = mid; flo = fm; } else hi = mid;
                if (hi - lo < 1e-15) break;
            }
            double r = 0.5 * (lo + hi);
            if (r > -1.0 && r < 1.0) roots.push_back(r);
        }
        xl = xr; fl = fr;
    }
    for (double& r : roots) r = ab2cd(r, -1, 1, a, b);
    return roots;
}

// ------------------------------------------------------------------------------------
// Brent's minimiser (BrentsMethod.hpp:42-156): returns {xmin, f(xmin)}
// ------------------------------------------------------------------------------------
static inline std::array<double, 2> brent_minimize(const std::function<double(double)>& f,
                                                   double lo, double hi,
                                                   double tol = 1e-6, int max_iter = 100) {
    const double golden = (double)0.3819660f;   // the reference stores it as a float literal
    double x, w, v, u, step = 0.0, step_prev = 0.0, fu, fv, fw, fx;
    x = w = v = hi;
    fw = fv = fx = f(x);
    int count = max_iter;
    do {
        const double mid = 0.5 * (lo + hi);
        const double tol1 = tol * std::fabs(x) + tol / 4;
        const double tol2 = 2 * tol1;
        if (std::fabs(x - mid) <= (tol2 - (hi - lo) / 2)) break;
        if (std::fabs(step_prev) > tol1) {
            double r = (x - w) * (fx - fv);
            double q = (x - v) * (fx - fw);
            double p = (x - v) * q - (x - w) * r;
            q = 2 * (q - r);
            if (q > 0) p = -p;
            q = std::fabs(q);
            const double td = step_prev;
            step_prev = step;
            if ((std::fabs(p) >= std::fabs(q * td / 2)) || (p <= q * (lo - x)) || (p >= q * (hi - x))) {
                step_prev = (x >= mid) ? lo - x : hi - x;
                step = golden * step_prev;
            } else {
                step = p / q;
                u = x + step;
                if (((u - lo) < tol2) || ((hi - u) < tol2))
                    step = (mid - x) < 0 ? -std::fabs(tol1) : std::fabs(tol1);
            }
        } else {
            step_prev = (x >= mid) ? lo - x : hi - x;
            step = golden * step_prev;
        }
        u = (std::fabs(step) >= tol1) ? x + step : (step > 0 ? x + std::fabs(tol1) : x - std::fabs(tol1));
        fu = f(u);
        if (fu <= fx) {
            if (u >= x) lo = x; else hi = x;
            v = w; w = x; x = u;
            fv = fw; fw = fx; fx = fu;
        } else {
            if (u < x) lo = u; else hi = u;
            if ((fu <= fw) || (w == x)) { v = w; w = u; fv = fw; fw = fu; }
            else if ((fu <= fv) || (v == x) || (v == w)) { v = u; fv = fu; }
        }
    } while (--count);
    return {x, fx};
}

}  // namespace orc
