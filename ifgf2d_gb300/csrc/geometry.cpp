// geometry.cpp -- host discretisation of the boundary (see geometry.hpp for the reference map).
#include "geometry.hpp"
#include "host_threads.hpp"
#include <algorithm>
#include <cstring>

namespace ifgf {

// ---------------------------------------------------------------- curves (Curve.cpp:104-155)
static double star_r(const double* p, double t, double& dr) {
    const int M = (int)p[2];
    double r = 1.0; dr = 0.0;
    for (int m = 1; m <= M; ++m) {
        const double c = std::cos(m * t), s = std::sin(m * t);
        r += p[2 + m] * c + p[2 + M + m] * s;
        dr += -m * p[2 + m] * s + m * p[2 + M + m] * c;
    }
    return r;
}
double HostCurve::x(double t) const {
    double dr;
    switch (type) {
        case IFGF2D_CURVE_CIRCLE: return p[2] * std::cos(t) + p[0];
        case IFGF2D_CURVE_KITE: return p[0] * std::cos(t) + p[1] * std::cos(2.0 * t) + p[2];
        case IFGF2D_CURVE_LINE: return (p[2] * (t + 1.0) - p[0] * (t - 1)) / 2.0;
        default: return p[0] + star_r(p, t, dr) * std::cos(t);
    }
}
double HostCurve::y(double t) const {
    double dr;
    switch (type) {
        case IFGF2D_CURVE_CIRCLE: return p[2] * std::sin(t) + p[1];
        case IFGF2D_CURVE_KITE: return p[3] * std::sin(t);
        case IFGF2D_CURVE_LINE: return (p[3] * (t + 1.0) - p[1] * (t - 1)) / 2.0;
        default: return p[1] + star_r(p, t, dr) * std::sin(t);
    }
}
double HostCurve::xp(double t) const {
    double dr, r;
    switch (type) {
        case IFGF2D_CURVE_CIRCLE: return -p[2] * std::sin(t);
        case IFGF2D_CURVE_KITE: return -p[0] * std::sin(t) - 2.0 * p[1] * std::sin(2.0 * t);
        case IFGF2D_CURVE_LINE: return (p[2] - p[0]) / 2.0;
        default: r = star_r(p, t, dr); return dr * std::cos(t) - r * std::sin(t);
    }
}
double HostCurve::yp(double t) const {
    double dr, r;
    switch (type) {
        case IFGF2D_CURVE_CIRCLE: return p[2] * std::cos(t);
        case IFGF2D_CURVE_KITE: return p[3] * std::cos(t);
        case IFGF2D_CURVE_LINE: return (p[3] - p[1]) / 2.0;
        default: r = star_r(p, t, dr); return dr * std::sin(t) + r * std::cos(t);
    }
}

double HostCurve::curvature(double t) const {
    double xpp = 0.0, ypp = 0.0;
    switch (type) {
        case IFGF2D_CURVE_CIRCLE: xpp = -p[2] * std::cos(t); ypp = -p[2] * std::sin(t); break;
        case IFGF2D_CURVE_KITE: xpp = -p[0] * std::cos(t) - 4.0 * p[1] * std::cos(2.0 * t); ypp = -p[3] * std::sin(t); break;
        case IFGF2D_CURVE_LINE: return 0.0;
        default: {
            const int M = (int)p[2];
            double r = 1.0, dr = 0.0, ddr = 0.0;
            for (int m = 1; m <= M; ++m) {
                const double c = std::cos(m * t), s = std::sin(m * t);
                r += p[2 + m] * c + p[2 + M + m] * s;
                dr += -m * p[2 + m] * s + m * p[2 + M + m] * c;
                ddr += -m * m * (p[2 + m] * c + p[2 + M + m] * s);
            }
            const double c = std::cos(t), s = std::sin(t);
            xpp = ddr * c - 2.0 * dr * s - r * c;
            ypp = ddr * s + 2.0 * dr * c - r * s;
        }
    }
    const double a = xp(t), b = yp(t);
    const double sp = std::sqrt(a * a + b * b);
    return (a * ypp - b * xpp) / (sp * sp * sp);
}

// ---------------------------------------------------------------- quadrature (Quadrature.hpp)
static inline double lin_map(double x, double a, double b, double c, double d) { return ((d - c) / (b - a)) * (x - a) + c; }

void fejer_rule(int n, std::vector<double>& nodes, std::vector<double>& weights) {
    nodes.resize(n); weights.resize(n);
    for (int i = 0; i < n; ++i) {
        nodes[i] = std::cos(kPiH * (2.0 * i + 1.0) / (2.0 * n));
        double s = 0.0;
        for (int j = 1; j <= n / 2; ++j) s += std::cos(j * kPiH * (2.0 * i + 1.0) / n) / (4.0 * j * j - 1.0);
        weights[i] = (2.0 / n) * (1.0 - 2.0 * s);
    }
}
// w change of variables of the rectangular-polar method and its derivative
static double vfun(double t, double p) { const double a = t / kPiH - 1.0; return (0.5 - 1.0 / p) * std::pow(a, 3) + (1.0 / p) * a + 0.5; }
static double vpfun(double t, double p) { const double a = t / kPiH - 1.0; return (3.0 / kPiH) * (0.5 - 1.0 / p) * std::pow(a, 2.0) + 1.0 / (p * kPiH); }
static double wfun(double t, double p) { const double a = std::pow(vfun(t, p), p); return 2.0 * kPiH * a / (a + std::pow(vfun(2 * kPiH - t, p), p)); }
static double wpfun(double t, double p) {
    const double a = vfun(t, p), b = vfun(2 * kPiH - t, p);
    return 2.0 * kPiH * p * vpfun(t, p) * std::pow(a, p - 1.0) * std::pow(b, p - 1.0) /
           std::pow(std::pow(a, p) + std::pow(b, p), 2.0);
}
static double edge_both(double t, double p) { return -1.0 + (1.0 / kPiH) * wfun(kPiH * (t + 1.0), p); }
static double edge_m1(double t, double p) { return -1.0 + 2.0 * (1.0 / kPiH) * wfun((kPiH / 2.0) * (t + 1.0), p); }
static double edge_p1(double t, double p) { return -3.0 + 2.0 * (1.0 / kPiH) * wfun(kPiH + (kPiH / 2.0) * (t + 1), p); }
static double dedge_both(double t, double p) { return wpfun(kPiH * (t + 1.0), p); }
static double dedge_p1(double t, double p) { return wpfun(kPiH + (kPiH / 2.0) * (t + 1), p); }

// ---------------------------------------------------------------- patch limits (Curve.cpp:5-68)
static double arc_length(const HostCurve& c, double a, double b, const std::vector<double>& n, const std::vector<double>& w) {
    double s = 0.0;
    for (size_t i = 0; i < n.size(); ++i) {
        const double t = lin_map(n[i], -1.0, 1.0, a, b);
        const double u = c.xp(t), v = c.yp(t);
        s += std::sqrt(u * u + v * v) * w[i];
    }
    return s * ((b - a) / 2.0);
}
static void bisect_to_length(const HostCurve& c, double a, double b, double lim, std::vector<double>& ends,
                             const std::vector<double>& n, const std::vector<double>& w) {
    if (arc_length(c, a, b, n, w) <= lim) { ends.push_back(b); return; }
    const double m = (a + b) / 2.0;
    bisect_to_length(c, a, m, lim, ends, n, w);
    bisect_to_length(c, m, b, lim, ends, n, w);
}
static std::vector<double> patch_limits(const HostCurve& c, double wl_per_patch, double k, int equal_split) {
    std::vector<double> lims{c.tlim1};
    if (equal_split > 0) {
        for (int i = 1; i <= equal_split; ++i) lims.push_back(c.tlim1 + (c.tlim2 - c.tlim1) * i / (double)equal_split);
        return lims;
    }
    std::vector<double> n, w; fejer_rule(200, n, w);
    const double lambda = 2 * kPiH / k;
    const double L = arc_length(c, c.tlim1, c.tlim2, n, w);
    const int nwl = (int)std::ceil(L / lambda);
    const int nint = (int)std::ceil(nwl / wl_per_patch);
    const double span = c.tlim2 - c.tlim1;
    // the intervals bisect independently: in parallel, then concatenated in order
    std::vector<std::vector<double>> part(std::max(nint, 0));
    parallel_for(nint, [&](long long i0, long long i1) {
        for (long long i = i0; i < i1; ++i)
            bisect_to_length(c, c.tlim1 + span * i / (double)nint, c.tlim1 + span * (i + 1) / (double)nint,
                             lambda * wl_per_patch, part[i], n, w);
    }, 1);
    for (const auto& q : part) lims.insert(lims.end(), q.begin(), q.end());
    return lims;
}

// ---------------------------------------------------------------- bounding box (Patch.tpp:36-64)
// Extremes of x(t), y(t) on [t1,t2] at the real roots of the degree-9 Chebyshev interpolant
// of x'(t), y'(t) (Chebyshev1d.hpp:460-496 finds them as colleague-matrix eigenvalues; here
// by sign changes of the same interpolant on a fine grid, then bisection).
static void interp_roots(const std::function<double(double)>& f, double a, double b, std::vector<double>& roots) {
    const int N = 10;
    double xs[N], fv[N], c[N];
    for (int i = 0; i < N; ++i) { xs[i] = std::cos(kPiH * (2.0 * i + 1.0) / (2.0 * N)); fv[i] = f(lin_map(xs[i], -1, 1, a, b)); }
    for (int i = 0; i < N; ++i) c[i] = 0.0;
    double tm1[N], t0[N];
    for (int k = 0; k < N; ++k) { tm1[k] = 1.0; t0[k] = xs[k]; c[0] += fv[k]; c[1] += fv[k] * xs[k]; }
    c[0] *= 1.0 / N; c[1] *= 2.0 / N;
    for (int i = 2; i < N; ++i) {
        for (int k = 0; k < N; ++k) { const double v = 2.0 * xs[k] * t0[k] - tm1[k]; c[i] += fv[k] * v; tm1[k] = t0[k]; t0[k] = v; }
        c[i] *= 2.0 / N;
    }
    auto ev = [&](double z) {
        double b1 = 0.0, b2 = 0.0;
        for (int k = N - 1; k >= 1; --k) { const double bb = 2.0 * z * b1 - b2 + c[k]; b2 = b1; b1 = bb; }
        return z * b1 - b2 + c[0];
    };
    const int S = 4000;
    // Grid steps over which the interpolant cannot change sign are skipped: |f'| <= M =
    // sum k^2 |c_k| on [-1, 1] (Markov), so from a point where |f| > 2 g + M h j the next j
    // steps keep |f| > g, and g = 1e-12 sum |c_k| is far above the evaluation's rounding error.
    // The points evaluated, and the roots, are those of the full scan.
    double M = 0.0, A = 0.0;
    for (int k = 0; k < N; ++k) { M += (double)k * k * std::fabs(c[k]); A += std::fabs(c[k]); }
    M = M * (1.0 + 1e-12) + 1e-300;
    const double g = 1e-12 * A, h = 2.0 / S;
    double zl = -1.0, fl = ev(zl);
    for (int s = 1; s <= S; ++s) {
        const double room = std::fabs(fl) - 2.0 * g;
        if (room > 0.0) {
            const double j = std::floor(room / (M * h));
            if (j >= 2.0) {
                const int skip = (int)std::min<double>(j - 1.0, (double)(S - s));
                if (skip > 0) {
                    s += skip;
                    zl = -1.0 + 2.0 * (s - 1) / S;
                    fl = ev(zl);
                }
            }
        }
        const double zr = -1.0 + 2.0 * s / S, fr = ev(zr);
        if (fl == 0.0 && zl > -1.0) roots.push_back(lin_map(zl, -1, 1, a, b));
        else if ((fl < 0.0 && fr > 0.0) || (fl > 0.0 && fr < 0.0)) {
            double lo = zl, hi = zr, flo = fl;
            for (int it = 0; it < 100 && hi - lo >= 1e-15; ++it) {
                const double m = 0.5 * (lo + hi), fm = ev(m);
                if ((fm < 0.0) == (flo < 0.0)) { lo = m; flo = fm; } else hi = m;
            }
            const double r = 0.5 * (lo + hi);
            if (r > -1.0 && r < 1.0) roots.push_back(lin_map(r, -1, 1, a, b));
        }
        zl = zr; fl = fr;
    }
}

struct Box4 { double ax, ay, bx, by, cx, cy, bax, bay, cbx, cby, ba2, cb2; };
static Box4 patch_box(const HostCurve& c, double t1, double t2, double delta) {
    std::vector<double> rx, ry;
    interp_roots([&](double t) { return c.xp(t); }, t1, t2, rx);
    interp_roots([&](double t) { return c.yp(t); }, t1, t2, ry);
    double x0 = std::min(c.x(t1), c.x(t2)), x1 = std::max(c.x(t1), c.x(t2));
    double y0 = std::min(c.y(t1), c.y(t2)), y1 = std::max(c.y(t1), c.y(t2));
    for (double r : rx) { const double v = c.x(r); x0 = std::min(x0, v); x1 = std::max(x1, v); }
    for (double r : ry) { const double v = c.y(r); y0 = std::min(y0, v); y1 = std::max(y1, v); }
    x0 -= delta; x1 += delta; y0 -= delta; y1 += delta;
    // corners A = (x1, y0), B = (x1, y1), C = (x0, y1) as in Patch.tpp:62-63
    Box4 b{x1, y0, x1, y1, x0, y1, 0, 0, 0, 0, 0, 0};
    b.bax = b.bx - b.ax; b.bay = b.by - b.ay; b.cbx = b.cx - b.bx; b.cby = b.cy - b.by;
    b.ba2 = b.bax * b.bax + b.bay * b.bay; b.cb2 = b.cbx * b.cbx + b.cby * b.cby;
    return b;
}
static bool box_contains(const Box4& b, double x, double y) {
    const double d1 = b.bax * (x - b.ax) + b.bay * (y - b.ay);
    const double d2 = b.cbx * (x - b.bx) + b.cby * (y - b.by);
    return 0 <= d1 && d1 <= b.ba2 && 0 <= d2 && d2 <= b.cb2;
}

// ---------------------------------------------------------------- Brent (BrentsMethod.hpp:42-156)
// Brent's localmin with golden-section fallback; the step sequence is kept identical to
// the reference because the returned t feeds the rectangular-polar weights.
static void brent_min(const std::function<double(double)>& f, double lo, double hi, double& xmin, double& fmin) {
    const double tol = 1e-6, g = (double)0.3819660f;
    double x = hi, w = hi, v = hi, u, fx = f(x), fw = fx, fv = fx, fu, d = 0.0, e = 0.0;
    for (int it = 100; it > 0; --it) {
        const double mid = 0.5 * (lo + hi), t1 = tol * std::fabs(x) + tol / 4, t2 = 2 * t1;
        if (std::fabs(x - mid) <= t2 - (hi - lo) / 2) break;
        bool golden = true;
        if (std::fabs(e) > t1) {
            double r = (x - w) * (fx - fv), q = (x - v) * (fx - fw), pp = (x - v) * q - (x - w) * r;
            q = 2 * (q - r);
            if (q > 0) pp = -pp;
            q = std::fabs(q);
            const double eold = e;
            e = d;
            if (!(std::fabs(pp) >= std::fabs(q * eold / 2) || pp <= q * (lo - x) || pp >= q * (hi - x))) {
                golden = false;
                d = pp / q; u = x + d;
                if ((u - lo) < t2 || (hi - u) < t2) d = (mid - x) < 0 ? -std::fabs(t1) : std::fabs(t1);
            }
        }
        if (golden) { e = (x >= mid) ? lo - x : hi - x; d = g * e; }
        u = std::fabs(d) >= t1 ? x + d : (d > 0 ? x + std::fabs(t1) : x - std::fabs(t1));
        fu = f(u);
        if (fu <= fx) {
            if (u >= x) lo = x; else hi = x;
            v = w; w = x; x = u; fv = fw; fw = fx; fx = fu;
        } else {
            if (u < x) lo = u; else hi = u;
            if (fu <= fw || w == x) { v = w; w = u; fv = fw; fw = fu; }
            else if (fu <= fv || v == x || v == w) { v = u; fv = fu; }
        }
    }
    xmin = x; fmin = fx;
}

// ---------------------------------------------------------------- discretise (ForwardMap.tpp:15-285)
std::string discretise(const ifgf2d_curve* curves, int ncurves, const ifgf2d_junction* junctions, int njunctions,
                       const ifgf2d_options& opt, Discretisation& D) {
    if (ncurves <= 0 || !curves) return "no curves";
    if (opt.Np < 2 || opt.Np > 64) return "Np must be in [2, 64]";
    if (!(opt.delta > 0)) return "delta must be > 0";
    if (opt.patches_per_curve <= 0 && (!(opt.wavelengths_per_patch > 0) || !(opt.patch_split_wavenumber > 0)))
        return "wavelengths_per_patch and patch_split_wavenumber must be > 0";
    const int Np = opt.Np;
    D = Discretisation();
    D.Np = Np; D.delta = opt.delta; D.p = opt.p > 0 ? opt.p : 4.0;
    const double p = D.p;
    fejer_rule(Np, D.fej_n, D.fej_w);
    fejer_rule(40, D.fej_ns_n, D.fej_ns_w);
    D.curves.resize(ncurves);
    for (int c = 0; c < ncurves; ++c) {
        HostCurve& h = D.curves[c];
        h.type = curves[c].type; h.closed = curves[c].closed != 0;
        h.tlim1 = curves[c].tlim1; h.tlim2 = curves[c].tlim2;
        std::memcpy(h.p, curves[c].params, sizeof(h.p));
        if (h.type < 0 || h.type > IFGF2D_CURVE_STAR) return "unknown curve type";
        if (h.type == IFGF2D_CURVE_STAR && (h.p[2] < 0 || h.p[2] > 6)) return "star curve: M must be in [0, 6]";
        if (!(h.tlim2 > h.tlim1)) return "tlim2 must exceed tlim1";
    }
    std::vector<std::vector<ifgf2d_junction>> touch;
    if (njunctions > 0) {
        touch.resize(ncurves);
        for (int j = 0; j < njunctions; ++j) {
            const ifgf2d_junction& J = junctions[j];
            if (J.curve < 0 || J.curve >= ncurves || J.touching_curve < 0 || J.touching_curve >= ncurves) return "bad junction";
            touch[J.curve].push_back(J);
        }
    }
    const bool on_device = opt.device_geometry != 0;
    std::vector<int> per(ncurves), first(ncurves), past(ncurves);
    for (int c = 0; c < ncurves; ++c) {
        const HostCurve& cv = D.curves[c];
        std::vector<double> lims = patch_limits(cv, opt.wavelengths_per_patch, opt.patch_split_wavenumber, opt.patches_per_curve);
        const int np = (int)lims.size() - 1;
        if (np < 1) return "curve produced no patches";
        per[c] = np; first[c] = (int)D.num_patches; D.num_patches += np; past[c] = (int)D.num_patches;
        for (int pi = 0; pi < np; ++pi) {
            const double a = lims[pi], b = lims[pi + 1];
            D.t1.push_back(a); D.t2.push_back(b); D.curve_of.push_back(c);
            const bool open = !cv.closed;
            const int s1 = open && (np == 1 || pi == 0), s2 = open && (np == 1 || pi == np - 1);
            D.ist1sing.push_back(s1); D.ist2sing.push_back(s2);
        }
    }
    D.N = D.num_patches * Np;
    // the points of each patch (Patch.tpp), patches in parallel
    if (!on_device) {
        for (auto* v : {&D.x, &D.y, &D.kappa, &D.nx, &D.ny, &D.t, &D.wq, &D.edge_jac}) v->resize(D.N);
        D.patch_of.resize(D.N);
        parallel_for(D.num_patches, [&](long long p0, long long p1) {
            for (long long pid = p0; pid < p1; ++pid) {
                const HostCurve& cv = D.curves[D.curve_of[pid]];
                const double a = D.t1[pid], b = D.t2[pid];
                const int s1 = D.ist1sing[pid], s2 = D.ist2sing[pid];
                for (int j = 0; j < Np; ++j) {
                    const long long i = pid * Np + j;
                    const double z = D.fej_n[j];
                    double tm = z, ej = 0.0;
                    if (s1 && s2) { tm = edge_both(z, p); ej = dedge_both(z, p); }
                    else if (s1) { tm = edge_m1(z, p); ej = dedge_both(z, p); }
                    else if (s2) { tm = edge_p1(z, p); ej = dedge_p1(z, p); }
                    const double t = lin_map(tm, -1.0, 1.0, a, b);
                    const double nx = cv.yp(t), ny = -cv.xp(t);
                    const double nn = std::sqrt(nx * nx + ny * ny);
                    double cj = nn;
                    if (s1 || s2) cj *= ej;
                    D.x[i] = cv.x(t); D.y[i] = cv.y(t);
                    D.kappa[i] = cv.curvature(t);
                    D.nx[i] = nx / nn; D.ny[i] = ny / nn;
                    D.t[i] = t;
                    D.wq[i] = ((b - a) / 2.0) * D.fej_w[j] * cj;
                    D.edge_jac[i] = ej;
                    D.patch_of[i] = (int)pid;
                }
            }
        }, 64);
    }
    // candidate patches (ForwardMap.tpp:164-219); junction entries keep the reference's
    // `curve_patches_end` index, which names the patch after the touching curve
    std::vector<std::vector<long long>> cand(D.num_patches);
    for (int c = 0; c < ncurves; ++c) {
        const int np = per[c], s = first[c];
        for (int pi = 0; pi < np; ++pi) {
            auto& e = cand[s + pi];
            const bool closed = D.curves[c].closed;
            if (pi == 0) {
                if (closed) { e.push_back(s + np - 1); e.push_back(s + pi + 1); }
                else if (!touch.empty()) { for (auto& J : touch[c]) e.push_back(J.t1_touches_t1 ? first[J.touching_curve] : past[J.touching_curve]); }
                else if (np != 1) e.push_back(s + pi + 1);
            } else if (pi == np - 1) {
                if (closed) { e.push_back(s + pi - 1); e.push_back(s); }
                else if (!touch.empty()) { for (auto& J : touch[c]) e.push_back(J.t1_touches_t1 ? past[J.touching_curve] : first[J.touching_curve]); }
                else if (np != 1) e.push_back(s + pi - 1);
            } else { e.push_back(s + pi - 1); e.push_back(s + pi + 1); }
        }
    }
    // points, bounding boxes and near-singular points on the GPU (geometry_device.cu)
    if (on_device) return discretise_on_device(D, cand);
    // patch bounding boxes (Patch.tpp:36-64), one per patch, independent of each other
    std::vector<Box4> boxes(D.num_patches);
    parallel_for(D.num_patches, [&](long long p0, long long p1) {
        for (long long pi = p0; pi < p1; ++pi) boxes[pi] = patch_box(D.curves[D.curve_of[pi]], D.t1[pi], D.t2[pi], D.delta);
    }, 16);
    // near-singular points (ForwardMap.tpp:224-285), per patch in parallel, then concatenated
    std::vector<std::vector<std::pair<long long, double>>> found(D.num_patches);
    parallel_for(D.num_patches, [&](long long p0, long long p1) {
        for (long long pi = p0; pi < p1; ++pi) {
            const HostCurve& cv = D.curves[D.curve_of[pi]];
            const double a = D.t1[pi], b = D.t2[pi];
            for (long long tp : cand[pi]) {
                if (tp < 0 || tp >= D.num_patches) continue;
                for (long long kk = tp * Np; kk < tp * Np + Np; ++kk) {
                    const double xp = D.x[kk], yp = D.y[kk];
                    if (!box_contains(boxes[pi], xp, yp)) continue;
                    auto dist = [&](double t) {
                        const double dx = cv.x(t) - xp, dy = cv.y(t) - yp;
                        return std::sqrt(std::fabs(dx * dx + dy * dy));
                    };
                    double tsing, dmin;
                    if (dist(a) < D.delta) tsing = a;
                    else if (dist(b) < D.delta) tsing = b;
                    else { brent_min(dist, a, b, tsing, dmin); if (!(dmin < D.delta)) continue; }
                    found[pi].push_back({kk, tsing});
                }
            }
        }
    }, 16);
    D.ns_ptr.assign(D.num_patches + 1, 0);
    for (long long pi = 0; pi < D.num_patches; ++pi) {
        for (auto& f : found[pi]) { D.ns_idx.push_back(f.first); D.ns_t.push_back(f.second); }
        D.ns_ptr[pi + 1] = (int)D.ns_idx.size();
    }
    return "";
}

}  // namespace ifgf
