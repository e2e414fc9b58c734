// oracle_fm.hpp -- CPU ORACLE (test infrastructure only; never linked into the product).
//
// Restatement of the IFGF2D geometry and forward map:
//   Geometry/Curve.hpp:20-161, Geometry/Curve.cpp:5-155   (curves, patch limits)
//   Geometry/Patch.hpp:38-88, Geometry/Patch.tpp:21-64      (patches, bounding boxes)
//   ForwardMap/GreenFunctions.hpp:36-131                     (GF, GF_far, factorization)
//   ForwardMap/ForwardMap.tpp:15-727                          (ForwardMap)
// Deviations (the reference does not compile as shipped):
//   GreenFunctions.hpp:103 `normdiff` -> the local `norm_diff`; GF_far returns its value.
//   Np is a run-time parameter instead of a template parameter.
//   An optional equal-parameter patch split (patches_per_curve > 0) sits beside the
//   reference's arc-length bisection rule (Curve.cpp:37-68).
//   A star curve r(t)=1+sum a_m cos mt + b_m sin mt is added beside Circle/Kite/Line.
#pragma once

#include "oracle_math.hpp"
#include <memory>
#include <unordered_set>
#include <unordered_map>
#include <stdexcept>

namespace orc {

enum CurveType { CURVE_CIRCLE = 0, CURVE_KITE = 1, CURVE_LINE = 2, CURVE_STAR = 3 };

struct Curve {
    int type = CURVE_CIRCLE;
    bool is_closed = true;
    double tlim1 = 0.0, tlim2 = 2.0 * PI;
    double p[16] = {0};      // circle: cx,cy,r ; kite: A,B,C,D ; line: x1,y1,x2,y2 ;
                             // star: cx, cy, M, a_1..a_M, b_1..b_M  (M <= 6)

    double xt(double t) const {
        switch (type) {
            case CURVE_CIRCLE: return p[2] * std::cos(t) + p[0];
            case CURVE_KITE: return p[0] * std::cos(t) + p[1] * std::cos(2.0 * t) + p[2];
            case CURVE_LINE: return (p[2] * (t + 1.0) - p[0] * (t - 1)) / 2.0;
            default: return p[0] + star_r(t) * std::cos(t);
        }
    }
    double yt(double t) const {
        switch (type) {
            case CURVE_CIRCLE: return p[2] * std::sin(t) + p[1];
            case CURVE_KITE: return p[3] * std::sin(t);
            case CURVE_LINE: return (p[3] * (t + 1.0) - p[1] * (t - 1)) / 2.0;
            default: return p[1] + star_r(t) * std::sin(t);
        }
    }
    double xpt(double t) const {
        switch (type) {
            case CURVE_CIRCLE: return -p[2] * std::sin(t);
            case CURVE_KITE: return -p[0] * std::sin(t) - 2.0 * p[1] * std::sin(2.0 * t);
            case CURVE_LINE: return (p[2] - p[0]) / 2.0;
            default: return star_rp(t) * std::cos(t) - star_r(t) * std::sin(t);
        }
    }
    double ypt(double t) const {
        switch (type) {
            case CURVE_CIRCLE: return p[2] * std::cos(t);
            case CURVE_KITE: return p[3] * std::cos(t);
            case CURVE_LINE: return (p[3] - p[1]) / 2.0;
            default: return star_rp(t) * std::sin(t) + star_r(t) * std::cos(t);
        }
    }
    double star_r(double t) const {
        int M = (int)p[2]; double r = 1.0;
        for (int m = 1; m <= M; ++m) r += p[2 + m] * std::cos(m * t) + p[2 + M + m] * std::sin(m * t);
        return r;
    }
    double star_rp(double t) const {
        int M = (int)p[2]; double r = 0.0;
        for (int m = 1; m <= M; ++m) r += -m * p[2 + m] * std::sin(m * t) + m * p[2 + M + m] * std::cos(m * t);
        return r;
    }
    // normal_t (Curve.hpp:97-102): (y'(t), -x'(t)), not normalised
    void normal_t(double t, double& nx, double& ny) const { nx = ypt(t); ny = -xpt(t); }

    // Curve.cpp:5-20 (200-node Fejer rule)
    double segment_length(double a, double b, const std::vector<double>& n, const std::vector<double>& w) const {
        double len = 0.0;
        for (size_t i = 0; i < n.size(); ++i) {
            double t = ab2cd(n[i], -1.0, 1.0, a, b);
            double xp = xpt(t), yp = ypt(t);
            len += std::sqrt(xp * xp + yp * yp) * w[i];
        }
        return len * ab2cdjac(-1.0, 1.0, a, b);
    }
    // Curve.cpp:23-35
    void refine(double a, double b, double lim, std::vector<double>& ends,
                const std::vector<double>& n, const std::vector<double>& w) const {
        if (segment_length(a, b, n, w) <= lim) { ends.push_back(b); return; }
        double mid = (a + b) / 2.0;
        refine(a, mid, lim, ends, n, w);
        refine(mid, b, lim, ends, n, w);
    }
    // Curve.cpp:37-68
    std::vector<double> patch_lims(double wavelengths_per_patch, double wavenumber) const {
        std::vector<double> n, w; fejer1(200, n, w);
        const double wavelength = 2 * PI / wavenumber;
        const double L = segment_length(tlim1, tlim2, n, w);
        const int num_wave_lens = (int)std::ceil(L / wavelength);
        const int num_intervals = (int)std::ceil(num_wave_lens / wavelengths_per_patch);
        std::vector<double> lims{tlim1};
        const double tl = tlim2 - tlim1;
        for (int i = 0; i < num_intervals; ++i) {
            double a = tlim1 + tl * i / (double)num_intervals;
            double b = tlim1 + tl * (i + 1) / (double)num_intervals;
            refine(a, b, wavelength * wavelengths_per_patch, lims, n, w);
        }
        return lims;
    }
};

struct Junction { int touching_curve; bool t1_touches_t1; };

// Patch.hpp:21-34, Patch.tpp:21-31
struct BoundingBox {
    double Ax = 0, Ay = 0, Bx = 0, By = 0, Cx = 0, Cy = 0, Dx = 0, Dy = 0;
    double BmAx = 0, BmAy = 0, CmBx = 0, CmBy = 0, BmA2 = 0, CmB2 = 0;
    BoundingBox() {}
    BoundingBox(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy)
        : Ax(ax), Ay(ay), Bx(bx), By(by), Cx(cx), Cy(cy), Dx(dx), Dy(dy) {
        BmAx = Bx - Ax; BmAy = By - Ay; CmBx = Cx - Bx; CmBy = Cy - By;
        BmA2 = BmAx * BmAx + BmAy * BmAy; CmB2 = CmBx * CmBx + CmBy * CmBy;
    }
    bool is_inside(double xp, double yp) const {
        double d1 = BmAx * (xp - Ax) + BmAy * (yp - Ay);
        double d2 = CmBx * (xp - Bx) + CmBy * (yp - By);
        return (0 <= d1 && d1 <= BmA2) && (0 <= d2 && d2 <= CmB2);
    }
};

struct Patch {
    double t1, t2;
    const Curve* curve;
    double delta;
    bool ist1singular = false, ist2singular = false;
    std::vector<cd> precomp;            // Np x (Np + n_ns), column-major (column j = Np moments)
    BoundingBox bbox;
    std::vector<double> point_t;        // Np parameter values
    std::vector<double> curve_jac;      // |x'(t)| (x edge jacobian on open curves)
    std::vector<double> edge_sing_jac;  // edge change-of-variables jacobian
    std::vector<long long> ns_idx;      // global indices of near-singular points
    std::vector<double> ns_t;
    std::unordered_set<long long> ns_lookup;
    std::vector<long long> ns_patches_est;

    // Patch.tpp:36-64 with Nroot = 10
    void comp_bounding_box(int Nroot = 10) {
        const Curve* c = curve;
        std::vector<double> xr = cheb1d_roots([c](double t) { return c->xpt(t); }, Nroot, t1, t2);
        std::vector<double> yr = cheb1d_roots([c](double t) { return c->ypt(t); }, Nroot, t1, t2);
        double xmin = std::min(c->xt(t1), c->xt(t2)), xmax = std::max(c->xt(t1), c->xt(t2));
        double ymin = std::min(c->yt(t1), c->yt(t2)), ymax = std::max(c->yt(t1), c->yt(t2));
        for (double r : xr) { double v = c->xt(r); xmin = std::min(xmin, v); xmax = std::max(xmax, v); }
        for (double r : yr) { double v = c->yt(r); ymin = std::min(ymin, v); ymax = std::max(ymax, v); }
        xmin -= delta; xmax += delta; ymin -= delta; ymax += delta;
        bbox = BoundingBox(xmax, ymin, xmax, ymax, xmin, ymax, xmin, ymin);
    }
};

// GreenFunctions.hpp:87-108 (SingleLayer) with the compile fix; returns 0 for r < 1e-14
static inline cd GF_SL(double p1x, double p1y, double p2x, double p2y, double k) {
    const double r = std::sqrt((p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
    if (r < 1e-14) return cd(0.0, 0.0);
    return cd(0.0, 0.25) * hankel1(0, k * r);
}
// Sound-soft combined field kernel without the jump term (not working in the reference,
// GreenFunctions.hpp:51-75; written from the Colton-Kress formulation): target t, source s with
// unit normal n_s,  dPhi/dn_s - i eta Phi = (ik/4) H1(kr) ((t - s).n_s)/r + (eta/4) H0(kr).
static inline cd GF_CF(double tx, double ty, double sx, double sy, double snx, double sny, double k, double eta) {
    const double dx = tx - sx, dy = ty - sy;
    const double r = std::sqrt(dx * dx + dy * dy);
    if (r < 1e-14) return cd(0.0, 0.0);
    return cd(0.0, 0.25 * k) * hankel1(1, k * r) * ((dx * snx + dy * sny) / r) + (0.25 * eta) * hankel1(0, k * r);
}
enum Formulation { FORM_SINGLE_LAYER = 0, FORM_COMBINED = 2 };
static inline cd GF_form(int form, double tx, double ty, double sx, double sy, double snx, double sny, double k, double eta) {
    return form == FORM_COMBINED ? GF_CF(tx, ty, sx, sy, snx, sny, k, eta) : GF_SL(tx, ty, sx, sy, k);
}

// GreenFunctions.hpp:125-131
static inline cd factorization(double r, double k) {
    return std::exp(cd(0.0, 1.0) * k * r) / std::sqrt(r);
}

struct ForwardMap {
    int Np;
    const int num_ns = 40;
    double delta, p;
    std::vector<Curve> curves;
    std::vector<std::vector<Junction>> touch;
    std::vector<Patch> patches;
    long long num_patches = 0, N = 0;
    std::vector<double> xs, ys, nxs, nys;
    std::vector<double> fej_n, fej_w, fej_ns_n, fej_ns_w;
    std::vector<std::vector<double>> chebT;         // T_n at the Np Chebyshev points
    double wavenumber = 0.0;
    int form = FORM_SINGLE_LAYER;
    double coupling = 0.0, eta = 0.0;               // eta = coupling, or k when coupling <= 0

    // ForwardMap.tpp:15-35
    ForwardMap(int Np_, double delta_, std::vector<Curve> curves_, std::vector<std::vector<Junction>> touch_,
               double wl_per_patch, double split_k, double p_, int patches_per_curve)
        : Np(Np_), delta(delta_), p(p_), curves(std::move(curves_)), touch(std::move(touch_)) {
        fejer1(Np, fej_n, fej_w);
        fejer1(num_ns, fej_ns_n, fej_ns_w);
        chebT = cheb1d_Tn(Np);
        init_points_and_patches(wl_per_patch, split_k, patches_per_curve);
        determine_patch_near_singular_points();
    }

    // ForwardMap.tpp:37-222
    void init_points_and_patches(double wl_per_patch, double split_k, int patches_per_curve_override) {
        num_patches = 0; N = 0;
        int pstart = 0;
        std::vector<int> per_curve(curves.size()), cstart(curves.size()), cend(curves.size());
        patches.clear();
        for (size_t ci = 0; ci < curves.size(); ++ci) {
            const Curve& cv = curves[ci];
            std::vector<double> lims;
            if (patches_per_curve_override > 0) {
                for (int i = 0; i <= patches_per_curve_override; ++i)
                    lims.push_back(cv.tlim1 + (cv.tlim2 - cv.tlim1) * i / (double)patches_per_curve_override);
            } else {
                lims = cv.patch_lims(wl_per_patch, split_k);
            }
            const int np = (int)lims.size() - 1;
            per_curve[ci] = np; cstart[ci] = pstart;
            num_patches += np; cend[ci] = (int)num_patches;
            N += (long long)np * Np;
            for (int pi = 0; pi < np; ++pi) {
                Patch P; P.t1 = lims[pi]; P.t2 = lims[pi + 1]; P.curve = &curves[ci]; P.delta = delta;
                P.comp_bounding_box();
                P.curve_jac.assign(Np, 0.0); P.edge_sing_jac.assign(Np, 0.0);
                if (!cv.is_closed) {
                    if (np == 1) { P.ist1singular = P.ist2singular = true; }
                    else if (pi == 0) P.ist1singular = true;
                    else if (pi == np - 1) P.ist2singular = true;
                }
                for (int j = 0; j < Np; ++j) {
                    double tm = fej_n[j];
                    if (!cv.is_closed) {
                        if (np == 1) tm = both_edge_cov(fej_n[j], p);
                        else if (pi == 0) tm = minus1_edge_cov(fej_n[j], p);
                        else if (pi == np - 1) tm = plus1_edge_cov(fej_n[j], p);
                    }
                    const double t = ab2cd(tm, -1.0, 1.0, lims[pi], lims[pi + 1]);
                    P.point_t.push_back(t);
                    double nx, ny; cv.normal_t(t, nx, ny);
                    const double nn = std::sqrt(nx * nx + ny * ny);
                    P.curve_jac[j] = nn;
                    if (!cv.is_closed) {
                        double e = 0.0; bool has = true;
                        if (np == 1) e = der_both_edge_cov(fej_n[j], p);
                        else if (pi == 0) e = der_minus1_edge_cov(fej_n[j], p);
                        else if (pi == np - 1) e = der_plus1_edge_cov(fej_n[j], p);
                        else has = false;
                        if (has) { P.edge_sing_jac[j] = e; P.curve_jac[j] *= e; }
                    }
                    xs.push_back(cv.xt(t)); ys.push_back(cv.yt(t));
                    nxs.push_back(nx / nn); nys.push_back(ny / nn);
                }
                patches.push_back(std::move(P));
            }
            pstart += np;
        }
        // adjacent-patch candidates, ForwardMap.tpp:164-219
        pstart = 0;
        for (size_t ci = 0; ci < curves.size(); ++ci) {
            const int np = per_curve[ci];
            for (int pi = 0; pi < np; ++pi) {
                auto& est = patches[pstart + pi].ns_patches_est;
                if (pi == 0) {
                    if (curves[ci].is_closed) { est.push_back(pstart + np - 1); est.push_back(pstart + pi + 1); }
                    else if (!touch.empty()) {
                        for (const Junction& J : touch[ci])
                            est.push_back(J.t1_touches_t1 ? cstart[J.touching_curve] : cend[J.touching_curve]);
                    } else if (np != 1) est.push_back(pstart + pi + 1);
                } else if (pi == np - 1) {
                    if (curves[ci].is_closed) { est.push_back(pstart + pi - 1); est.push_back(pstart); }
                    else if (!touch.empty()) {
                        for (const Junction& J : touch[ci])
                            est.push_back(J.t1_touches_t1 ? cend[J.touching_curve] : cstart[J.touching_curve]);
                    } else if (np != 1) est.push_back(pstart + pi - 1);
                } else {
                    est.push_back(pstart + pi - 1); est.push_back(pstart + pi + 1);
                }
            }
            pstart += np;
        }
    }

    // ForwardMap.tpp:224-285
    void determine_patch_near_singular_points() {
        for (long long ii = 0; ii < num_patches; ++ii) {
            Patch& P = patches[ii];
            for (long long tp : P.ns_patches_est) {
                // the junction rule can name the one-past-the-end patch of a curve (cend);
                // those indices stay as in the reference but must not read past the arrays
                if (tp < 0 || tp >= num_patches) continue;
                for (long long kk = tp * Np; kk < tp * Np + Np; ++kk) {
                    const double xp = xs[kk], yp = ys[kk];
                    if (!P.bbox.is_inside(xp, yp)) continue;
                    const Curve* c = P.curve;
                    auto f = [xp, yp, c](double t) {
                        double xt = c->xt(t), yt = c->yt(t);
                        return std::sqrt(std::fabs((xt - xp) * (xt - xp) + (yt - yp) * (yt - yp)));
                    };
                    if (f(P.t1) < delta) { P.ns_idx.push_back(kk); P.ns_lookup.insert(kk); P.ns_t.push_back(P.t1); }
                    else if (f(P.t2) < delta) { P.ns_idx.push_back(kk); P.ns_lookup.insert(kk); P.ns_t.push_back(P.t2); }
                    else {
                        std::array<double, 2> o = brent_minimize(f, P.t1, P.t2);
                        if (o[1] < delta) { P.ns_idx.push_back(kk); P.ns_lookup.insert(kk); P.ns_t.push_back(o[0]); }
                    }
                }
            }
        }
    }

    // ForwardMap.tpp:287-389: one column of rectangular-polar weights
    void single_patch_point_precomp(const Patch& P, double tsing, double xsing, double ysing, double k, cd* out) const {
        const int M = num_ns;
        std::vector<double> xi(M), dxi(M), cj(M);
        std::vector<cd> green(M);
        const double alpha = ab2cd(tsing, P.t1, P.t2, -1.0, 1.0);
        int loc = 0;
        if (std::fabs(-1.0 - alpha) < 1e-5) loc = -1;
        else if (std::fabs(1.0 - alpha) < 1e-5) loc = 1;
        for (int i = 0; i < M; ++i) {
            if (loc == 0) { xi[i] = xi_cov_center(fej_ns_n[i], alpha, p); dxi[i] = dxi_cov_center(fej_ns_n[i], alpha, p); }
            else if (loc == -1) { xi[i] = xi_cov_left(fej_ns_n[i], p); dxi[i] = dxi_cov_left(fej_ns_n[i], p); }
            else { xi[i] = xi_cov_right(fej_ns_n[i], p); dxi[i] = dxi_cov_right(fej_ns_n[i], p); }
            double g;
            if (P.ist1singular && P.ist2singular) g = ab2cd(both_edge_cov(xi[i], p), -1.0, 1.0, P.t1, P.t2);
            else if (P.ist1singular) g = ab2cd(minus1_edge_cov(xi[i], p), -1.0, 1.0, P.t1, P.t2);
            else if (P.ist2singular) g = ab2cd(plus1_edge_cov(xi[i], p), -1.0, 1.0, P.t1, P.t2);
            else g = ab2cd(xi[i], -1.0, 1.0, P.t1, P.t2);
            const double xt = P.curve->xt(g), yt = P.curve->yt(g);
            double nx, ny; P.curve->normal_t(g, nx, ny);
            cj[i] = std::sqrt(nx * nx + ny * ny);
            green[i] = GF_form(form, xsing, ysing, xt, yt, nx / cj[i], ny / cj[i], k, eta);
        }
        std::vector<cd> integ(M);
        for (int i = 0; i < M; ++i)
            integ[i] = ((P.t2 - P.t1) / 2.0) * green[i] * cj[i] * dxi[i] * fej_ns_w[i];
        cd s0 = 0.0, s1 = 0.0;
        for (int i = 0; i < M; ++i) { s0 += integ[i]; s1 += integ[i] * xi[i]; }
        out[0] = s0; if (Np > 1) out[1] = s1;
        std::vector<double> tnm1(M, 1.0), tn(xi), tnp1(M);
        for (int n = 2; n < Np; ++n) {
            cd s = 0.0;
            for (int i = 0; i < M; ++i) { tnp1[i] = 2.0 * xi[i] * tn[i] - tnm1[i]; s += integ[i] * tnp1[i]; }
            out[n] = s;
            std::swap(tnm1, tn); std::swap(tn, tnp1);
        }
    }

    // ForwardMap.tpp:391-423
    void compute_precomputations(double k) {
        wavenumber = k;
        eta = coupling > 0 ? coupling : k;
        for (long long ii = 0; ii < num_patches; ++ii) {
            Patch& P = patches[ii];
            const size_t ncol = Np + P.ns_t.size();
            P.precomp.assign(Np * ncol, cd(0.0, 0.0));
            for (int j = 0; j < Np; ++j)
                single_patch_point_precomp(P, P.point_t[j], xs[ii * Np + j], ys[ii * Np + j], k, &P.precomp[(size_t)j * Np]);
            for (size_t j = 0; j < P.ns_idx.size(); ++j)
                single_patch_point_precomp(P, P.ns_t[j], xs[P.ns_idx[j]], ys[P.ns_idx[j]], k, &P.precomp[(size_t)(Np + j) * Np]);
        }
    }

    // per-point quadrature factor (t2-t1)/2 * w_j * curve_jac_j (ForwardMap.tpp:425-435)
    void compute_intensities(std::vector<cd>& d) const {
        for (long long ii = 0; ii < num_patches; ++ii) {
            const double jac = ab2cdjac(-1, 1, patches[ii].t1, patches[ii].t2);
            for (int j = 0; j < Np; ++j) d[ii * Np + j] *= jac * fej_w[j] * patches[ii].curve_jac[j];
        }
    }

    // ForwardMap.tpp:438-478
    std::vector<cd> non_singular_unacc(const std::vector<cd>& d, double k) const {
        std::vector<cd> out(N, cd(0.0, 0.0));
        for (long long p1 = 0; p1 < num_patches; ++p1)
            for (long long xi = p1 * Np; xi < p1 * Np + Np; ++xi) {
                const double xt = xs[xi], yt = ys[xi];
                cd acc = 0.0;
                for (long long p2 = 0; p2 < num_patches; ++p2) {
                    if (p1 == p2 || patches[p2].ns_lookup.count(xi)) continue;
                    cd s = 0.0;
                    for (int j = 0; j < Np; ++j) {
                        const long long q = Np * p2 + j;
                        s += GF_form(form, xt, yt, xs[q], ys[q], nxs[q], nys[q], k, eta) * d[q];
                    }
                    acc += s;
                }
                out[xi] += acc;
            }
        return out;
    }

    // ForwardMap.tpp:481-515
    std::vector<cd> sing_near_sing(const std::vector<cd>& d) const {
        std::vector<cd> out(N, cd(0.0, 0.0));
        std::vector<cd> seg(Np), coef(Np);
        for (long long pi = 0; pi < num_patches; ++pi) {
            const Patch& P = patches[pi];
            for (int j = 0; j < Np; ++j) {
                seg[j] = d[pi * Np + j];
                if (P.ist1singular || P.ist2singular) seg[j] *= P.edge_sing_jac[j];
            }
            cheb1d_coeffs(Np, seg.data(), coef.data(), chebT);
            const size_t ncol = Np + P.ns_idx.size();
            for (size_t c = 0; c < ncol; ++c) {
                cd s = 0.0;
                for (int r = 0; r < Np; ++r) s += coef[r] * P.precomp[c * Np + r];
                if ((int)c < Np) out[pi * Np + c] += s;
                else out[P.ns_idx[c - Np]] += s;
            }
        }
        return out;
    }

    // ForwardMap.tpp:517-540
    std::vector<cd> apply_unacc(const std::vector<cd>& density) const {
        std::vector<cd> d = density;
        std::vector<cd> sns = sing_near_sing(d);
        compute_intensities(d);
        std::vector<cd> ns = non_singular_unacc(d, wavenumber);
        for (long long i = 0; i < N; ++i) sns[i] += ns[i];
        add_jump(density, sns);
        return sns;
    }

    // 1/2 I of the combined formulation (exterior limit of the double layer)
    void add_jump(const std::vector<cd>& density, std::vector<cd>& y) const {
        if (form != FORM_COMBINED) return;
        for (long long i = 0; i < N; ++i) y[i] += 0.5 * density[i];
    }

    // ForwardMap.tpp:701-727
    std::vector<cd> propagate_unacc(const std::vector<double>& xp, const std::vector<double>& yp,
                                    std::vector<cd> d, double k) const {
        compute_intensities(d);
        std::vector<cd> out(xp.size());
        for (size_t i = 0; i < xp.size(); ++i) {
            cd s = 0.0;
            for (size_t j = 0; j < xs.size(); ++j) s += d[j] * GF_form(form, xp[i], yp[i], xs[j], ys[j], nxs[j], nys[j], k, eta);
            out[i] = s;
        }
        return out;
    }
};

}  // namespace orc
