// ifgf2d/ForwardMap.hpp -- header-only C++ drop-in for IFGF2D's ForwardMap, over the C ABI.
//
// Keeps the reference's class interface (ForwardMap/ForwardMap.hpp:49-177,
// ForwardMap/LinearOperator.hpp:27-58 in ifgf2d/LinearOperator.hpp, the opGMRES solver of
// ForwardMap/opGMRES.hpp:273-396 in ifgf2d/opGMRES.hpp, Geometry/Curve.hpp:10-161,
// IFGF_Source/BoxTree.h) so that code written against the reference compiles against this
// header:
//
//   std::vector<std::unique_ptr<Curve>> curves;
//   curves.emplace_back(std::make_unique<Kite>());
//   ForwardMap<16, FormulationType::SingleLayer, 5, 5> FM(0.01, std::move(curves), {}, 1.0, k);
//   BoxTree<5, 5> boxes;
//   FM.precomps_and_setup(k, nlevels, boxes);
//   FM.compute_Ax_acc(x, y, boxes);            // y = A x on the GPU
//
// Vectors are Eigen::VectorXcd when Eigen is available (as in the reference), otherwise
// std::vector<std::complex<double>>.  Errors throw std::logic_error / std::invalid_argument like
// the reference; BoxTree is an opaque handle (the device tree lives in the ForwardMap's context).
// The operator is fixed by the wavenumber of the last compute_precomputations /
// precomps_and_setup: compute_Ax_unacc and propagate_unacc throw std::invalid_argument when
// called with another one (the reference would mix the two wavenumbers, ForwardMap.tpp:517-540).
// Link with -lifgf2d.
#pragma once

#include <complex>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#include <cmath>

#include "../ifgf2d.h"
#include "LinearOperator.hpp"
#include "opGMRES.hpp"

// FormulationType (ForwardMap/GreenFunctions.hpp:15-20).  SingleLayer and Combined are
// supported; Combined is the sound-soft combined field operator (1/2 I + K - i eta S).
enum class FormulationType { SingleLayer, DoubleLayer, Combined, ThreeD };

// Junction (Geometry/Curve.hpp:10-17)
struct Junction {
    int touching_curve;
    bool t1_touches_t1;
    Junction(int touching_curve, bool t1_touches_t1) : touching_curve(touching_curve), t1_touches_t1(t1_touches_t1) {}
};

// Curves (Geometry/Curve.hpp:20-161): descriptors of the device-side parametrisations
class Curve {
  public:
    bool is_closed;
    double tlim1, tlim2;
    virtual ~Curve() = default;
    ifgf2d_curve descriptor() const {
        ifgf2d_curve c{};
        c.type = type_; c.closed = is_closed ? 1 : 0; c.tlim1 = tlim1; c.tlim2 = tlim2;
        for (int i = 0; i < 16; ++i) c.params[i] = params_[i];
        return c;
    }
  protected:
    Curve(int type, bool closed, double t1, double t2) : is_closed(closed), tlim1(t1), tlim2(t2), type_(type) {}
    int type_;
    double params_[16] = {0};
};
class Circle : public Curve {
  public:
    double centerx, centery, radius;
    Circle(bool /*is_closed*/ = true, double /*tlim1*/ = 0, double /*tlim2*/ = 2.0 * M_PI, double cx = 0.0, double cy = 0.0,
           double r = 1.0)
        : Curve(IFGF2D_CURVE_CIRCLE, true, 0.0, 2.0 * M_PI), centerx(cx), centery(cy), radius(r) {
        params_[0] = cx; params_[1] = cy; params_[2] = r;
    }
};
class Kite : public Curve {
  public:
    double A, B, C, D;
    Kite(bool is_closed = true, double t1 = 0, double t2 = 2.0 * M_PI, double A = 1.0, double B = 0.65, double C = -0.65,
         double D = 1.5)
        : Curve(IFGF2D_CURVE_KITE, is_closed, t1, t2), A(A), B(B), C(C), D(D) {
        params_[0] = A; params_[1] = B; params_[2] = C; params_[3] = D;
    }
};
class Line : public Curve {
  public:
    double x1, y1, x2, y2;
    Line(double x1, double y1, double x2, double y2) : Curve(IFGF2D_CURVE_LINE, false, -1.0, 1.0), x1(x1), y1(y1), x2(x2), y2(y2) {
        params_[0] = x1; params_[1] = y1; params_[2] = x2; params_[3] = y2;
    }
};
// r(t) = 1 + sum_m a_m cos mt + b_m sin mt, m <= 6 (not in the reference)
class Star : public Curve {
  public:
    Star(const std::vector<double>& a, const std::vector<double>& b, double cx = 0.0, double cy = 0.0)
        : Curve(IFGF2D_CURVE_STAR, true, 0.0, 2.0 * M_PI) {
        if (a.size() != b.size() || a.size() > 6) throw std::invalid_argument("Star: a, b must have equal length <= 6");
        const int M = (int)a.size();
        params_[0] = cx; params_[1] = cy; params_[2] = M;
        for (int m = 0; m < M; ++m) { params_[3 + m] = a[m]; params_[3 + M + m] = b[m]; }
    }
};

// BoxTree<Ps, Pang> (IFGF_Source/BoxTree.h:24-1171): opaque; the device tree belongs to the
// ForwardMap context, this object only records that precomps_and_setup ran with it.
template <int Ps = 5, int Pang = 5>
class BoxTree {
  public:
    BoxTree() = default;
    int nlevels() const { return nlevels_; }
    const std::vector<long long>& getSorting() const { return sorting_; }
    std::vector<long long> getInverse() const {
        std::vector<long long> inv(sorting_.size());
        for (size_t i = 0; i < sorting_.size(); ++i) inv[sorting_[i]] = (long long)i;
        return inv;
    }
    int nlevels_ = 0;
    std::vector<long long> sorting_;
};

// Patch<Nroot> (Geometry/Patch.hpp:36-110): the parameter limits and near-singular lists of
// one patch, as the device discretisation computed them.  The rectangular-polar matrix
// (precomputations_) stays on the device; ForwardMap::precomputations(patch) reads it.
template <int N>
struct Patch {
    double t1 = 0.0, t2 = 0.0;
    double delta = 0.0;
    std::vector<long long> near_singular_point_indices_;
    std::vector<double> near_singular_point_ts_;
};

template <int Np, FormulationType Formulation, int Ps = 5, int Pang = 5, int Nroot = 10>
class ForwardMap {
    static_assert(Formulation == FormulationType::SingleLayer || Formulation == FormulationType::Combined,
                  "ifgf2d supports the single layer and the combined field formulations");
  public:
    using Vec = ifgf2d_cpp::Vector;

    std::vector<Patch<Nroot>> patches_;
    long long num_patches_ = 0;
    long long total_num_unknowns_ = 0;
    double delta_;
    std::vector<std::unique_ptr<Curve>> curves_;
    std::vector<std::vector<Junction>> curve_touch_tracker_;
    double p_;
    double eta_ = 0.0;                   // coupling of Combined (<= 0: eta = wavenumber)
    std::vector<double> xs_, ys_, nxs_, nys_;
    int GMRES_MAX_ITER_ = 300;
    double GMRES_TOLERANCE_ = 1e-10;

    // ForwardMap.tpp:15-35
    ForwardMap(double delta, std::vector<std::unique_ptr<Curve>> curves, const std::vector<std::vector<Junction>>& touch,
               double wavelengths_per_patch, double patch_split_wavenumber, double p = 4, int patches_per_curve = 0,
               double eta = 0.0, bool device_geometry = false)
        : delta_(delta), curve_touch_tracker_(touch), p_(p), eta_(eta) {
        std::vector<ifgf2d_curve> cs;
        for (auto& c : curves) cs.push_back(c->descriptor());
        std::vector<ifgf2d_junction> js;
        for (size_t c = 0; c < touch.size(); ++c)
            for (const Junction& j : touch[c]) js.push_back(ifgf2d_junction{(int)c, j.touching_curve, j.t1_touches_t1 ? 1 : 0});
        ifgf2d_options o{};
        o.Np = Np; o.delta = delta; o.wavelengths_per_patch = wavelengths_per_patch;
        o.patch_split_wavenumber = patch_split_wavenumber; o.p = p; o.patches_per_curve = patches_per_curve;
        o.Ps = Ps; o.Pang = Pang;
        o.formulation = Formulation == FormulationType::Combined ? IFGF2D_COMBINED : IFGF2D_SINGLE_LAYER;
        o.coupling = eta;
        o.device_geometry = device_geometry ? 1 : 0;
        ifgf2d_ctx* ctx = nullptr;
        const int rc = ifgf2d_create(cs.data(), (int)cs.size(), js.empty() ? nullptr : js.data(), (int)js.size(), &o, &ctx);
        ctx_.reset(ctx);
        check(rc);
        curves_ = std::move(curves);
        total_num_unknowns_ = ifgf2d_num_unknowns(ctx);
        num_patches_ = ifgf2d_num_patches(ctx);
        const size_t n = (size_t)total_num_unknowns_;
        xs_.resize(n); ys_.resize(n); nxs_.resize(n); nys_.resize(n);
        check(ifgf2d_get_points(ctx, xs_.data(), ys_.data(), nxs_.data(), nys_.data()));
        // patches_: limits and near-singular lists (ForwardMap.tpp:37-285)
        std::vector<double> t12(2 * (size_t)num_patches_);
        std::vector<long long> cnt((size_t)num_patches_);
        check(ifgf2d_get_patches(ctx, t12.data(), cnt.data()));
        long long tot = 0;
        for (long long c : cnt) tot += c;
        std::vector<long long> idx((size_t)std::max(tot, 1LL));
        std::vector<double> tv((size_t)std::max(tot, 1LL));
        check(ifgf2d_get_near_singular(ctx, idx.data(), tv.data()));
        patches_.resize((size_t)num_patches_);
        long long o0 = 0;
        for (long long q = 0; q < num_patches_; ++q) {
            Patch<Nroot>& P = patches_[(size_t)q];
            P.t1 = t12[2 * q]; P.t2 = t12[2 * q + 1]; P.delta = delta;
            P.near_singular_point_indices_.assign(idx.begin() + o0, idx.begin() + o0 + cnt[q]);
            P.near_singular_point_ts_.assign(tv.begin() + o0, tv.begin() + o0 + cnt[q]);
            o0 += cnt[q];
        }
    }

    // ForwardMap.tpp:391-423
    void compute_precomputations(std::complex<double> wavenumber) {
        const double k = real_k(wavenumber);
        check(ifgf2d_precompute(ctx_.get(), k));
        k_ = k;
    }
    // patch p's precomputations_ (Patch.hpp:55): Np x (Np + n_ns), column-major
    Vec precomputations(long long patch) {
        if (patch < 0 || patch >= num_patches_) throw std::invalid_argument("patch index out of range");
        Vec m((size_t)Np * (Np + patches_[(size_t)patch].near_singular_point_indices_.size()));
        check(ifgf2d_get_precomputations(ctx_.get(), patch, reinterpret_cast<double*>(m.data())));
        return m;
    }
    // ForwardMap.tpp:542-565 (nlevels <= 0: the deepest tree passing the neighbourhood check)
    void precomps_and_setup(std::complex<double> wavenumber, int nlevels, BoxTree<Ps, Pang>& boxes) {
        const double k = real_k(wavenumber);
        check(ifgf2d_setup(ctx_.get(), k, nlevels));
        k_ = k;
        boxes.nlevels_ = ifgf2d_get_nlevels(ctx_.get());
        boxes.sorting_.resize((size_t)total_num_unknowns_);
        check(ifgf2d_get_sorting(ctx_.get(), boxes.sorting_.data()));
    }
    // ForwardMap.tpp:517-540
    void compute_Ax_unacc(const Vec& density, Vec& out, std::complex<double> wavenumber) {
        same_k(wavenumber, "compute_Ax_unacc");
        apply(density, out, IFGF2D_APPLY_DIRECT);
    }
    Vec compute_Ax_unacc(const Vec& density, std::complex<double> k) { Vec y; compute_Ax_unacc(density, y, k); return y; }
    // ForwardMap.tpp:609-655
    void compute_Ax_acc(const Vec& density, Vec& out, BoxTree<Ps, Pang>& /*boxes*/) { apply(density, out, IFGF2D_APPLY_IFGF); }
    Vec compute_Ax_acc(const Vec& density, BoxTree<Ps, Pang>& boxes) { Vec y; compute_Ax_acc(density, y, boxes); return y; }
    // ForwardMap.tpp:658-697: set-up, then GMRES on the device (initial guess 0)
    Vec solve(const Vec& rhs, std::complex<double> wavenumber, int nlevels = 5, bool accelerated = true) {
        BoxTree<Ps, Pang> boxes;
        if (accelerated) precomps_and_setup(wavenumber, nlevels, boxes);
        else compute_precomputations(wavenumber);
        LinearOperator B = linear_operator(boxes, accelerated);
        Eigen::opGMRES<LinearOperator> func(B);
        func.setMaxIterations(GMRES_MAX_ITER_);
        func.set_restart(GMRES_MAX_ITER_);
        func.setTolerance(GMRES_TOLERANCE_);
        Vec x = func.solve(rhs);
        last_iters_ = (int)func.iterations();
        last_error_ = func.error();
        return x;
    }
    // Not in the reference: the solve above in the chosen form.  complex64 inner solves inside FP64
    // iterative refinement (the stop test is the FP64 relative residual, GMRES_TOLERANCE_), with
    // the spectral right preconditioner in flexible GMRES (ifgf2d_solve_flexible).  The same
    // answer within the tolerance, in fewer iterations; combined formulation and closed curves
    // only (std::invalid_argument otherwise).
    Vec solve_preconditioned(const Vec& rhs, std::complex<double> wavenumber, int nlevels = 5) {
        BoxTree<Ps, Pang> boxes;
        precomps_and_setup(wavenumber, nlevels, boxes);
        if ((long long)rhs.size() != total_num_unknowns_) throw std::invalid_argument("rhs has the wrong length");
        Vec x(rhs.size());
        int it = 0;
        double err = 0.0;
        const int rc = ifgf2d_solve_flexible(ctx_.get(), nullptr, IFGF2D_PRECOND_SPECTRAL, reinterpret_cast<const double*>(rhs.data()),
                                             reinterpret_cast<double*>(x.data()), IFGF2D_APPLY_IFGF_MIXED, GMRES_TOLERANCE_,
                                             GMRES_MAX_ITER_, GMRES_MAX_ITER_, &it, &err);
        if (rc != IFGF2D_OK && rc != IFGF2D_ERR_NOCONV) check(rc);
        last_iters_ = it;
        last_error_ = err;
        return x;
    }
    // ForwardMap.tpp:701-727
    Vec propagate_unacc(const std::vector<double> x_prop, const std::vector<double> y_prop, Vec density,
                        std::complex<double> wavenumber) {
        same_k(wavenumber, "propagate_unacc");
        if (x_prop.size() != y_prop.size()) throw std::invalid_argument("x_prop and y_prop differ in length");
        if ((long long)density.size() != total_num_unknowns_) throw std::invalid_argument("density has the wrong length");
        Vec out(x_prop.size());
        check(ifgf2d_propagate(ctx_.get(), (long long)x_prop.size(), x_prop.data(), y_prop.data(),
                               reinterpret_cast<const double*>(density.data()), reinterpret_cast<double*>(out.data())));
        return out;
    }
    // The operator ForwardMap::solve hands to GMRES (ForwardMap.tpp:673-682), bound to this map's
    // context so that Eigen::opGMRES (ifgf2d/opGMRES.hpp) solves it on the GPU.
    LinearOperator linear_operator(BoxTree<Ps, Pang>& boxes, bool accelerated = true) {
        return LinearOperator((int)total_num_unknowns_, (int)total_num_unknowns_,
                              [this, &boxes, accelerated](const Vec& x, Vec& y) {
                                  if (accelerated) compute_Ax_acc(x, y, boxes);
                                  else compute_Ax_unacc(x, y, k_);
                              },
                              ctx_.get(), accelerated ? IFGF2D_APPLY_IFGF : IFGF2D_APPLY_DIRECT);
    }
    double wavenumber() const { return k_; }
    int last_iterations() const { return last_iters_; }
    double last_error() const { return last_error_; }
    ifgf2d_ctx* context() { return ctx_.get(); }

  private:
    struct Deleter { void operator()(ifgf2d_ctx* c) const { if (c) ifgf2d_destroy(c); } };
    std::unique_ptr<ifgf2d_ctx, Deleter> ctx_;
    double k_ = 0.0;                     // wavenumber of the current operator (0: none yet)
    int last_iters_ = 0;
    double last_error_ = 0.0;

    static double real_k(std::complex<double> k) {
        if (k.imag() != 0.0) throw std::invalid_argument("ifgf2d: the wavenumber must be real");
        return k.real();
    }
    // the operator's singular corrections were computed for k_; another wavenumber is an error
    void same_k(std::complex<double> wavenumber, const char* who) const {
        const double k = real_k(wavenumber);
        if (k_ == 0.0) throw std::logic_error(std::string("ifgf2d: ") + who + " before compute_precomputations");
        if (k != k_)
            throw std::invalid_argument(std::string("ifgf2d: ") + who + " called with wavenumber " + std::to_string(k) +
                                        ", but the operator was precomputed for " + std::to_string(k_));
    }
    void apply(const Vec& x, Vec& y, int mode) {
        if ((long long)x.size() != total_num_unknowns_) throw std::invalid_argument("density has the wrong length");
        y.resize(x.size());
        check(ifgf2d_apply(ctx_.get(), reinterpret_cast<const double*>(x.data()), reinterpret_cast<double*>(y.data()), mode));
    }
    void check(int rc) {
        if (rc == IFGF2D_OK) return;
        const std::string msg = std::string("ifgf2d: ") + (ctx_ ? ifgf2d_last_error(ctx_.get()) : "error");
        if (rc == IFGF2D_ERR_ARG || rc == IFGF2D_ERR_NLEVELS) throw std::invalid_argument(msg);
        throw std::logic_error(msg);
    }
};
