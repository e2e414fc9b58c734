// ifgf2d/opGMRES.hpp -- drop-in for IFGF2D's Eigen::opGMRES (ForwardMap/opGMRES.hpp:273-396).
//
// Include this header instead of the reference's opGMRES.hpp.  It keeps the solver's name and
// the calls ForwardMap::solve makes on it (ForwardMap.tpp:684-694): construction from the
// operator, setMaxIterations, set_restart / get_restart, setTolerance, solve, solveWithGuess,
// iterations, error and info (Success, NoConvergence or NumericalIssue, as opGMRES.hpp:385-393
// sets them).
//
// * An operator bound to a libifgf2d context (ForwardMap::linear_operator) is solved entirely
//   on the GPU by ifgf2d_solve: Arnoldi, the least-squares update and the stop test run on the
//   device, with no per-iteration copies of the mapping's vectors.
// * Any other operator (a LinearOperator over a user mapping) runs restarted GMRES on the host:
//   modified Gram-Schmidt Arnoldi and Givens rotations, one mapping call per iteration.  The
//   reference's Householder variant (opGMRES.hpp:68-269) takes the same iterations up to
//   rounding where its reflectors are Hermitian; this one is minimal-residual for complex
//   systems too.
// In both, error() is the residual estimate relative to the initial residual, and the
// iteration stops when it falls below the tolerance or after maxIterations() iterations.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

#include "LinearOperator.hpp"

#if IFGF2D_WITH_EIGEN
#include <Eigen/IterativeLinearSolvers>
#else
namespace Eigen {
struct IdentityPreconditioner {};
}  // namespace Eigen
#endif

namespace ifgf2d_cpp {

using cplx = std::complex<double>;

inline double norm2(const cplx* v, long long n) {
    double s = 0.0;
    for (long long i = 0; i < n; ++i) s += std::norm(v[i]);
    return std::sqrt(s);
}

// Rotation [c s; -conj(s) c] (c real) taking (a, b) to (r, 0).
inline void givens(cplx a, cplx b, double& c, cplx& s, cplx& r) {
    const double ab = std::abs(b);
    if (ab == 0.0) { c = 1.0; s = 0.0; r = a; return; }
    const double aa = std::abs(a);
    const double nu = std::hypot(aa, ab);
    if (aa == 0.0) { c = 0.0; s = std::conj(b) / ab; r = ab; return; }
    const cplx phase = a / aa;
    c = aa / nu;
    s = phase * std::conj(b) / nu;
    r = phase * nu;
}

// Restarted GMRES on a mapping-only operator: x holds the initial guess on entry.  Returns
// false on a breakdown that leaves no usable update.  iters: iterations run; err: the
// residual estimate over the initial residual norm.
template <typename Op>
bool host_gmres(const Op& A, const Vector& b, Vector& x, long long restart, long long max_iters, double tol,
                long long& iters, double& err) {
    const long long n = (long long)b.size();
    iters = 0;
    err = 0.0;
    if (norm2(b.data(), n) <= 0.0) {
        for (long long i = 0; i < n; ++i) x[i] = 0.0;
        return true;
    }
    const long long m = std::max(1LL, std::min(restart, n));
    Vector r = A * x;
    for (long long i = 0; i < n; ++i) r[i] = b[i] - r[i];
    const double r0 = norm2(r.data(), n);
    if (r0 == 0.0) return true;
    std::vector<cplx> V((size_t)n * (size_t)(m + 1)), H((size_t)(m + 1) * (size_t)m), g((size_t)m + 1), sn((size_t)m), y((size_t)m);
    std::vector<double> cs((size_t)m);
    Vector v(n);
    double beta = r0;
    while (true) {
        for (long long i = 0; i < n; ++i) V[(size_t)i] = r[i] / beta;
        std::fill(g.begin(), g.end(), cplx(0.0));
        g[0] = beta;
        long long k = 0;
        bool stop = false;
        for (long long j = 0; j < m; ++j) {
            for (long long i = 0; i < n; ++i) v[i] = V[(size_t)j * n + i];
            Vector w = A * v;
            ++iters;
            cplx* h = &H[(size_t)j * (m + 1)];
            for (long long q = 0; q <= j; ++q) {          // modified Gram-Schmidt
                const cplx* vq = &V[(size_t)q * n];
                cplx d = 0.0;
                for (long long i = 0; i < n; ++i) d += std::conj(vq[i]) * w[i];
                h[q] = d;
                for (long long i = 0; i < n; ++i) w[i] -= d * vq[i];
            }
            const double hn = norm2(w.data(), n);
            for (long long q = 0; q < j; ++q) {            // earlier rotations on the new column
                const cplx t = cs[q] * h[q] + sn[q] * h[q + 1];
                h[q + 1] = -std::conj(sn[q]) * h[q] + cs[q] * h[q + 1];
                h[q] = t;
            }
            cplx rr;
            givens(h[j], cplx(hn), cs[j], sn[j], rr);
            h[j] = rr;
            h[j + 1] = 0.0;
            g[j + 1] = -std::conj(sn[j]) * g[j];
            g[j] = cs[j] * g[j];
            err = std::abs(g[j + 1]) / r0;
            k = j + 1;
            stop = err < tol || iters >= max_iters || k >= n || hn == 0.0;
            if (stop || j + 1 == m) break;
            for (long long i = 0; i < n; ++i) V[(size_t)(j + 1) * n + i] = w[i] / hn;
        }
        for (long long i = k - 1; i >= 0; --i) {           // back-substitution, R y = g
            cplx s = g[i];
            for (long long q = i + 1; q < k; ++q) s -= H[(size_t)q * (m + 1) + i] * y[q];
            const cplx d = H[(size_t)i * (m + 1) + i];
            if (d == 0.0) return false;
            y[i] = s / d;
        }
        for (long long q = 0; q < k; ++q)
            for (long long i = 0; i < n; ++i) x[i] += y[q] * V[(size_t)q * n + i];
        if (stop) return true;
        r = A * x;                                          // restart from the true residual
        for (long long i = 0; i < n; ++i) r[i] = b[i] - r[i];
        beta = norm2(r.data(), n);
        if (beta == 0.0) { err = 0.0; return true; }
    }
}

}  // namespace ifgf2d_cpp

namespace Eigen {

template <typename MatrixType, typename Preconditioner = IdentityPreconditioner>
class opGMRES {
  public:
    typedef typename MatrixType::Scalar Scalar;
    typedef typename MatrixType::RealScalar RealScalar;

    opGMRES() = default;
    explicit opGMRES(const MatrixType& A) : mat_(&A) {}
    opGMRES& compute(const MatrixType& A) { mat_ = &A; return *this; }

    Index get_restart() { return restart_; }
    void set_restart(const Index restart) { restart_ = restart; }
    opGMRES& setMaxIterations(Index max_iters) { max_iters_ = max_iters; return *this; }
    Index maxIterations() const { return max_iters_ > 0 ? max_iters_ : 2 * (mat_ ? (Index)mat_->cols() : 0); }
    opGMRES& setTolerance(const RealScalar& tol) { tol_ = tol; return *this; }
    RealScalar tolerance() const { return tol_; }

    Index iterations() const { return iters_; }
    RealScalar error() const { return error_; }
    ComputationInfo info() const { return info_; }

    ifgf2d_cpp::Vector solve(const ifgf2d_cpp::Vector& b) const {
        ifgf2d_cpp::Vector x(b.size());
        for (long long i = 0; i < (long long)b.size(); ++i) x[i] = 0.0;
        run(b, x, false);
        return x;
    }
    ifgf2d_cpp::Vector solveWithGuess(const ifgf2d_cpp::Vector& b, const ifgf2d_cpp::Vector& x0) const {
        ifgf2d_cpp::Vector x = x0;
        run(b, x, true);
        return x;
    }

  private:
    const MatrixType* mat_ = nullptr;
    Index restart_ = 30;
    Index max_iters_ = -1;
    RealScalar tol_ = 1e-16;
    mutable Index iters_ = 0;
    mutable RealScalar error_ = 0;
    mutable ComputationInfo info_ = Success;

    void run(const ifgf2d_cpp::Vector& b, ifgf2d_cpp::Vector& x, bool guess) const {
        if (!mat_) throw std::logic_error("opGMRES: no operator (construct with the operator or call compute)");
        if ((long long)b.size() != (long long)mat_->rows()) throw std::invalid_argument("opGMRES: right-hand side has the wrong length");
        const long long maxit = (long long)maxIterations();
        ifgf2d_ctx* ctx = mat_->device_context();
        if (!ctx) {
            long long it = 0;
            double err = 0.0;
            const bool ok = ifgf2d_cpp::host_gmres(*mat_, b, x, (long long)restart_, maxit, (double)tol_, it, err);
            iters_ = (Index)it;
            error_ = err;
            info_ = !ok ? NumericalIssue : err <= tol_ ? Success : NoConvergence;
            return;
        }
        // On the device: ifgf2d_solve starts from zero, so a guess is handled as a correction
        // A d = b - A x0, whose residual estimate is relative to the same initial residual.
        ifgf2d_cpp::Vector rhs = b;
        if (guess) {
            ifgf2d_cpp::Vector ax = (*mat_) * x;
            for (long long i = 0; i < (long long)b.size(); ++i) rhs[i] = b[i] - ax[i];
        }
        ifgf2d_cpp::Vector d(b.size());
        int it = 0;
        double err = 0.0;
        const int restart = (int)std::min<long long>(std::max<long long>(1, (long long)restart_), maxit);
        const int rc = ifgf2d_solve(ctx, reinterpret_cast<const double*>(rhs.data()), reinterpret_cast<double*>(d.data()),
                                    mat_->apply_mode(), (double)tol_, restart, (int)maxit, &it, &err);
        if (rc != IFGF2D_OK && rc != IFGF2D_ERR_NOCONV) {
            const std::string msg = std::string("opGMRES: ") + ifgf2d_last_error(ctx);
            if (rc == IFGF2D_ERR_ARG) throw std::invalid_argument(msg);
            throw std::logic_error(msg);
        }
        if (guess)
            for (long long i = 0; i < (long long)b.size(); ++i) x[i] += d[i];
        else
            x = d;
        iters_ = (Index)it;
        error_ = err;
        info_ = rc == IFGF2D_OK ? Success : NoConvergence;
    }
};

}  // namespace Eigen
