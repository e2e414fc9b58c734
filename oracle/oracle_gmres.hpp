// oracle_gmres.hpp -- CPU ORACLE (test infrastructure only; never linked into the product).
//
// Householder-Arnoldi GMRES with Givens rotations (Walker 1988), restated from
// ForwardMap/opGMRES.hpp:68-269 (`internal::opgmres`, identity preconditioner) and the
// opGMRES wrapper (:323-396): initial guess 0, stopping test |w(k)|/||r0|| < tol,
// restart after `restart` steps.  Householder and Givens conventions follow Eigen's
// makeHouseholder / applyHouseholderOnTheLeft / JacobiRotation::makeGivens.
//
// With complex tau the reflector H = I - tau u u^H is unitary but not Hermitian, and the
// reference applies H (not H^{-1} = H^H) when it forms the basis vector P_1..P_k e_k and the
// update (opGMRES.hpp:147-149, 224-229).  The iteration stays consistent (estimate = true
// residual) but is not the minimal-residual one.  exact_adjoint = true applies H^H there,
// which gives the minimal-residual (textbook GMRES) iterates; false restates the reference.
#pragma once

#include "oracle_math.hpp"
#include <functional>
#include <limits>

namespace orc {

// x (length n) -> H x = beta e_1, H = I - tau u u^H, u = [1; ess]
static inline void make_householder(const cd* x, long long n, cd* ess, cd& tau, double& beta) {
    double tail2 = 0.0;
    for (long long i = 1; i < n; ++i) tail2 += std::norm(x[i]);
    const cd c0 = x[0];
    const double tiny = std::numeric_limits<double>::min();
    if (tail2 <= tiny && c0.imag() * c0.imag() <= tiny) {
        tau = 0.0; beta = c0.real();
        for (long long i = 1; i < n; ++i) ess[i - 1] = 0.0;
    } else {
        beta = std::sqrt(std::norm(c0) + tail2);
        if (c0.real() >= 0.0) beta = -beta;
        for (long long i = 1; i < n; ++i) ess[i - 1] = x[i] / (c0 - beta);
        tau = std::conj((beta - c0) / beta);
    }
}
static inline void apply_householder(cd* y, long long n, const cd* ess, cd tau) {
    if (n == 1) { y[0] *= (1.0 - tau); return; }
    cd t = y[0];
    for (long long i = 1; i < n; ++i) t += std::conj(ess[i - 1]) * y[i];
    y[0] -= tau * t;
    for (long long i = 1; i < n; ++i) y[i] -= tau * ess[i - 1] * t;
}

struct Givens { cd c = 1.0, s = 0.0; };
// Eigen JacobiRotation::makeGivens (complex): G^* [p; q] = [r; 0]
static inline Givens make_givens(cd p, cd q) {
    Givens g;
    if (q == cd(0.0)) { g.c = p.real() < 0 ? -1.0 : 1.0; g.s = 0.0; }
    else if (p == cd(0.0)) { g.c = 0.0; g.s = -q / std::abs(q); }
    else {
        double p1 = std::fabs(p.real()) + std::fabs(p.imag());
        double q1 = std::fabs(q.real()) + std::fabs(q.imag());
        if (p1 >= q1) {
            cd ps = p / p1; double p2 = std::norm(ps);
            cd qs = q / p1; double q2 = std::norm(qs);
            double u = std::sqrt(1.0 + q2 / p2);
            if (p.real() < 0) u = -u;
            g.c = 1.0 / u;
            g.s = -qs * std::conj(ps) * (g.c / p2);
        } else {
            cd ps = p / q1; double p2 = std::norm(ps);
            cd qs = q / q1; double q2 = std::norm(qs);
            double u = q1 * std::sqrt(p2 + q2);
            if (p.real() < 0) u = -u;
            p1 = std::abs(p);
            ps = p / p1;
            g.c = p1 / u;
            g.s = -std::conj(ps) * (q / u);
        }
    }
    return g;
}
// (x, y) <- G^* (x, y), with G = [c, conj(s); -s, conj(c)] (Eigen's JacobiRotation)
static inline void apply_givens_adj(const Givens& g, cd& x, cd& y) {
    const cd nx = std::conj(g.c) * x - std::conj(g.s) * y;
    const cd ny = g.s * x + g.c * y;
    x = nx; y = ny;
}

struct GmresResult { bool ok; long long iters; double error; long long matvecs; };

static inline GmresResult householder_gmres(const std::function<void(const std::vector<cd>&, std::vector<cd>&)>& A,
                                            const std::vector<cd>& rhs, std::vector<cd>& x,
                                            long long restart, long long max_iters, double tol,
                                            bool exact_adjoint = false) {
    const long long m = (long long)rhs.size();
    GmresResult R{true, 0, 0.0, 0};
    x.assign(m, 0.0);
    double bn = 0.0; for (auto& v : rhs) bn += std::norm(v);
    if (std::sqrt(bn) <= std::numeric_limits<double>::min()) { R.error = 0; return R; }
    std::vector<cd> t(m), v(m), r0(m), xnew(m);
    A(x, t); R.matvecs++;
    for (long long i = 0; i < m; ++i) r0[i] = rhs[i] - t[i];
    double r0n = 0.0; for (auto& z : r0) r0n += std::norm(z); r0n = std::sqrt(r0n);
    if (r0n == 0.0) { R.error = 0; return R; }
    std::vector<cd> H((size_t)m * (restart + 1), cd(0.0)), w(restart + 1, 0.0), tau(restart + 1, 0.0);
    std::vector<Givens> G(restart);
    auto col = [&](long long c) { return &H[(size_t)c * m]; };
    double beta;
    make_householder(r0.data(), m, col(0) + 1, tau[0], beta);
    w[0] = beta;
    for (long long k = 1; k <= restart; ++k) {
        ++R.iters;
        std::fill(v.begin(), v.end(), cd(0.0)); v[k - 1] = 1.0;
        for (long long i = k - 1; i >= 0; --i)
            apply_householder(&v[i], m - i, col(i) + i + 1, exact_adjoint ? std::conj(tau[i]) : tau[i]);
        A(v, t); R.matvecs++;
        v = t;
        for (long long i = 0; i < k; ++i) apply_householder(&v[i], m - i, col(i) + i + 1, tau[i]);
        double tn = 0.0; for (long long i = k; i < m; ++i) tn += std::norm(v[i]);
        if (k < m && tn != 0.0) {
            make_householder(&v[k], m - k, col(k) + k + 1, tau[k], beta);
            apply_householder(&v[k], m - k, col(k) + k + 1, tau[k]);
        }
        for (long long i = 0; i + 1 < k; ++i) apply_givens_adj(G[i], v[i], v[i + 1]);
        if (k < m && v[k] != cd(0.0)) {
            G[k - 1] = make_givens(v[k - 1], v[k]);
            apply_givens_adj(G[k - 1], v[k - 1], v[k]);
            apply_givens_adj(G[k - 1], w[k - 1], w[k]);
        }
        for (long long i = 0; i < k; ++i) col(k - 1)[i] = v[i];
        R.error = std::abs(w[k]) / r0n;
        const bool stop = (k == m || R.error < tol || R.iters == max_iters);
        if (stop || k == restart) {
            std::vector<cd> y(w.begin(), w.begin() + k);
            for (long long i = k - 1; i >= 0; --i) {
                cd s = y[i];
                for (long long j = i + 1; j < k; ++j) s -= col(j)[i] * y[j];
                y[i] = s / col(i)[i];
            }
            std::fill(xnew.begin(), xnew.end(), cd(0.0));
            for (long long i = k - 1; i >= 0; --i) {
                xnew[i] += y[i];
                apply_householder(&xnew[i], m - i, col(i) + i + 1, exact_adjoint ? std::conj(tau[i]) : tau[i]);
            }
            for (long long i = 0; i < m; ++i) x[i] += xnew[i];
            if (stop) return R;
            k = 0;
            A(x, t); R.matvecs++;
            for (long long i = 0; i < m; ++i) r0[i] = rhs[i] - t[i];
            std::fill(H.begin(), H.end(), cd(0.0));
            std::fill(w.begin(), w.end(), cd(0.0));
            std::fill(tau.begin(), tau.end(), cd(0.0));
            make_householder(r0.data(), m, col(0) + 1, tau[0], beta);
            w[0] = beta;
        }
    }
    R.ok = false;
    return R;
}

}  // namespace orc
