// dropin_check.cpp -- a program written against the reference's ForwardMap / LinearOperator /
// opGMRES interface, built against include/ifgf2d/ForwardMap.hpp.
//
// Writes to the file named by argv[1], as interleaved doubles:
//   y = A x with the IFGF (compute_Ax_acc) and directly (compute_Ax_unacc) for a fixed density,
//   then three GMRES solutions of the combined-field equation A x = b for a plane wave b:
//   * a LinearOperator over a user mapping, solved by Eigen::opGMRES in the way
//     ForwardMap::solve drives it (host GMRES, one GPU apply per iteration);
//   * the operator of ForwardMap::linear_operator, solved by the same opGMRES (all on the GPU);
//   * ForwardMap::solve.
// It also checks the exception behaviour: nlevels < 3 and a wavenumber other than the
// precomputed one throw std::invalid_argument.
#include <cstdio>
#include <fstream>
#include <iostream>
#include "ifgf2d/ForwardMap.hpp"

using FM_t = ForwardMap<16, FormulationType::SingleLayer, 5, 5>;
using FC_t = ForwardMap<16, FormulationType::Combined, 5, 5>;

// A caller-side solve in the shape of ForwardMap::solve (ForwardMap.tpp:658-697): set-up, a
// mapping lambda over compute_Ax_acc, a LinearOperator around it, opGMRES configured with the
// map's GMRES settings.
static Eigen::VectorXcd user_solve(FC_t& fm, const Eigen::VectorXcd& rhs, std::complex<double> k, int nlevels, int& iters,
                                   double& err) {
    BoxTree<5, 5> boxes;
    fm.precomps_and_setup(k, nlevels, boxes);
    auto mapping = [&fm, &boxes](const Eigen::VectorXcd& x, Eigen::VectorXcd& y) { fm.compute_Ax_acc(x, y, boxes); };
    LinearOperator op((int)rhs.size(), (int)rhs.size(), mapping);
    Eigen::opGMRES<LinearOperator> gmres(op);
    gmres.setMaxIterations(fm.GMRES_MAX_ITER_);
    gmres.set_restart(fm.GMRES_MAX_ITER_);
    gmres.setTolerance(fm.GMRES_TOLERANCE_);
    Eigen::VectorXcd x = gmres.solve(rhs);
    iters = (int)gmres.iterations();
    err = gmres.error();
    if (gmres.info() != Eigen::Success) throw std::runtime_error("user solve did not converge");
    return x;
}

template <typename V>
static void put(std::ofstream& f, const V& v) {
    f.write(reinterpret_cast<const char*>(v.data()), sizeof(std::complex<double>) * v.size());
}

int main(int argc, char** argv) {
    if (argc < 2) { std::cerr << "usage: dropin_check out.bin\n"; return 2; }
    const double k = 100.0;
    std::vector<std::unique_ptr<Curve>> curves;
    curves.emplace_back(std::make_unique<Kite>());
    std::vector<std::vector<Junction>> touch;
    FM_t FM(0.01, std::move(curves), touch, 1.0, k, 4.0, /*patches_per_curve*/ 64);
    if (FM.curves_.size() != 1 || (long long)FM.patches_.size() != FM.num_patches_) { std::cerr << "members\n"; return 1; }
    BoxTree<5, 5> boxes;
    FM.precomps_and_setup(k, 0, boxes);
    const long long n = FM.total_num_unknowns_;
    Eigen::VectorXcd x(n), y_acc, y_unacc;
    for (long long j = 0; j < n; ++j) x[j] = std::complex<double>(std::cos(0.1 * j), std::sin(0.2 * j));
    FM.compute_Ax_acc(x, y_acc, boxes);
    FM.compute_Ax_unacc(x, y_unacc, k);
    std::ofstream f(argv[1], std::ios::binary);
    put(f, y_acc);
    put(f, y_unacc);
    // LinearOperator as ForwardMap::solve builds it
    LinearOperator A = FM.linear_operator(boxes);
    Eigen::VectorXcd y_op = A * x;
    double d = 0.0;
    for (long long i = 0; i < n; ++i) d = std::max(d, std::abs(y_op[i] - y_acc[i]));
    if (d != 0.0) { std::cerr << "LinearOperator differs from compute_Ax_acc\n"; return 1; }

    // three solves of the combined-field equation A x = b (second kind, so GMRES converges in
    // a few dozen iterations), b a plane wave
    std::vector<std::unique_ptr<Curve>> curves_c;
    curves_c.emplace_back(std::make_unique<Kite>());
    FC_t FC(0.01, std::move(curves_c), touch, 1.0, k, 4.0, /*patches_per_curve*/ 64);
    Eigen::VectorXcd b(n);
    for (long long j = 0; j < n; ++j) b[j] = -std::exp(std::complex<double>(0.0, k * FC.xs_[j]));
    FC.GMRES_TOLERANCE_ = 1e-8;
    int it_user = 0;
    double err_user = 0.0;
    Eigen::VectorXcd x_user = user_solve(FC, b, k, 0, it_user, err_user);
    BoxTree<5, 5> boxes_c;
    FC.precomps_and_setup(k, 0, boxes_c);
    LinearOperator Ac = FC.linear_operator(boxes_c);
    Eigen::opGMRES<LinearOperator> gmres(Ac);
    gmres.setMaxIterations(300);
    gmres.set_restart(300);
    gmres.setTolerance(1e-8);
    Eigen::VectorXcd x_dev = gmres.solve(b);
    if (gmres.info() != Eigen::Success) { std::cerr << "device opGMRES did not converge\n"; return 1; }
    Eigen::VectorXcd x_solve = FC.solve(b, k, 0, true);
    const int it_solve = FC.last_iterations();
    const double err_solve = FC.last_error();
    Eigen::VectorXcd x_pre = FC.solve_preconditioned(b, k, 0);   // the chosen form, same tolerance
    put(f, x_user);
    put(f, x_dev);
    put(f, x_solve);
    put(f, x_pre);
    const double meta[8] = {(double)it_user, err_user, (double)gmres.iterations(), gmres.error(), (double)it_solve,
                            err_solve, (double)FC.last_iterations(), FC.last_error()};
    f.write(reinterpret_cast<const char*>(meta), sizeof(meta));

    // the reference throws std::invalid_argument for nlevels < 3 (BoxTree.h:1024-1025)
    bool threw = false;
    try { FM.precomps_and_setup(k, 2, boxes); } catch (const std::invalid_argument&) { threw = true; }
    if (!threw) { std::cerr << "nlevels < 3 did not throw\n"; return 1; }
    // the operator belongs to the precomputed wavenumber
    threw = false;
    try { FM.compute_Ax_unacc(x, y_unacc, 2.0 * k); } catch (const std::invalid_argument&) { threw = true; }
    if (!threw) { std::cerr << "a second wavenumber did not throw\n"; return 1; }
    std::printf("dropin ok: N=%lld nlevels=%d iterations user %d device %d solve %d preconditioned %d\n", n, boxes.nlevels(),
                it_user, (int)gmres.iterations(), it_solve, FC.last_iterations());
    return 0;
}
