// dropin_check.cpp -- a program written against the reference's ForwardMap interface, built
// against include/ifgf2d/ForwardMap.hpp.  Writes y = A x (IFGF and direct) for a fixed density
// to the file named by argv[1] as interleaved doubles, then checks the exception behaviour.
#include <cstdio>
#include <fstream>
#include <iostream>
#include "ifgf2d/ForwardMap.hpp"

int main(int argc, char** argv) {
    if (argc < 2) { std::cerr << "usage: dropin_check out.bin\n"; return 2; }
    const double k = 100.0;
    std::vector<std::unique_ptr<Curve>> curves;
    curves.emplace_back(std::make_unique<Kite>());
    std::vector<std::vector<Junction>> touch;
    ForwardMap<16, FormulationType::SingleLayer, 5, 5> FM(0.01, std::move(curves), touch, 1.0, k, 4.0, /*patches_per_curve*/ 64);
    BoxTree<5, 5> boxes;
    FM.precomps_and_setup(k, 0, boxes);
    ifgf2d_cpp::Vector x(FM.total_num_unknowns_), y_acc, y_unacc;
    for (long long j = 0; j < FM.total_num_unknowns_; ++j) x[j] = std::complex<double>(std::cos(0.1 * j), std::sin(0.2 * j));
    FM.compute_Ax_acc(x, y_acc, boxes);
    FM.compute_Ax_unacc(x, y_unacc, k);
    std::ofstream f(argv[1], std::ios::binary);
    f.write(reinterpret_cast<const char*>(y_acc.data()), sizeof(std::complex<double>) * y_acc.size());
    f.write(reinterpret_cast<const char*>(y_unacc.data()), sizeof(std::complex<double>) * y_unacc.size());
    // LinearOperator as ForwardMap::solve builds it
    LinearOperator A = FM.linear_operator(boxes);
    ifgf2d_cpp::Vector y_op = A * x;
    double d = 0.0;
    for (size_t i = 0; i < y_op.size(); ++i) d = std::max(d, std::abs(y_op[i] - y_acc[i]));
    if (d != 0.0) { std::cerr << "LinearOperator differs from compute_Ax_acc\n"; return 1; }
    // the reference throws std::invalid_argument for nlevels < 3 (BoxTree.h:1024-1025)
    bool threw = false;
    try { FM.precomps_and_setup(k, 2, boxes); } catch (const std::invalid_argument&) { threw = true; }
    if (!threw) { std::cerr << "nlevels < 3 did not throw\n"; return 1; }
    std::printf("dropin ok: N=%lld nlevels=%d\n", FM.total_num_unknowns_, boxes.nlevels());
    return 0;
}
