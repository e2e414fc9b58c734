// ifgf2d/LinearOperator.hpp -- drop-in for IFGF2D's LinearOperator (ForwardMap/LinearOperator.hpp:27-58).
//
// A matrix-free operator: rows, cols and a mapping(x, out).  With Eigen on the include path it
// derives from Eigen::EigenBase with the Scalar / RealScalar / StorageIndex / StorageKind
// typedefs and evalTo the reference declares, so Eigen-style solvers accept it as they accept
// the reference's.  Without Eigen, vectors are std::vector<std::complex<double>> and a minimal
// Eigen namespace (VectorXcd, Index, ComputationInfo) lets code written against the reference
// compile unchanged.
//
// Beyond the reference: an operator made by ForwardMap::linear_operator() also carries its
// libifgf2d context and apply mode, so ifgf2d/opGMRES.hpp runs the whole GMRES on the GPU
// (ifgf2d_solve) instead of calling the mapping once per iteration from the host.
#pragma once

#include <complex>
#include <cstddef>
#include <functional>
#include <vector>

#include "../ifgf2d.h"

#if __has_include(<Eigen/Dense>)
#include <Eigen/Dense>
#define IFGF2D_WITH_EIGEN 1
namespace ifgf2d_cpp { using Vector = Eigen::VectorXcd; }
class LinearOperator;
namespace Eigen {
namespace internal {
// the storage traits Eigen reads through EigenBase<LinearOperator> (LinearOperator.hpp:12-22)
template <>
struct traits<LinearOperator> {
    typedef Eigen::Dense StorageKind;
    typedef int StorageIndex;
};
}  // namespace internal
}  // namespace Eigen
#else
#define IFGF2D_WITH_EIGEN 0
namespace ifgf2d_cpp { using Vector = std::vector<std::complex<double>>; }
// The names of Eigen that code written against the reference uses around the forward map.
namespace Eigen {
using VectorXcd = ifgf2d_cpp::Vector;
using Index = std::ptrdiff_t;
enum ComputationInfo { Success = 0, NumericalIssue = 1, NoConvergence = 2, InvalidInput = 3 };
}  // namespace Eigen
#endif

#if IFGF2D_WITH_EIGEN
class LinearOperator : public Eigen::EigenBase<LinearOperator> {
#else
class LinearOperator {
#endif
  public:
    typedef std::complex<double> Scalar;
    typedef double RealScalar;
    typedef int StorageIndex;
#if IFGF2D_WITH_EIGEN
    typedef Eigen::Dense StorageKind;
#endif
    enum { ColsAtCompileTime = 0 };
    enum { MaxColsAtCompileTime = 0 };
    using Vec = ifgf2d_cpp::Vector;

    // LinearOperator.cpp:3-9
    LinearOperator(int rows, int cols, const std::function<void(const Vec&, Vec&)>& mapping)
        : rows_(rows), cols_(cols), mapping_(mapping) {}
    // the same, bound to a libifgf2d context and apply mode (IFGF2D_APPLY_*)
    LinearOperator(int rows, int cols, const std::function<void(const Vec&, Vec&)>& mapping, ifgf2d_ctx* ctx, int mode)
        : rows_(rows), cols_(cols), mapping_(mapping), ctx_(ctx), mode_(mode) {}

    // an operator is never formed densely (LinearOperator.hpp:36-37)
    template <typename Dest>
    void evalTo(Dest&) const {}

    int rows() const { return rows_; }
    int cols() const { return cols_; }
    // LinearOperator.cpp:14-22
    Vec operator*(const Vec& x) const {
        Vec y;
        mapping_(x, y);
        return y;
    }

    // the libifgf2d context behind the mapping, or nullptr for a plain mapping
    ifgf2d_ctx* device_context() const { return ctx_; }
    int apply_mode() const { return mode_; }

  protected:
    int rows_;
    int cols_;
    std::function<void(const Vec&, Vec&)> mapping_;
    ifgf2d_ctx* ctx_ = nullptr;
    int mode_ = -1;
};
