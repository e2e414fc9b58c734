// geometry.hpp -- host-side discretisation of the boundary (the ForwardMap constructor).
//
// Produces the flat arrays the device path consumes: points, unit normals, quadrature
// factors, patch limits and the near-singular lists.  Follows:
//   Geometry/Curve.hpp:97-161, Curve.cpp:5-155       curves, normals, patch limits
//   Geometry/Patch.tpp:21-64                          bounding boxes
//   ForwardMap/ForwardMap.tpp:37-285                  points/patches, near-singular detection
//   utils/Quadrature.hpp:12-173                       Fejer rule, changes of variables
//   utils/BrentsMethod.hpp:42-156                     Brent's minimiser
#pragma once

#include <cmath>
#include <vector>
#include <array>
#include <string>
#include <functional>
#include "../../include/ifgf2d.h"

namespace ifgf {

constexpr double kPiH = 3.14159265358979323846;

// Parametrised curve evaluated on the host (device twin: DevCurve in ifgf2d_kernels.cuh)
struct HostCurve {
    int type = IFGF2D_CURVE_CIRCLE;
    bool closed = true;
    double tlim1 = 0.0, tlim2 = 2.0 * kPiH;
    double p[16] = {0};

    double x(double t) const;
    double y(double t) const;
    double xp(double t) const;
    double yp(double t) const;
    // signed curvature (x' y'' - y' x'') / |x'|^3 (for the learned preconditioner's features)
    double curvature(double t) const;
};

// Everything the constructor of ForwardMap computes (ForwardMap.tpp:15-285)
struct Discretisation {
    int Np = 0;
    double delta = 0.0, p = 4.0;
    long long N = 0, num_patches = 0;
    std::vector<HostCurve> curves;
    // per point (patch-major order, as in ForwardMap::xs_)
    std::vector<double> x, y, nx, ny, t, wq, edge_jac, kappa;
    std::vector<int> patch_of;
    // per patch
    std::vector<double> t1, t2;
    std::vector<int> curve_of, ist1sing, ist2sing;
    std::vector<int> ns_ptr;          // CSR over patches: near-singular point indices / t values
    std::vector<long long> ns_idx;
    std::vector<double> ns_t;
    // quadrature rules
    std::vector<double> fej_n, fej_w, fej_ns_n, fej_ns_w;
};

// Returns an empty string on success, else an error message.
std::string discretise(const ifgf2d_curve* curves, int ncurves, const ifgf2d_junction* junctions,
                       int njunctions, const ifgf2d_options& opt, Discretisation& out);

void fejer_rule(int n, std::vector<double>& nodes, std::vector<double>& weights);

// The per-point discretisation, the patch bounding boxes and the near-singular detection of
// `D` (whose patches are set) on the current GPU (geometry_device.cu); cand holds each patch's
// candidate patches.  Returns an empty string on success, else an error message.
std::string discretise_on_device(Discretisation& D, const std::vector<std::vector<long long>>& cand);

}  // namespace ifgf
