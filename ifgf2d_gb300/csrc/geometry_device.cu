// geometry_device.cu -- the discretisation of the ForwardMap constructor on the device.
//
// ForwardMap::init_points_and_patches and determine_patch_near_singular_points
// (ForwardMap/ForwardMap.tpp:37-285) on the GPU, for a context created with
// ifgf2d_options.device_geometry:
// * k_points: one thread per point -- Fejer node, the edge change of variables on open curves
//   (utils/Quadrature.hpp:151-173), position, unit normal (y', -x') / |x'| (Curve.hpp:97-102),
//   quadrature factor, edge jacobian and signed curvature;
// * k_patch_boxes: one block per patch -- the bounding box of Patch::comp_bounding_box
//   (Geometry/Patch.tpp:36-64) from the real roots of the degree-9 Chebyshev interpolants of
//   x'(t) and y'(t), located by sign changes on a 4000-interval grid and bisection, widened by
//   delta;
// * k_near_singular: one warp per patch -- every point of the candidate patches inside the box
//   is tested for distance below delta at the patch ends, else by Brent's minimiser
//   (utils/BrentsMethod.hpp:42-156) over the patch parameter.
// The patch limits (arc-length bisection) and the candidate lists stay on the host, as do the
// results' order: near-singular points are listed per patch in candidate order, then point
// order, as the host discretisation lists them.  The translation unit is compiled without FMA
// contraction; positions and parameters agree with the host's to a few ulps (the device's
// sin / cos / pow differ from glibc's in the last bits).
#include "geometry.hpp"
#include "curve_device.cuh"

#include <cuda_runtime.h>
#include <math_constants.h>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

namespace ifgf {
namespace {

struct GeoPatch { double t1, t2; int curve, s1, s2, pad; };

__device__ __forceinline__ double lin_map_d(double x, double a, double b, double c, double d) { return ((d - c) / (b - a)) * (x - a) + c; }
__device__ __forceinline__ double edge_both_d(double t, double p) { return -1.0 + (1.0 / kPi) * d_w(kPi * (t + 1.0), p); }
__device__ __forceinline__ double edge_m1_d(double t, double p) { return -1.0 + 2.0 * (1.0 / kPi) * d_w((kPi / 2.0) * (t + 1.0), p); }
__device__ __forceinline__ double edge_p1_d(double t, double p) { return -3.0 + 2.0 * (1.0 / kPi) * d_w(kPi + (kPi / 2.0) * (t + 1), p); }
__device__ __forceinline__ double dedge_both_d(double t, double p) { return d_wp(kPi * (t + 1.0), p); }
__device__ __forceinline__ double dedge_p1_d(double t, double p) { return d_wp(kPi + (kPi / 2.0) * (t + 1), p); }

// out: 8 arrays of N doubles -- x, y, nx, ny, t, wq, edge jacobian, curvature
__global__ void k_points(const GeoPatch* __restrict__ patches, const DevCurve* __restrict__ curves, const double* __restrict__ fej_n,
                         const double* __restrict__ fej_w, int Np, double p, long long N, double* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const long long pi = i / Np;
    const int j = (int)(i - pi * Np);
    const GeoPatch P = patches[pi];
    const DevCurve cv = curves[P.curve];
    const double z = fej_n[j];
    double tm = z, ej = 0.0;
    if (P.s1 && P.s2) { tm = edge_both_d(z, p); ej = dedge_both_d(z, p); }
    else if (P.s1) { tm = edge_m1_d(z, p); ej = dedge_both_d(z, p); }
    else if (P.s2) { tm = edge_p1_d(z, p); ej = dedge_p1_d(z, p); }
    const double t = lin_map_d(tm, -1.0, 1.0, P.t1, P.t2);
    double x, y, xp, yp;
    curve_eval(cv, t, x, y, xp, yp);
    const double nx = yp, ny = -xp;
    const double nn = sqrt(nx * nx + ny * ny);
    double cj = nn;
    if (P.s1 || P.s2) cj *= ej;
    double kappa = 0.0;
    if (cv.type != 2) {
        double xpp, ypp;
        curve_eval2(cv, t, xpp, ypp);
        const double sp = sqrt(xp * xp + yp * yp);
        kappa = (xp * ypp - yp * xpp) / (sp * sp * sp);
    }
    out[i] = x;
    out[N + i] = y;
    out[2 * N + i] = nx / nn;
    out[3 * N + i] = ny / nn;
    out[4 * N + i] = t;
    out[5 * N + i] = ((P.t2 - P.t1) / 2.0) * fej_w[j] * cj;
    out[6 * N + i] = ej;
    out[7 * N + i] = kappa;
}

// Clenshaw sum of a degree-9 Chebyshev series
__device__ __forceinline__ double cheb_ev(const double* c, double z) {
    double b1 = 0.0, b2 = 0.0;
    for (int k = 9; k >= 1; --k) { const double bb = 2.0 * z * b1 - b2 + c[k]; b2 = b1; b1 = bb; }
    return z * b1 - b2 + c[0];
}

constexpr int kBoxThreads = 128;
constexpr int kBoxGrid = 4000;

// per patch: x0, x1, y0, y1 of the bounding box (widened by delta)
__global__ void __launch_bounds__(kBoxThreads) k_patch_boxes(const GeoPatch* __restrict__ patches, const DevCurve* __restrict__ curves,
                                                             double delta, double* __restrict__ box) {
    __shared__ double coef[2][10];
    __shared__ double red[4][kBoxThreads];
    const int pi = blockIdx.x, tid = threadIdx.x;
    const GeoPatch P = patches[pi];
    const DevCurve cv = curves[P.curve];
    const double a = P.t1, b = P.t2;
    if (tid < 2) {   // interpolants of x'(t) (tid 0) and y'(t) (tid 1) at the 10 Chebyshev nodes
        double xs[10], fv[10], c[10], tm1[10], t0[10];
        for (int i = 0; i < 10; ++i) {
            xs[i] = cos(kPi * (2.0 * i + 1.0) / 20.0);
            double x, y, xp, yp;
            curve_eval(cv, lin_map_d(xs[i], -1, 1, a, b), x, y, xp, yp);
            fv[i] = tid == 0 ? xp : yp;
            c[i] = 0.0;
        }
        for (int k = 0; k < 10; ++k) { tm1[k] = 1.0; t0[k] = xs[k]; c[0] += fv[k]; c[1] += fv[k] * xs[k]; }
        c[0] *= 1.0 / 10; c[1] *= 2.0 / 10;
        for (int i = 2; i < 10; ++i) {
            for (int k = 0; k < 10; ++k) { const double v = 2.0 * xs[k] * t0[k] - tm1[k]; c[i] += fv[k] * v; tm1[k] = t0[k]; t0[k] = v; }
            c[i] *= 2.0 / 10;
        }
        for (int i = 0; i < 10; ++i) coef[tid][i] = c[i];
    }
    __syncthreads();
    double ex[2] = {1e308, 1e308}, ey[2] = {-1e308, -1e308};   // min / max of x (0) and y (1)
    if (tid == 0) {
        double x, y, xp, yp;
        curve_eval(cv, a, x, y, xp, yp);
        ex[0] = fmin(ex[0], x); ey[0] = fmax(ey[0], x); ex[1] = fmin(ex[1], y); ey[1] = fmax(ey[1], y);
        curve_eval(cv, b, x, y, xp, yp);
        ex[0] = fmin(ex[0], x); ey[0] = fmax(ey[0], x); ex[1] = fmin(ex[1], y); ey[1] = fmax(ey[1], y);
    }
    for (int f = 0; f < 2; ++f) {
        const double* c = coef[f];
        for (int s = tid + 1; s <= kBoxGrid; s += kBoxThreads) {
            const double zl = -1.0 + 2.0 * (s - 1) / kBoxGrid, zr = -1.0 + 2.0 * s / kBoxGrid;
            const double fl = cheb_ev(c, zl), fr = cheb_ev(c, zr);
            double z = 2.0;   // no root in this interval
            if (fl == 0.0 && zl > -1.0) z = zl;
            else if ((fl < 0.0 && fr > 0.0) || (fl > 0.0 && fr < 0.0)) {
                double lo = zl, hi = zr, flo = fl;
                for (int it = 0; it < 100 && hi - lo >= 1e-15; ++it) {
                    const double m = 0.5 * (lo + hi), fm = cheb_ev(c, m);
                    if ((fm < 0.0) == (flo < 0.0)) { lo = m; flo = fm; } else hi = m;
                }
                const double r = 0.5 * (lo + hi);
                if (r > -1.0 && r < 1.0) z = r;
            }
            if (z < 2.0) {
                double x, y, xp, yp;
                curve_eval(cv, lin_map_d(z, -1, 1, a, b), x, y, xp, yp);
                const double v = f == 0 ? x : y;
                ex[f] = fmin(ex[f], v);
                ey[f] = fmax(ey[f], v);
            }
        }
    }
    red[0][tid] = ex[0]; red[1][tid] = ey[0]; red[2][tid] = ex[1]; red[3][tid] = ey[1];
    __syncthreads();
    for (int w = kBoxThreads / 2; w > 0; w >>= 1) {
        if (tid < w) {
            red[0][tid] = fmin(red[0][tid], red[0][tid + w]);
            red[1][tid] = fmax(red[1][tid], red[1][tid + w]);
            red[2][tid] = fmin(red[2][tid], red[2][tid + w]);
            red[3][tid] = fmax(red[3][tid], red[3][tid + w]);
        }
        __syncthreads();
    }
    if (tid == 0) {
        box[4 * pi] = red[0][0] - delta;
        box[4 * pi + 1] = red[1][0] + delta;
        box[4 * pi + 2] = red[2][0] - delta;
        box[4 * pi + 3] = red[3][0] + delta;
    }
}

__device__ __forceinline__ double dist_to(const DevCurve& cv, double t, double px, double py) {
    double x, y, xp, yp;
    curve_eval(cv, t, x, y, xp, yp);
    const double dx = x - px, dy = y - py;
    return sqrt(fabs(dx * dx + dy * dy));
}

// Brent's localmin with golden-section fallback (BrentsMethod.hpp:42-156), the host's step sequence
__device__ void brent_min_d(const DevCurve& cv, double px, double py, double lo, double hi, double& xmin, double& fmin) {
    const double tol = 1e-6, g = (double)0.3819660f;
    double x = hi, w = hi, v = hi, u, fx = dist_to(cv, x, px, py), fw = fx, fv = fx, fu, d = 0.0, e = 0.0;
    for (int it = 100; it > 0; --it) {
        const double mid = 0.5 * (lo + hi), t1 = tol * fabs(x) + tol / 4, t2 = 2 * t1;
        if (fabs(x - mid) <= t2 - (hi - lo) / 2) break;
        bool golden = true;
        if (fabs(e) > t1) {
            double r = (x - w) * (fx - fv), q = (x - v) * (fx - fw), pp = (x - v) * q - (x - w) * r;
            q = 2 * (q - r);
            if (q > 0) pp = -pp;
            q = fabs(q);
            const double eold = e;
            e = d;
            if (!(fabs(pp) >= fabs(q * eold / 2) || pp <= q * (lo - x) || pp >= q * (hi - x))) {
                golden = false;
                d = pp / q; u = x + d;
                if ((u - lo) < t2 || (hi - u) < t2) d = (mid - x) < 0 ? -fabs(t1) : fabs(t1);
            }
        }
        if (golden) { e = (x >= mid) ? lo - x : hi - x; d = g * e; }
        u = fabs(d) >= t1 ? x + d : (d > 0 ? x + fabs(t1) : x - fabs(t1));
        fu = dist_to(cv, u, px, py);
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

// one warp per patch: tout[cand_ptr[pi] * Np + q] = the near-singular parameter of the q-th
// candidate point, or NaN when it is not near-singular
__global__ void k_near_singular(const GeoPatch* __restrict__ patches, const DevCurve* __restrict__ curves,
                                const double* __restrict__ box, const int* __restrict__ cand_ptr, const long long* __restrict__ cand,
                                const double* __restrict__ px, const double* __restrict__ py, int Np, long long npatch, double delta,
                                double* __restrict__ tout) {
    const long long pi = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pi >= npatch) return;
    const GeoPatch P = patches[pi];
    const DevCurve cv = curves[P.curve];
    // corners A = (x1, y0), B = (x1, y1), C = (x0, y1), as Patch.tpp:62-63 orders them
    const double x0 = box[4 * pi], x1 = box[4 * pi + 1], y0 = box[4 * pi + 2], y1 = box[4 * pi + 3];
    const double ax = x1, ay = y0, bx = x1, by = y1, cx = x0, cy = y1;
    const double bax = bx - ax, bay = by - ay, cbx = cx - bx, cby = cy - by;
    const double ba2 = bax * bax + bay * bay, cb2 = cbx * cbx + cby * cby;
    const int c0 = cand_ptr[pi], nq = (cand_ptr[pi + 1] - c0) * Np;
    for (int q = lane; q < nq; q += 32) {
        const long long slot = (long long)c0 * Np + q;
        tout[slot] = CUDART_NAN;
        const long long tp = cand[c0 + q / Np];
        if (tp < 0 || tp >= npatch) continue;
        const long long kk = tp * Np + q % Np;
        const double xq = px[kk], yq = py[kk];
        const double d1 = bax * (xq - ax) + bay * (yq - ay);
        const double d2 = cbx * (xq - bx) + cby * (yq - by);
        if (!(0 <= d1 && d1 <= ba2 && 0 <= d2 && d2 <= cb2)) continue;
        double ts, dmin;
        if (dist_to(cv, P.t1, xq, yq) < delta) ts = P.t1;
        else if (dist_to(cv, P.t2, xq, yq) < delta) ts = P.t2;
        else {
            brent_min_d(cv, xq, yq, P.t1, P.t2, ts, dmin);
            if (!(dmin < delta)) continue;
        }
        tout[slot] = ts;
    }
}

struct DevMem {
    std::vector<void*> ptrs;
    ~DevMem() { for (void* p : ptrs) cudaFree(p); }
    template <class T>
    T* get(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
};

}  // namespace

std::string discretise_on_device(Discretisation& D, const std::vector<std::vector<long long>>& cand) {
    const long long N = D.N, np = D.num_patches;
    const int Np = D.Np;
    DevMem mem;
    auto fail = [](const char* what, cudaError_t e) { return std::string("device geometry: ") + what + ": " + cudaGetErrorString(e); };
    std::vector<DevCurve> dc(D.curves.size());
    for (size_t c = 0; c < D.curves.size(); ++c) { dc[c].type = D.curves[c].type; dc[c].pad = 0; for (int i = 0; i < 16; ++i) dc[c].p[i] = D.curves[c].p[i]; }
    std::vector<GeoPatch> gp(np);
    for (long long p = 0; p < np; ++p) gp[p] = GeoPatch{D.t1[p], D.t2[p], D.curve_of[p], D.ist1sing[p], D.ist2sing[p], 0};
    std::vector<int> cptr(np + 1, 0);
    std::vector<long long> cflat;
    for (long long p = 0; p < np; ++p) { for (long long c : cand[p]) cflat.push_back(c); cptr[p + 1] = (int)cflat.size(); }
    DevCurve* d_curves = mem.get<DevCurve>(dc.size());
    GeoPatch* d_patches = mem.get<GeoPatch>(np);
    double* d_fn = mem.get<double>(Np);
    double* d_fw = mem.get<double>(Np);
    double* d_out = mem.get<double>((size_t)8 * N);
    double* d_box = mem.get<double>((size_t)4 * np);
    int* d_cptr = mem.get<int>(np + 1);
    long long* d_cand = mem.get<long long>(cflat.size());
    double* d_t = mem.get<double>((size_t)cflat.size() * Np);
    if (!d_curves || !d_patches || !d_fn || !d_fw || !d_out || !d_box || !d_cptr || !d_cand || !d_t)
        return "device geometry: cudaMalloc failed";
    cudaError_t e;
    if ((e = cudaMemcpy(d_curves, dc.data(), sizeof(DevCurve) * dc.size(), cudaMemcpyHostToDevice)) != cudaSuccess) return fail("upload", e);
    if ((e = cudaMemcpy(d_patches, gp.data(), sizeof(GeoPatch) * np, cudaMemcpyHostToDevice)) != cudaSuccess) return fail("upload", e);
    if ((e = cudaMemcpy(d_fn, D.fej_n.data(), sizeof(double) * Np, cudaMemcpyHostToDevice)) != cudaSuccess) return fail("upload", e);
    if ((e = cudaMemcpy(d_fw, D.fej_w.data(), sizeof(double) * Np, cudaMemcpyHostToDevice)) != cudaSuccess) return fail("upload", e);
    if ((e = cudaMemcpy(d_cptr, cptr.data(), sizeof(int) * (np + 1), cudaMemcpyHostToDevice)) != cudaSuccess) return fail("upload", e);
    if (!cflat.empty() && (e = cudaMemcpy(d_cand, cflat.data(), sizeof(long long) * cflat.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail("upload", e);
    k_points<<<(unsigned)((N + 255) / 256), 256>>>(d_patches, d_curves, d_fn, d_fw, Np, D.p, N, d_out);
    k_patch_boxes<<<(unsigned)np, kBoxThreads>>>(d_patches, d_curves, D.delta, d_box);
    k_near_singular<<<(unsigned)((np * 32 + 127) / 128), 128>>>(d_patches, d_curves, d_box, d_cptr, d_cand, d_out, d_out + N, Np, np,
                                                               D.delta, d_t);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail("launch", e);
    std::vector<double> out((size_t)8 * N), tv((size_t)cflat.size() * Np);
    if ((e = cudaMemcpy(out.data(), d_out, sizeof(double) * 8 * N, cudaMemcpyDeviceToHost)) != cudaSuccess) return fail("kernels", e);
    if (!tv.empty() && (e = cudaMemcpy(tv.data(), d_t, sizeof(double) * tv.size(), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return fail("kernels", e);
    D.x.assign(out.begin(), out.begin() + N);
    D.y.assign(out.begin() + N, out.begin() + 2 * N);
    D.nx.assign(out.begin() + 2 * N, out.begin() + 3 * N);
    D.ny.assign(out.begin() + 3 * N, out.begin() + 4 * N);
    D.t.assign(out.begin() + 4 * N, out.begin() + 5 * N);
    D.wq.assign(out.begin() + 5 * N, out.begin() + 6 * N);
    D.edge_jac.assign(out.begin() + 6 * N, out.begin() + 7 * N);
    D.kappa.assign(out.begin() + 7 * N, out.begin() + 8 * N);
    D.patch_of.resize(N);
    for (long long i = 0; i < N; ++i) D.patch_of[i] = (int)(i / Np);
    D.ns_ptr.assign(np + 1, 0);
    D.ns_idx.clear();
    D.ns_t.clear();
    for (long long p = 0; p < np; ++p) {
        for (int ci = cptr[p]; ci < cptr[p + 1]; ++ci)
            for (int j = 0; j < Np; ++j) {
                const double t = tv[(size_t)ci * Np + j];
                if (std::isnan(t)) continue;
                D.ns_idx.push_back(cflat[ci] * Np + j);
                D.ns_t.push_back(t);
            }
        D.ns_ptr[p + 1] = (int)D.ns_idx.size();
    }
    return "";
}

}  // namespace ifgf
