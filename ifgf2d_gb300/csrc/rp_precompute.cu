// rp_precompute.cu -- rectangular-polar singular / near-singular weights on the GPU.
//
// ForwardMap::single_patch_point_compute_precomputations (ForwardMap/ForwardMap.tpp:287-389)
// and the fold of the per-patch Chebyshev transform (utils/Chebyshev1d.hpp:363-392) into the
// weights.  Singular points sit within 1e-16 (in parameter) of open-curve ends, where the
// changes of variables are evaluated next to cancellation; this translation unit is compiled
// with -fmad=false so that its arithmetic rounds like the host restatement (no contraction).
#include "ifgf2d_kernels.cuh"
#include "hankel.cuh"
#include "curve_device.cuh"

namespace ifgf {

__device__ __forceinline__ double warp_sum_rp(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------------ set-up: RP weights
// One warp per column: 40 Fejer nodes after the singularity-resolving change of variables,
// the Green function at each node, then the Np Chebyshev moments (ForwardMap.tpp:287-389).
__global__ void k_rp_precompute(const RPColumn* __restrict__ cols, int ncols, const DevPatch* __restrict__ patches,
                                const DevCurve* __restrict__ curves, const double* __restrict__ nsn,
                                const double* __restrict__ nsw, int Np, double p, double k0, int form, double eta0,
                                const double2* __restrict__ keta, double2* __restrict__ M) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= ncols) return;
    const double k = keta ? keta[w].x : k0, eta = keta ? keta[w].y : eta0;   // per column for a group of obstacles
    const RPColumn c = cols[w];
    const DevPatch P = patches[c.patch];
    const DevCurve cv = curves[P.curve];
    const double alpha = (2.0 / (P.t2 - P.t1)) * (c.tsing - P.t1) + (-1.0);
    const int loc = fabs(-1.0 - alpha) < 1e-5 ? -1 : (fabs(1.0 - alpha) < 1e-5 ? 1 : 0);
    double xi[2] = {0.0, 0.0};
    double2 ig[2] = {make_double2(0, 0), make_double2(0, 0)};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int i = lane + 32 * q;
        if (i >= 40) continue;
        const double z = nsn[i];
        double x, dx;
        if (loc == 0) {
            x = alpha + ((d_sgn(z) - alpha) / kPi) * d_w(kPi * fabs(z), p);
            dx = (1.0 - alpha * d_sgn(z)) * d_wp(kPi * fabs(z), p);
        } else if (loc == -1) {
            const double h = (z + 1.0) / 2.0;
            x = -1.0 + (2.0 / kPi) * d_w(kPi * fabs(h), p);
            dx = d_wp(kPi * fabs(h), p) * d_sgn(h);
        } else {
            const double h = (z - 1.0) / 2.0;
            x = 1.0 - (2.0 / kPi) * d_w(kPi * fabs(h), p);
            dx = -d_wp(kPi * fabs(h), p) * d_sgn(h);
        }
        double u = x;
        if (P.ist1 && P.ist2) u = -1.0 + (1.0 / kPi) * d_w(kPi * (x + 1.0), p);
        else if (P.ist1) u = -1.0 + 2.0 * (1.0 / kPi) * d_w((kPi / 2.0) * (x + 1.0), p);
        else if (P.ist2) u = -3.0 + 2.0 * (1.0 / kPi) * d_w(kPi + (kPi / 2.0) * (x + 1), p);
        const double g = ((P.t2 - P.t1) / 2.0) * (u - (-1.0)) + P.t1;
        double px, py, pxp, pyp;
        curve_eval(cv, g, px, py, pxp, pyp);
        const double cj = sqrt(pyp * pyp + pxp * pxp);
        // target: the (near-)singular point; source: x(g) with its unit normal (y', -x') / |x'|
        const double2 G = green_form(form, c.xs - px, c.ys - py, pyp / cj, -pxp / cj, k, eta);
        const double f = ((P.t2 - P.t1) / 2.0);
        double2 v = make_double2(f * G.x, f * G.y);
        v.x *= cj; v.y *= cj; v.x *= dx; v.y *= dx; v.x *= nsw[i]; v.y *= nsw[i];
        xi[q] = x; ig[q] = v;
    }
    double tm1[2] = {1.0, 1.0}, t0[2] = {xi[0], xi[1]};
    for (int n = 0; n < Np; ++n) {
        double tn[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (n == 0) tn[q] = 1.0;
            else if (n == 1) tn[q] = xi[q];
            else { tn[q] = 2.0 * xi[q] * t0[q] - tm1[q]; tm1[q] = t0[q]; t0[q] = tn[q]; }
        }
        double re = ig[0].x * tn[0] + ig[1].x * tn[1];
        double im = ig[0].y * tn[0] + ig[1].y * tn[1];
        re = warp_sum_rp(re); im = warp_sum_rp(im);
        if (lane == 0) M[(long long)w * Np + n] = make_double2(re, im);
    }
}

// W[col][k] = e_k sum_r C[r][k] M[col][r]: the Chebyshev transform of the density segment
// (Chebyshev1d.hpp:363-392) folded into the weights, with the edge jacobian on open ends.
__global__ void k_rp_fold(const double2* __restrict__ M, const RPColumn* __restrict__ cols, int ncols,
                          const double* __restrict__ edge, const DevPatch* __restrict__ patches, int Np,
                          double2* __restrict__ W) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)ncols * Np) return;
    const int col = (int)(id / Np), kk = (int)(id % Np);
    const double xk = cos(kPi * (2.0 * kk + 1.0) / (2.0 * Np));
    double tm1 = 1.0, t0 = xk;
    const double2* m = M + (long long)col * Np;
    double2 acc = make_double2(m[0].x * (1.0 / Np), m[0].y * (1.0 / Np));
    for (int r = 1; r < Np; ++r) {
        double tr;
        if (r == 1) tr = xk; else { tr = 2.0 * xk * t0 - tm1; tm1 = t0; t0 = tr; }
        const double c = tr * (2.0 / Np);
        acc.x = fma(c, m[r].x, acc.x); acc.y = fma(c, m[r].y, acc.y);
    }
    const int pt = cols[col].patch;
    const DevPatch P = patches[pt];
    if (P.ist1 || P.ist2) { const double e = edge[(long long)pt * Np + kk]; acc.x *= e; acc.y *= e; }
    W[id] = acc;
}

static inline unsigned nblk_rp(long long n, int b) { return (unsigned)((n + b - 1) / b); }

void launch_rp_precompute(const RPColumn* cols, int ncols, const DevPatch* patches, const DevCurve* curves,
                          const double* nsn, const double* nsw, int Np, double p, double k, int form, double eta, double2* M,
                          cudaStream_t s, const double2* keta) {
    if (ncols <= 0) return;
    k_rp_precompute<<<nblk_rp((long long)ncols * 32, 128), 128, 0, s>>>(cols, ncols, patches, curves, nsn, nsw, Np, p, k, form, eta,
                                                                        keta, M);
}
void launch_rp_fold(const double2* M, const RPColumn* cols, int ncols, const double* edge, const DevPatch* patches,
                    int Np, double2* W, cudaStream_t s) {
    if (ncols <= 0) return;
    k_rp_fold<<<nblk_rp((long long)ncols * Np, 256), 256, 0, s>>>(M, cols, ncols, edge, patches, Np, W);
}
}  // namespace ifgf
