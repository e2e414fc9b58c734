// spectral_precond.cu -- the spectral right preconditioner of the combined-field operator.
//
// The reference's GMRES is unpreconditioned (ForwardMap/ForwardMap.tpp:658-697,
// ForwardMap/opGMRES.hpp:68-269).  This file adds a right preconditioner for the sound-soft
// combined field A = 1/2 I + K - i eta S on closed curves.  Along a curve, A acts on a wave
// e^{i xi s} (s arc length) approximately as the flat boundary's symbol
//
//     sigma(xi) = 1/2 + eta / (2 sqrt(k_eps^2 - xi^2)),   k_eps = k + i eps,  Im sqrt >= 0,
//
// (the single layer's flat symbol is i / (2 sqrt(k^2 - xi^2)) and the flat double layer
// vanishes); the complex wavenumber smooths the square-root singularity at glancing
// incidence xi = k (the on-surface radiation condition device of Antoine and Darbas, M2AN
// 2005), eps = scale k^(1/3).  The preconditioner applies the inverse symbol:
//
//     z = M r = 2 r + B F^{-1} [ (1/sigma - 2) F (W r) ].
//
// 1/sigma -> 2 at high frequency, so the part that goes through the resampling decays like
// k / xi and the identity part 2 r stays exact at the nodes.
//   W  resamples each closed curve's node values onto a uniform arc-length grid of
//      nu = 2^m >= n points: per grid point the Lagrange interpolant (barycentric form) of the
//      Np nodes of its patch, at the local coordinate that the same interpolation through the
//      nodes' arc lengths (spectral integrals of |x'| from the quadrature factors) gives;
//   F  is the length-nu discrete Fourier transform, computed in four steps (nu = N1 N2):
//      FFTs of length N1 down the columns of the N1 x N2 view, a twiddle factor, FFTs of
//      length N2 along the rows.  The spectrum stays in that transposed order; the multiplier
//      table is stored in it, so the inverse runs the same steps backwards with no transpose;
//   B  interpolates back to each node from the 8 uniform grid points around it.
// Everything runs in FP32 (a preconditioner only has to be a fixed linear map); the solver's
// vectors stay FP64.  Per application: four launches, O(nu log nu) work, a few hundred KB of
// traffic at nu = 32768.
#include "context.hpp"
#include "host_threads.hpp"

#include <algorithm>
#include <complex>
#include <memory>

namespace ifgf {

constexpr int kSpecTile = 2;      // grid columns per block of the column FFTs (more blocks: these kernels are latency-bound)
constexpr int kSpecTaps = 8;      // back-interpolation taps
constexpr int kSpecThreads = 256;
constexpr int kSpecMinLog = 6;    // smallest grid: 64 points
constexpr int kSpecMaxLog = 20;   // largest grid: 2^20 points per curve

struct SpecCurve {
    long long off = 0;            // the curve's points: [off, off + n) of the context (patch-major)
    int n = 0;
    int lg = 0, lg1 = 0, lg2 = 0; // nu = 2^lg = N1 N2, N1 = 2^lg1, N2 = 2^lg2
    double length = 0.0;
    DBuf<int> fw_base;            // per grid point: first point of its patch
    DBuf<float> fw_w;             // per grid point: Np Lagrange weights
    DBuf<int> bk_base;            // per node: first of its kSpecTaps grid points (mod nu)
    DBuf<float> bk_w;             // per node: kSpecTaps weights
    // per frequency, in the transposed order k1 N2 + k2, three multipliers m, nu values each, each
    // with the base b it is paired with (z = b v + B F^-1 [m F W v]):
    //   0: 1/sigma - 2 (b = 2), the preconditioner;  1: |sigma| - 1/2 (b = 1/2), the operator's
    //   magnitude;  2: 1/|sigma| - 2 (b = 2), its inverse
    DBuf<float2> mult;
    DBuf<float2> twN;             // e^{-2 pi i k1 n2 / nu} at k1 N2 + n2
    DBuf<float2> tw1, tw2;        // e^{-2 pi i j / N1}, j < N1 / 2; the same for N2
};

// a curve's tables as the kernels see them
struct SpecDesc {
    long long off, uoff;          // first point of the curve; first grid value in the work buffer
    int n, lg, lg1, lg2;
    const int* fw_base;
    const float* fw_w;
    const int* bk_base;
    const float* bk_w;
    const float2 *mult, *twN, *tw1, *tw2;
};

}  // namespace ifgf

struct SpectralWork {
    std::vector<std::unique_ptr<ifgf::SpecCurve>> curves;
    DBuf<ifgf::SpecDesc> desc;    // per curve: its tables
    DBuf<int> pre;                // per kernel (columns, rows, nodes): the curves' block-count prefix, ncurves + 1 each
    int ncurves = 0, blocks_cols = 0, blocks_rows = 0, blocks_back = 0;
    size_t smem_cols = 0, smem_rows = 0;
    DBuf<float2> u;               // the grid values of every curve, one right-hand side
    long long grid_total = 0;     // grid points of all curves
    double scale = 0.0;
};

namespace ifgf {
namespace {

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ int brev(int i, int lg) { return lg ? (int)(__brev((unsigned)i) >> (32 - lg)) : 0; }

// radix-2 decimation-in-time FFT, in place, of `cols` interleaved columns of length 2^lg held
// in bit-reversed order: element i of column c at s[i * cols + c].  tw[j] = e^{-2 pi i j / L};
// inv: conjugate twiddles (unnormalised inverse).  Ends with a barrier.
__device__ void fft_shared(float2* s, int lg, int cols, const float2* __restrict__ tw, bool inv) {
    const int half = 1 << (lg - 1);
    for (int st = 0; st < lg; ++st) {
        const int hs = 1 << st;
        for (int b = threadIdx.x; b < half * cols; b += blockDim.x) {
            const int c = b % cols, q = b / cols;
            const int j = q & (hs - 1);
            const int i0 = ((q >> st) << (st + 1)) + j, i1 = i0 + hs;
            float2 w = tw[j << (lg - 1 - st)];
            if (inv) w.y = -w.y;
            const float2 a = s[i0 * cols + c], t = cmulf(w, s[i1 * cols + c]);
            s[i0 * cols + c] = make_float2(a.x + t.x, a.y + t.y);
            s[i1 * cols + c] = make_float2(a.x - t.x, a.y - t.y);
        }
        __syncthreads();
    }
}

// Every kernel serves all curves of the context in one launch: block b of a launch belongs to
// the curve c with pre[c] <= b < pre[c + 1] (pre: the curves' block-count prefix for that kernel),
// and works on that curve's tables (SpecDesc).  Vectors hold right-hand side q = blockIdx.y of
// point i at i * ld + q (ld 1 for one vector, the batch size for interleaved batches); its grid
// values at u + q * ustride + desc.uoff.
__device__ __forceinline__ int spec_curve_of(const int* __restrict__ pre, int ncurves, int b) {
    int lo = 0, hi = ncurves - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// W r and the column FFTs: grid point g = n1 N2 + n2 takes its patch's Np node values; each
// block transforms kSpecTile columns n2 over n1, multiplies by the twiddle and writes
// Y[k1 N2 + n2].
__global__ void __launch_bounds__(kSpecThreads) k_spec_fwd_cols(const double2* __restrict__ r, int ld, const SpecDesc* __restrict__ cd,
                                                                const int* __restrict__ pre, int ncurves, int Np,
                                                                float2* __restrict__ u, long long ustride) {
    extern __shared__ float2 sm[];
    const int c = spec_curve_of(pre, ncurves, blockIdx.x);
    const SpecDesc d = cd[c];
    const int N1 = 1 << d.lg1, N2 = 1 << d.lg2;
    const int cols = min(kSpecTile, N2), c0 = (blockIdx.x - pre[c]) * cols;
    r += blockIdx.y;
    float2* Y = u + blockIdx.y * ustride + d.uoff;
    for (int e = threadIdx.x; e < N1 * cols; e += blockDim.x) {
        const int n1 = e / cols, cc = e - n1 * cols;
        const int g = n1 * N2 + c0 + cc;
        const double2* src = r + (long long)d.fw_base[g] * ld;
        const float* w = d.fw_w + (size_t)g * Np;
        float re = 0.f, im = 0.f;
        for (int j = 0; j < Np; ++j) {
            const double2 v = src[(long long)j * ld];
            re = fmaf(w[j], (float)v.x, re);
            im = fmaf(w[j], (float)v.y, im);
        }
        sm[brev(n1, d.lg1) * cols + cc] = make_float2(re, im);
    }
    __syncthreads();
    fft_shared(sm, d.lg1, cols, d.tw1, false);
    for (int e = threadIdx.x; e < N1 * cols; e += blockDim.x) {
        const int k1 = e / cols, cc = e - k1 * cols;
        const int o = k1 * N2 + c0 + cc;
        Y[o] = cmulf(sm[k1 * cols + cc], d.twN[o]);
    }
}

// per row k1: the row FFT, the multiplier, the inverse row FFT and the inverse twiddle, in place
__global__ void __launch_bounds__(kSpecThreads) k_spec_rows(const SpecDesc* __restrict__ cd, const int* __restrict__ pre, int ncurves,
                                                            float2* __restrict__ u, long long ustride, int which) {
    extern __shared__ float2 sm[];
    const int c = spec_curve_of(pre, ncurves, blockIdx.x);
    const SpecDesc d = cd[c];
    const int N2 = 1 << d.lg2, k1 = blockIdx.x - pre[c];
    float2* row = u + blockIdx.y * ustride + d.uoff + (size_t)k1 * N2;
    const float2* mrow = d.mult + ((size_t)which << d.lg) + (size_t)k1 * N2;
    const float2* trow = d.twN + (size_t)k1 * N2;
    for (int i = threadIdx.x; i < N2; i += blockDim.x) sm[brev(i, d.lg2)] = row[i];
    __syncthreads();
    fft_shared(sm, d.lg2, 1, d.tw2, false);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) sm[i] = cmulf(sm[i], mrow[i]);
    __syncthreads();
    for (int i = threadIdx.x; i < N2; i += blockDim.x) {   // back to bit-reversed order: disjoint swaps
        const int j = brev(i, d.lg2);
        if (i < j) { const float2 t = sm[i]; sm[i] = sm[j]; sm[j] = t; }
    }
    __syncthreads();
    fft_shared(sm, d.lg2, 1, d.tw2, true);
    for (int i = threadIdx.x; i < N2; i += blockDim.x) {
        const float2 t = trow[i];
        row[i] = cmulf(sm[i], make_float2(t.x, -t.y));
    }
}

// the inverse column FFTs, scaled by 1/nu, in place: u[n1 N2 + n2] on the uniform grid (a block
// reads all of its columns before it writes them)
__global__ void __launch_bounds__(kSpecThreads) k_spec_inv_cols(const SpecDesc* __restrict__ cd, const int* __restrict__ pre, int ncurves,
                                                                float2* __restrict__ u, long long ustride) {
    extern __shared__ float2 sm[];
    const int c = spec_curve_of(pre, ncurves, blockIdx.x);
    const SpecDesc d = cd[c];
    const int N1 = 1 << d.lg1, N2 = 1 << d.lg2;
    const int cols = min(kSpecTile, N2), c0 = (blockIdx.x - pre[c]) * cols;
    float2* U = u + blockIdx.y * ustride + d.uoff;
    const float scale = 1.0f / (float)(N1 * N2);
    for (int e = threadIdx.x; e < N1 * cols; e += blockDim.x) {
        const int k1 = e / cols, cc = e - k1 * cols;
        sm[brev(k1, d.lg1) * cols + cc] = U[k1 * N2 + c0 + cc];
    }
    __syncthreads();
    fft_shared(sm, d.lg1, cols, d.tw1, true);
    for (int e = threadIdx.x; e < N1 * cols; e += blockDim.x) {
        const int n1 = e / cols, cc = e - n1 * cols;
        const float2 v = sm[n1 * cols + cc];
        U[n1 * N2 + c0 + cc] = make_float2(v.x * scale, v.y * scale);
    }
}

// z = base r + B u on every curve's nodes
__global__ void k_spec_back(const double2* __restrict__ r, int ld, const SpecDesc* __restrict__ cd, const int* __restrict__ pre,
                            int ncurves, const float2* __restrict__ u, long long ustride, double base, double2* __restrict__ z) {
    const int c = spec_curve_of(pre, ncurves, blockIdx.x);
    const SpecDesc d = cd[c];
    const int j = (blockIdx.x - pre[c]) * blockDim.x + threadIdx.x;
    if (j >= d.n) return;
    const float2* uc = u + blockIdx.y * ustride + d.uoff;
    const int mask = (1 << d.lg) - 1;
    const int b = d.bk_base[j];
    float re = 0.f, im = 0.f;
#pragma unroll
    for (int t = 0; t < kSpecTaps; ++t) {
        const float w = d.bk_w[(size_t)j * kSpecTaps + t];
        const float2 v = uc[(b + t) & mask];
        re = fmaf(w, v.x, re);
        im = fmaf(w, v.y, im);
    }
    const long long o = (d.off + j) * ld + blockIdx.y;
    const double2 x = r[o];
    z[o] = make_double2(base * x.x + (double)re, base * x.y + (double)im);
}

// z = a x + b y
__global__ void k_axpby(double2* z, double a, const double2* x, double b, const double2* y, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 p = x[i], q = y[i];
    z[i] = make_double2(a * p.x + b * q.x, a * p.y + b * q.y);
}

// z += zn - 2 r: the network's correction on top of the spectral preconditioner
__global__ void k_precond_sum(double2* __restrict__ z, const double2* __restrict__ zn, const double2* __restrict__ r, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 a = z[i], b = zn[i], c = r[i];
    z[i] = make_double2(a.x + b.x - 2.0 * c.x, a.y + b.y - 2.0 * c.y);
}

// ---------------------------------------------------------------- host tables

// Q[j][m] = integral from -1 to z_j of the m-th Lagrange basis polynomial of the n first-kind
// Chebyshev (Fejer) nodes z: node m's weight in the arc length from the patch's start to node j
std::vector<double> cumulative_weights(const std::vector<double>& z) {
    const int n = (int)z.size();
    std::vector<double> Q((size_t)n * n, 0.0);
    auto T = [](int k, double x) { return std::cos(k * std::acos(std::min(1.0, std::max(-1.0, x)))); };
    auto I = [&](int k, double x) {   // integral of T_k from -1 to x
        if (k == 0) return x + 1.0;
        if (k == 1) return 0.5 * (x * x - 1.0);
        const double lo = 0.5 * ((k % 2 ? 1.0 : -1.0) / (k + 1) - (k % 2 ? 1.0 : -1.0) / (k - 1));
        return 0.5 * (T(k + 1, x) / (k + 1) - T(k - 1, x) / (k - 1)) - lo;
    };
    for (int j = 0; j < n; ++j)
        for (int m = 0; m < n; ++m) {
            double q = 0.0;
            for (int k = 0; k < n; ++k) q += (k == 0 ? 1.0 : 2.0) / n * T(k, z[m]) * I(k, z[j]);
            Q[(size_t)j * n + m] = q;
        }
    return Q;
}

int build_curve(const Discretisation& D, int c, double k, double eta, double eps, SpecCurve& out, std::string& err) {
    const HostCurve& C = D.curves[c];
    if (!C.closed) { err = "the spectral preconditioner needs closed curves"; return IFGF2D_ERR_ARG; }
    const int Np = D.Np;
    std::vector<int> pats;
    for (long long p = 0; p < D.num_patches; ++p) if (D.curve_of[p] == c) pats.push_back((int)p);
    if (pats.empty()) { err = "a curve without patches"; return IFGF2D_ERR_ARG; }
    std::sort(pats.begin(), pats.end(), [&](int a, int b) { return D.t1[a] < D.t1[b]; });
    for (size_t i = 1; i < pats.size(); ++i)
        if (pats[i] != pats[0] + (int)i) { err = "the spectral preconditioner needs each curve's patches stored in parameter order"; return IFGF2D_ERR_ARG; }
    const int P = (int)pats.size();
    const long long n = (long long)P * Np;
    int lg = kSpecMinLog;
    while ((1LL << lg) < n) ++lg;
    if (lg > kSpecMaxLog) { err = "the spectral preconditioner takes at most 2^20 points per curve"; return IFGF2D_ERR_ARG; }
    out.off = (long long)pats[0] * Np;
    out.n = (int)n;
    out.lg = lg; out.lg1 = lg / 2; out.lg2 = lg - lg / 2;   // N2 >= N1: N2 / kSpecTile column blocks
    const long long nu = 1LL << lg;
    const int N1 = 1 << out.lg1, N2 = 1 << out.lg2;
    // arc lengths from the nodes' quadrature factors: a closed curve's node j of a patch on
    // [a, b] has wq_j = (b - a) / 2 w_j |x'(t_j)| (Fejer weight w_j), so the patch length is
    // sum_j wq_j and the length up to node j is sum_m Q[j][m] wq_m / w_m (spectral integration
    // of the interpolant of |x'|)
    const std::vector<double> Q = cumulative_weights(D.fej_n);
    std::vector<double> S(P + 1, 0.0);
    for (int i = 0; i < P; ++i) {
        double l = 0.0;
        for (int j = 0; j < Np; ++j) l += D.wq[out.off + (long long)i * Np + j];
        S[i + 1] = S[i] + l;
    }
    const double L = S[P];
    out.length = L;
    const double h = L / (double)nu;
    // per patch: its nodes' local coordinates and arc lengths, and the barycentric weights of
    // both node sets (the grid point's local coordinate is interpolated from its arc length
    // through the nodes, then its value from the nodes' values)
    std::vector<double> loc((size_t)n), lam((size_t)n), sn((size_t)n), lams((size_t)n);
    parallel_for(P, [&](long long i0, long long i1) {
        for (long long i = i0; i < i1; ++i) {
            const int p = pats[i];
            const double a = D.t1[p], b = D.t2[p];
            double* ln = &loc[(size_t)i * Np];
            double* sl = &sn[(size_t)i * Np];
            const double* wq = &D.wq[out.off + i * Np];
            for (int j = 0; j < Np; ++j) {
                const double t = D.t[out.off + i * Np + j];
                ln[j] = (2.0 * t - a - b) / (b - a);
                double acc = 0.0;
                for (int m = 0; m < Np; ++m) acc += Q[(size_t)j * Np + m] * wq[m] / D.fej_w[m];
                sl[j] = S[i] + acc;
            }
            for (int j = 0; j < Np; ++j) {
                double q = 1.0, qs = 1.0;
                for (int m = 0; m < Np; ++m)
                    if (m != j) { q *= ln[j] - ln[m]; qs *= sl[j] - sl[m]; }
                lam[(size_t)i * Np + j] = 1.0 / q;
                lams[(size_t)i * Np + j] = 1.0 / qs;
            }
        }
    }, 16);
    // barycentric interpolation through the nodes xs (weights lw) of values v, at x
    auto bary = [&](const double* xs, const double* lw, double x, auto&& value) {
        double num = 0.0, den = 0.0;
        for (int j = 0; j < Np; ++j) {
            if (x == xs[j]) return value(j);
            const double c = lw[j] / (x - xs[j]);
            num += c * value(j);
            den += c;
        }
        return num / den;
    };
    // forward: each grid point's local coordinate in its patch, then its Np weights
    std::vector<int> fb((size_t)nu);
    std::vector<float> fw((size_t)nu * Np);
    parallel_for(nu, [&](long long g0, long long g1) {
        for (long long g = g0; g < g1; ++g) {
            const double sg = h * (double)g;
            // a grid point on a patch boundary (up to rounding) belongs to the patch that starts there
            int i = (int)(std::upper_bound(S.begin(), S.end(), sg + 1e-10 * L) - S.begin()) - 1;
            i = std::min(std::max(i, 0), P - 1);
            const double* ln = &loc[(size_t)i * Np];
            const double* lm = &lam[(size_t)i * Np];
            const double x = std::min(1.0, std::max(-1.0, bary(&sn[(size_t)i * Np], &lams[(size_t)i * Np], sg,
                                                               [&](int j) { return ln[j]; })));
            fb[(size_t)g] = (int)(out.off + (long long)i * Np);
            for (int j = 0; j < Np; ++j)
                fw[(size_t)g * Np + j] = (float)bary(ln, lm, x, [&](int m) { return m == j ? 1.0 : 0.0; });
        }
    }, 256);
    // back: kSpecTaps-point Lagrange weights on the grid at each node's arc length
    std::vector<int> bb((size_t)n);
    std::vector<float> bw((size_t)n * kSpecTaps);
    parallel_for(n, [&](long long j0, long long j1) {
        for (long long j = j0; j < j1; ++j) {
            const double x = sn[(size_t)j] / h;
            const long long q0 = (long long)std::floor(x) - (kSpecTaps / 2 - 1);
            const double xr = x - (double)q0;
            bb[(size_t)j] = (int)(((q0 % nu) + nu) % nu);
            for (int a = 0; a < kSpecTaps; ++a) {
                double v = 1.0;
                for (int m = 0; m < kSpecTaps; ++m) if (m != a) v *= (xr - m) / (double)(a - m);
                bw[(size_t)j * kSpecTaps + a] = (float)v;
            }
        }
    }, 256);
    // the multiplier in transposed order, and the twiddles
    std::vector<float2> mult((size_t)nu * 3), twN((size_t)nu), tw1(std::max(1, N1 / 2)), tw2(std::max(1, N2 / 2));
    const std::complex<double> ke(k, eps);
    for (int k1 = 0; k1 < N1; ++k1)
        for (int k2 = 0; k2 < N2; ++k2) {
            const long long q = k1 + (long long)N1 * k2;
            const double f = (double)(q < nu / 2 ? q : q - nu);
            const double xi = 2.0 * kPiH * f / L;
            const std::complex<double> sig = 0.5 + eta / (2.0 * std::sqrt(ke * ke - xi * xi));
            const std::complex<double> m = 1.0 / sig - 2.0;
            const double g = std::abs(sig);
            mult[(size_t)k1 * N2 + k2] = make_float2((float)m.real(), (float)m.imag());
            mult[(size_t)nu + (size_t)k1 * N2 + k2] = make_float2((float)(g - 0.5), 0.f);
            mult[2 * (size_t)nu + (size_t)k1 * N2 + k2] = make_float2((float)(1.0 / g - 2.0), 0.f);
            const long long a = ((long long)k1 * k2) % nu;
            const double th = -2.0 * kPiH * (double)a / (double)nu;
            twN[(size_t)k1 * N2 + k2] = make_float2((float)std::cos(th), (float)std::sin(th));
        }
    for (int j = 0; j < N1 / 2; ++j) { const double th = -2.0 * kPiH * j / N1; tw1[j] = make_float2((float)std::cos(th), (float)std::sin(th)); }
    for (int j = 0; j < N2 / 2; ++j) { const double th = -2.0 * kPiH * j / N2; tw2[j] = make_float2((float)std::cos(th), (float)std::sin(th)); }
    if (out.fw_base.upload(fb.data(), fb.size()) != cudaSuccess || out.fw_w.upload(fw.data(), fw.size()) != cudaSuccess ||
        out.bk_base.upload(bb.data(), bb.size()) != cudaSuccess || out.bk_w.upload(bw.data(), bw.size()) != cudaSuccess ||
        out.mult.upload(mult.data(), mult.size()) != cudaSuccess || out.twN.upload(twN.data(), twN.size()) != cudaSuccess ||
        out.tw1.upload(tw1.data(), tw1.size()) != cudaSuccess || out.tw2.upload(tw2.data(), tw2.size()) != cudaSuccess) {
        err = "uploading the spectral preconditioner's tables failed";
        return IFGF2D_ERR_CUDA;
    }
    return IFGF2D_OK;
}

}  // namespace

void free_spectral(ifgf2d_ctx* ctx) {
    delete ctx->sw;
    ctx->sw = nullptr;
}

// z = M r on the context's stream (capturable; the tables stay fixed until the next set-up):
// B interleaved vectors (point i of vector b at i * B + b; B = 1 for one vector) through the
// grid buffer `u` of B * spectral_grid_size(sw) values; four launches for all curves
void spectral_launch_batch(SpectralWork* sw, const double2* r, double2* z, int B, float2* u, int Np, cudaStream_t s, int which) {
    const double base = which == 1 ? 0.5 : 2.0;
    const long long us = sw->grid_total;
    const int nc = sw->ncurves;
    const int* pre = sw->pre.p;
    k_spec_fwd_cols<<<dim3(sw->blocks_cols, B), kSpecThreads, sw->smem_cols, s>>>(r, B, sw->desc.p, pre, nc, Np, u, us);
    k_spec_rows<<<dim3(sw->blocks_rows, B), kSpecThreads, sw->smem_rows, s>>>(sw->desc.p, pre + (nc + 1), nc, u, us, which);
    k_spec_inv_cols<<<dim3(sw->blocks_cols, B), kSpecThreads, sw->smem_cols, s>>>(sw->desc.p, pre, nc, u, us);
    k_spec_back<<<dim3(sw->blocks_back, B), 256, 0, s>>>(r, B, sw->desc.p, pre + 2 * (nc + 1), nc, u, us, base, z);
}
void spectral_launch(SpectralWork* sw, const double2* r, double2* z, int Np, cudaStream_t s, int which) {
    spectral_launch_batch(sw, r, z, 1, sw->u.p, Np, s, which);
}
long long spectral_grid_size(const SpectralWork* sw) { return sw ? sw->grid_total : 0; }

void launch_axpby(double2* z, double a, const double2* x, double b, const double2* y, long long n, cudaStream_t s) {
    k_axpby<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(z, a, x, b, y, n);
}
void launch_precond_sum(double2* z, const double2* zn, const double2* r, long long n, cudaStream_t s) {
    k_precond_sum<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(z, zn, r, n);
}

int spectral_setup(ifgf2d_ctx* ctx, double scale, const double* curve_k, const double* curve_eta) {
    const Discretisation& D = ctx->D;
    if (ctx->form != IFGF2D_COMBINED) return fail(ctx, IFGF2D_ERR_ARG, "the spectral preconditioner is for the combined-field formulation");
    if (!(scale > 0.0) || !std::isfinite(scale)) return fail(ctx, IFGF2D_ERR_ARG, "the glancing damping scale must be positive");
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) before the spectral preconditioner");
    if (ctx->sw && ctx->sw->scale == scale) return IFGF2D_OK;
    AllocStream guard(ctx->stream);
    if (ctx->gw) ctx->gw->drop_graphs();
    free_spectral(ctx);
    std::unique_ptr<SpectralWork> sw(new SpectralWork);
    long long covered = 0;
    for (int c = 0; c < (int)D.curves.size(); ++c) {
        std::unique_ptr<SpecCurve> sc(new SpecCurve);
        std::string err;
        const double kc = curve_k ? curve_k[c] : ctx->k, ec = curve_eta ? curve_eta[c] : ctx->eta;
        const int rc = build_curve(D, c, kc, ec, scale * std::cbrt(kc), *sc, err);
        if (rc != IFGF2D_OK) return fail(ctx, rc, err);
        covered += sc->n;
        sw->curves.push_back(std::move(sc));
    }
    if (covered != D.N) return fail(ctx, IFGF2D_ERR_ARG, "the spectral preconditioner needs every point on a closed curve");
    const int nc = (int)sw->curves.size();
    std::vector<SpecDesc> desc(nc);
    std::vector<int> pre(3 * (nc + 1), 0);
    long long uoff = 0, bc = 0, br = 0, bb = 0;
    for (int c = 0; c < nc; ++c) {
        const SpecCurve& sc = *sw->curves[c];
        const int N1 = 1 << sc.lg1, N2 = 1 << sc.lg2, cols = std::min(kSpecTile, N2);
        desc[c] = SpecDesc{sc.off, uoff, sc.n, sc.lg, sc.lg1, sc.lg2, sc.fw_base.p, sc.fw_w.p, sc.bk_base.p, sc.bk_w.p,
                           sc.mult.p, sc.twN.p, sc.tw1.p, sc.tw2.p};
        pre[c] = (int)bc; pre[(nc + 1) + c] = (int)br; pre[2 * (nc + 1) + c] = (int)bb;
        bc += N2 / cols; br += N1; bb += (sc.n + 255) / 256;
        uoff += 1LL << sc.lg;
        sw->smem_cols = std::max(sw->smem_cols, sizeof(float2) * (size_t)N1 * cols);
        sw->smem_rows = std::max(sw->smem_rows, sizeof(float2) * (size_t)N2);
    }
    if (bc > (1LL << 30) || br > (1LL << 30) || bb > (1LL << 30)) return fail(ctx, IFGF2D_ERR_ARG, "too many curves for the spectral preconditioner");
    pre[nc] = (int)bc; pre[2 * nc + 1] = (int)br; pre[3 * nc + 2] = (int)bb;
    sw->ncurves = nc; sw->blocks_cols = (int)bc; sw->blocks_rows = (int)br; sw->blocks_back = (int)bb;
    sw->grid_total = uoff;
    CK(sw->desc.upload(desc));
    CK(sw->pre.upload(pre));
    CK(sw->u.alloc((size_t)uoff));
    sw->scale = scale;
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->sw = sw.release();
    return IFGF2D_OK;
}

}  // namespace ifgf

extern "C" int ifgf2d_spectral_setup(ifgf2d_ctx* ctx, double scale) {
    if (!ctx) return IFGF2D_ERR_ARG;
    return ifgf::spectral_setup(ctx, scale <= 0.0 ? IFGF2D_SPECTRAL_DEFAULT_SCALE : scale);
}

extern "C" int ifgf2d_spectral_apply(ifgf2d_ctx* ctx, const double* r, double* z) {
    return ifgf2d_spectral_symbol(ctx, IFGF2D_SYMBOL_PRECONDITIONER, r, z);
}

extern "C" int ifgf2d_spectral_symbol(ifgf2d_ctx* ctx, int which, const double* r, double* z) {
    if (!ctx || !r || !z || which < 0 || which > 2) return IFGF2D_ERR_ARG;
    if (!ctx->sw) return fail(ctx, IFGF2D_ERR_STATE, "ifgf2d_spectral_setup first");
    const long long N = ctx->D.N;
    if (!all_finite(r, 2 * N)) return fail(ctx, IFGF2D_ERR_NONFINITE, "non-finite value in the residual");
    AllocStream guard(ctx->stream);
    DBuf<double2> dr, dz;
    CK(dr.alloc(N)); CK(dz.alloc(N));
    CK(cudaMemcpyAsync(dr.p, r, sizeof(double2) * N, cudaMemcpyHostToDevice, ctx->stream));
    ifgf::spectral_launch(ctx->sw, dr.p, dz.p, ctx->D.Np, ctx->stream, which);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(z, dz.p, sizeof(double2) * N, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return IFGF2D_OK;
}
