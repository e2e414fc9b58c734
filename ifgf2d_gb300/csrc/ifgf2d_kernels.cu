// ifgf2d_kernels.cu -- CUDA kernels of the GB300 IFGF2D forward map (FP64 plain form).
//
// Set-up kernels evaluate every geometry-only Green-function value once (rectangular-polar
// weights, near-field blocks, leaf-cone matrices) with the device Hankel evaluator and keep
// them resident in HBM.  Each apply streams them:
//   sing_apply   singular / near-singular correction        ForwardMap.tpp:481-515
//   intensities  density * quadrature weight (+ Morton perm) ForwardMap.tpp:425-435, BoxTree.h:954-963
//   direct_far   O(N^2) far sum with exclusions             ForwardMap.tpp:438-478
//   leaf_apply   leaf cone coefficients                      BoxTree.h:685-762
//   propagate    child -> parent cone coefficients           BoxTree.h:767-868
//   final        near field + all-level interpolation + un-permute
//                                                             BoxTree.h:614-683, 876-937, 1063-1069
#include "ifgf2d_kernels.cuh"
#include "hankel.cuh"

namespace ifgf {

// ------------------------------------------------------------------ small helpers
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
    acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------------ set-up: near field
// One CTA per leaf box: block [target][source] over the neighbour boxes' points (sources in
// neighbour order), zero for excluded pairs (self, same patch, near-singular patches of the
// target).
__global__ void k_near_setup(const int* __restrict__ leaf_start, const int* __restrict__ leaf_count,
                             const int* __restrict__ nbr_ptr, const int* __restrict__ nbr_box,
                             const long long* __restrict__ near_off, const double* __restrict__ xs,
                             const double* __restrict__ ys, const double* __restrict__ nxs, const double* __restrict__ nys,
                             const int* __restrict__ patch_s, const int* __restrict__ nsp_ptr, const int* __restrict__ nsp,
                             double k0, int form, double eta0, const double2* __restrict__ keta, double2* __restrict__ near) {
    const int b = blockIdx.x;
    const double k = keta ? keta[b].x : k0, eta = keta ? keta[b].y : eta0;   // per leaf box for a group of obstacles
    const int nB = leaf_count[b], t0 = leaf_start[b];
    const int n0 = nbr_ptr[b], n1 = nbr_ptr[b + 1];
    int nsrc = 0;
    for (int q = n0; q < n1; ++q) nsrc += leaf_count[nbr_box[q]];
    const long long total = (long long)nsrc * nB;
    for (long long e = threadIdx.x; e < total; e += blockDim.x) {
        const int t = (int)(e / nsrc), s = (int)(e % nsrc);
        int rem = s, j = -1;
        for (int q = n0; q < n1; ++q) {
            const int c = leaf_count[nbr_box[q]];
            if (rem < c) { j = leaf_start[nbr_box[q]] + rem; break; }
            rem -= c;
        }
        const int i = t0 + t;
        double2 v = make_double2(0.0, 0.0);
        bool skip = (j == i) || (patch_s[j] == patch_s[i]);
        for (int q = nsp_ptr[i]; q < nsp_ptr[i + 1] && !skip; ++q) skip = (nsp[q] == patch_s[j]);
        if (!skip) v = green_form(form, xs[i] - xs[j], ys[i] - ys[j], nxs[j], nys[j], k, eta);
        near[near_off[b] + e] = v;
    }
}

// ------------------------------------------------------------------ set-up: leaf cones
// One warp per (leaf cone, source): lanes are the P interpolation nodes; each lane evaluates
// G(source, node) / (e^{ikr}/sqrt r), then the values-to-coefficients map (Interpolator.h:81-120)
// is applied across lanes.  L layout: [cone][source][coefficient].
// block = one leaf cone, warp = one source at a time: the Green values at the cone's P nodes
// (node l * Ps + q: angular l, radial q) times 1/factorization, then the values -> coefficients
// map in separable form through the warp's shared memory, u[l][m] = sum_q Gs[m][q] h[l][q] and
// c[n * Ps + m] = sum_l Ga[n][l] u[l][m].  Up to 64 nodes (two per lane).
constexpr int kLeafSetupWarps = 8;
__global__ void __launch_bounds__(kLeafSetupWarps * 32) k_leaf_setup(const int* __restrict__ cone_box, int ncones,
                                                                     const int* __restrict__ leaf_start,
                                                                     const int* __restrict__ leaf_count,
                                                                     const long long* __restrict__ leaf_off,
                                                                     const LeafNode* __restrict__ nodes, const double* __restrict__ xs,
                                                                     const double* __restrict__ ys, const double* __restrict__ nxs,
                                                                     const double* __restrict__ nys, int Ps, int Pa, double k0, int form,
                                                                     double eta0, const double2* __restrict__ keta,
                                                                     const double* __restrict__ Gsep, double2* __restrict__ L) {
    __shared__ double sG[2 * 64];
    __shared__ double2 hv[kLeafSetupWarps][64], uv[kLeafSetupWarps][64];
    for (int i = threadIdx.x; i < Ps * Ps + Pa * Pa; i += blockDim.x) sG[i] = Gsep[i];
    __syncthreads();
    const double* Gs = sG;
    const double* Ga = sG + Ps * Ps;
    const int P = Ps * Pa;
    const int c = blockIdx.x;
    if (c >= ncones) return;
    const double k = keta ? keta[c].x : k0, eta = keta ? keta[c].y : eta0;   // per cone for a group of obstacles
    const int b = cone_box[c];
    const int n = leaf_count[b], s0 = leaf_start[b];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    LeafNode nd[2];
#pragma unroll
    for (int h2 = 0; h2 < 2; ++h2) {
        const int q = lane + 32 * h2;
        nd[h2] = q < P ? nodes[(long long)c * P + q] : LeafNode{0, 0, 0, 0};
    }
    for (int s = warp; s < n; s += kLeafSetupWarps) {
        const int j = s0 + s;
        const double xj = xs[j], yj = ys[j], nxj = nxs[j], nyj = nys[j];
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const int q = lane + 32 * h2;
            if (q < P)
                hv[warp][q] = cmul(green_form(form, nd[h2].x - xj, nd[h2].y - yj, nxj, nyj, k, eta), make_double2(nd[h2].ir, nd[h2].ii));
        }
        __syncwarp();
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const int o = lane + 32 * h2;
            if (o < P) {
                const int l = o / Ps, m = o - (o / Ps) * Ps;
                double2 u = make_double2(0.0, 0.0);
                for (int q = 0; q < Ps; ++q) {
                    const double g = Gs[m * Ps + q];
                    const double2 v = hv[warp][l * Ps + q];
                    u.x = fma(g, v.x, u.x); u.y = fma(g, v.y, u.y);
                }
                uv[warp][o] = u;
            }
        }
        __syncwarp();
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2) {
            const int o = lane + 32 * h2;
            if (o < P) {
                const int nn = o / Ps, m = o - (o / Ps) * Ps;
                double2 a = make_double2(0.0, 0.0);
                for (int l = 0; l < Pa; ++l) {
                    const double g = Ga[nn * Pa + l];
                    const double2 v = uv[warp][l * Ps + m];
                    a.x = fma(g, v.x, a.x); a.y = fma(g, v.y, a.y);
                }
                L[leaf_off[c] + (long long)s * P + o] = a;
            }
        }
        __syncwarp();   // hv and uv are rewritten for the next source
    }
}

// ------------------------------------------------------------------ apply: singular part
// Eight lanes per output row: lane k8 takes the nodes k = k8, k8+8, ... of every weight column of
// the row, then the row's eight partial sums are reduced with shuffles.  Optionally also writes
// the row's quadrature-weighted density into rho64 / rho32 at inv[o] (the Morton position) or
// at o, which fuses ForwardMap::compute_intensities into the same pass.
template <typename RhoT>
__global__ void k_sing_apply(const double2* __restrict__ x, const double2* __restrict__ W, const int* __restrict__ row_ptr,
                             const int* __restrict__ row_col, const RPColumn* __restrict__ cols, int N, int Np,
                             double half, double2* __restrict__ y, const double* __restrict__ wq,
                             const long long* __restrict__ inv, RhoT* __restrict__ rho) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int o = (int)(t >> 3), k8 = (int)(t & 7);
    const bool active = o < N;
    double2 acc = make_double2(0.0, 0.0);
    if (active) {
        for (int q = row_ptr[o]; q < row_ptr[o + 1]; ++q) {
            const int col = row_col[q];
            const double2* w = W + (long long)col * Np;
            const double2* d = x + (long long)cols[col].patch * Np;
            for (int kk = k8; kk < Np; kk += 8) cfma(acc, d[kk], w[kk]);
        }
    }
#pragma unroll
    for (int off = 4; off > 0; off >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
    }
    if (active && k8 == 0) {
        const double2 v = x[o];
        if (half != 0.0) { acc.x += half * v.x; acc.y += half * v.y; }   // jump term
        y[o] = acc;
        if (rho) {
            const double wv = wq[o];
            RhoT r; r.x = v.x * wv; r.y = v.y * wv;
            rho[inv ? inv[o] : o] = r;
        }
    }
}

// ------------------------------------------------------------------ apply: direct far sum
// Tiled all-pairs sum, one thread per target, sources staged in shared memory 128 at a time.
// A tile whose patch range holds neither the target's patch nor a patch the target is
// near-singular to runs without exclusion tests.
constexpr int kTile = 128;
__global__ void __launch_bounds__(kTile) k_direct_far(const double* __restrict__ tx, const double* __restrict__ ty, int nt,
                             const int* __restrict__ t_patch, const int* __restrict__ t_nsp_ptr, const int* __restrict__ t_nsp,
                             const double* __restrict__ sx, const double* __restrict__ sy, const double* __restrict__ snx,
                             const double* __restrict__ sny, const int* __restrict__ s_patch,
                             const double2* __restrict__ rho, int ns, double k, int form, double eta,
                             double2* __restrict__ y, int accumulate) {
    __shared__ double shx[kTile], shy[kTile], shnx[kTile], shny[kTile];
    __shared__ double2 shr[kTile];
    __shared__ int shp[kTile];
    const int i = blockIdx.x * kTile + threadIdx.x;
    const bool active = i < nt;
    const double xi = active ? tx[i] : 0.0, yi = active ? ty[i] : 0.0;
    const int pi = (active && t_patch) ? t_patch[i] : -1;
    int ex[8], nex = 0;
    if (active && t_nsp_ptr) for (int q = t_nsp_ptr[i]; q < t_nsp_ptr[i + 1] && nex < 8; ++q) ex[nex++] = t_nsp[q];
    double2 acc = make_double2(0.0, 0.0);
    for (int s0 = 0; s0 < ns; s0 += kTile) {
        const int n = min(kTile, ns - s0);
        __syncthreads();
        if (threadIdx.x < n) {
            const int j = s0 + threadIdx.x;
            shx[threadIdx.x] = sx[j]; shy[threadIdx.x] = sy[j]; shr[threadIdx.x] = rho[j];
            shnx[threadIdx.x] = snx ? snx[j] : 0.0; shny[threadIdx.x] = sny ? sny[j] : 0.0;
            shp[threadIdx.x] = s_patch ? s_patch[j] : -2;
        }
        __syncthreads();
        if (!active) continue;
        const int pa = shp[0], pb = shp[n - 1];
        bool check = s_patch && (pi >= pa && pi <= pb);
        for (int q = 0; q < nex; ++q) check |= (ex[q] >= pa && ex[q] <= pb);
        if (!check) {
            for (int j = 0; j < n; ++j) cfma(acc, green_form(form, xi - shx[j], yi - shy[j], shnx[j], shny[j], k, eta), shr[j]);
        } else {
            for (int j = 0; j < n; ++j) {
                const int pj = shp[j];
                bool skip = (pj == pi);
                for (int q = 0; q < nex; ++q) skip |= (ex[q] == pj);
                if (!skip) cfma(acc, green_form(form, xi - shx[j], yi - shy[j], shnx[j], shny[j], k, eta), shr[j]);
            }
        }
    }
    if (active) {
        if (accumulate) { double2 v = y[i]; y[i] = cadd(v, acc); } else y[i] = acc;
    }
}

// The same sum with one 128-thread block per target, for target counts that would leave most
// SMs idle with one thread per target (N = 200: 2 blocks).  Thread t takes sources t, t + 128, ...;
// the partial sums combine in a fixed order (warp butterfly, then warps 0..3), so the result
// does not depend on scheduling.
constexpr int kDirectSplitBelow = 2 * 152 * kTile;
__global__ void __launch_bounds__(kTile) k_direct_far_split(const double* __restrict__ tx, const double* __restrict__ ty,
                             const int* __restrict__ t_patch, const int* __restrict__ t_nsp_ptr, const int* __restrict__ t_nsp,
                             const double* __restrict__ sx, const double* __restrict__ sy, const double* __restrict__ snx,
                             const double* __restrict__ sny, const int* __restrict__ s_patch,
                             const double2* __restrict__ rho, int ns, double k, int form, double eta,
                             double2* __restrict__ y, int accumulate) {
    __shared__ double2 part[kTile / 32];
    const int i = blockIdx.x;
    const double xi = tx[i], yi = ty[i];
    const int pi = t_patch ? t_patch[i] : -1;
    int ex[8], nex = 0;
    if (t_nsp_ptr) for (int q = t_nsp_ptr[i]; q < t_nsp_ptr[i + 1] && nex < 8; ++q) ex[nex++] = t_nsp[q];
    double2 acc = make_double2(0.0, 0.0);
    for (int j = threadIdx.x; j < ns; j += kTile) {
        bool skip = false;
        if (s_patch) {
            const int pj = s_patch[j];
            skip = (pj == pi);
            for (int q = 0; q < nex; ++q) skip |= (ex[q] == pj);
        }
        if (!skip) cfma(acc, green_form(form, xi - sx[j], yi - sy[j], snx ? snx[j] : 0.0, sny ? sny[j] : 0.0, k, eta), rho[j]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 t = part[0];
        for (int w = 1; w < kTile / 32; ++w) t = cadd(t, part[w]);
        if (accumulate) { const double2 v = y[i]; y[i] = cadd(v, t); } else y[i] = t;
    }
}

// ------------------------------------------------------------------ tests and GMRES helpers
__global__ void k_hankel(int order, const double* __restrict__ x, int n, double2* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (order >= 2) {   // the fused evaluator of the combined-field kernel: 2 -> its H0, 3 -> its H1
        double2 h0, h1;
        hankel01(x[i], h0, h1);
        out[i] = order == 2 ? h0 : h1;
        return;
    }
    out[i] = order == 0 ? hankel1<0>(x[i]) : hankel1<1>(x[i]);
}

// h[j] = sum_i conj(V[j][i]) w[i]
__global__ void k_multidot(const double2* __restrict__ V, long long ldv, const double2* __restrict__ w, long long n,
                           double2* __restrict__ h) {
    const int j = blockIdx.x;
    const double2* v = V + (long long)j * ldv;
    double re = 0.0, im = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 a = v[i], b = w[i];
        re = fma(a.x, b.x, fma(a.y, b.y, re));
        im = fma(a.x, b.y, fma(-a.y, b.x, im));
    }
    __shared__ double sr[32], si[32];
    re = warp_sum(re); im = warp_sum(im);
    if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = re; si[threadIdx.x >> 5] = im; }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x >> 5;
        re = threadIdx.x < nw ? sr[threadIdx.x] : 0.0; im = threadIdx.x < nw ? si[threadIdx.x] : 0.0;
        re = warp_sum(re); im = warp_sum(im);
        if (threadIdx.x == 0) h[j] = make_double2(re, im);
    }
}
// w[i] += sign * sum_j V[j][i] h[j]
__global__ void k_multi_axpy(const double2* __restrict__ V, long long ldv, int ncols, const double2* __restrict__ h, double sign,
                             long long n, double2* __restrict__ w) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 acc = make_double2(0.0, 0.0);
    for (int j = 0; j < ncols; ++j) cfma(acc, V[(long long)j * ldv + i], h[j]);
    double2 v = w[i];
    v.x += sign * acc.x; v.y += sign * acc.y;
    w[i] = v;
}
__global__ void k_scale(const double2* __restrict__ w, double2 a, long long n, double2* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = cmul(w[i], a);
}
__global__ void k_sub(const double2* __restrict__ a, const double2* __restrict__ b, long long n, double2* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_double2(a[i].x - b[i].x, a[i].y - b[i].y);
}
__global__ void k_nonfinite(const double2* __restrict__ v, long long n, int* __restrict__ flag) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && !(isfinite(v[i].x) && isfinite(v[i].y))) atomicOr(flag, 1);
}

// ------------------------------------------------------------------ device-side Arnoldi bookkeeping
// ---- variants that read the Arnoldi index j from device memory, for a captured iteration graph
__global__ void k_copy_col(const double2* __restrict__ V, long long n, const int* __restrict__ jp, double2* __restrict__ out,
                           double* __restrict__ nrm2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = V[(long long)(*jp) * n + i];
    if (i == 0 && nrm2) *nrm2 = 0.0;
}
// h[c] = V[:, c]^H w for c <= *jp in two deterministic stages: blocks (row chunk, column)
// write partial sums, then one thread per column adds its chunks in order.  The grid spans
// every column and row chunk, so even the first iterations keep all SMs busy.
constexpr int kDotChunk = 2048;
__global__ void __launch_bounds__(256) k_multidot_part(const double2* __restrict__ V, long long ldv, const int* __restrict__ jp,
                                                       const double2* __restrict__ w, long long n, double2* __restrict__ part) {
    const int col = blockIdx.y;
    if (col > *jp) return;
    const int chunk = blockIdx.x;
    const long long i0 = (long long)chunk * kDotChunk;
    const long long i1 = i0 + kDotChunk < n ? i0 + kDotChunk : n;
    const double2* v = V + (long long)col * ldv;
    double re = 0.0, im = 0.0;
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double2 a = v[i], b = w[i];
        re = fma(a.x, b.x, fma(a.y, b.y, re));
        im = fma(a.x, b.y, fma(-a.y, b.x, im));
    }
    __shared__ double sr[8], si[8];
    re = warp_sum(re); im = warp_sum(im);
    if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = re; si[threadIdx.x >> 5] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += sr[q]; b += si[q]; }
        part[(long long)col * gridDim.x + chunk] = make_double2(a, b);
    }
}
__global__ void k_multidot_fin(const double2* __restrict__ part, int nchunk, const int* __restrict__ jp, int ncol,
                               double2* __restrict__ h) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ncol || col > *jp) return;
    double a = 0.0, b = 0.0;
    for (int q = 0; q < nchunk; ++q) { const double2 v = part[(long long)col * nchunk + q]; a += v.x; b += v.y; }
    h[col] = make_double2(a, b);
}
// Z[:, *jp] = z (flexible GMRES keeps the preconditioned vectors)
__global__ void k_store_col(const double2* __restrict__ z, long long n, const int* __restrict__ jp, double2* __restrict__ Z) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) Z[(long long)(*jp) * n + i] = z[i];
}
__global__ void k_multidot_dyn(const double2* __restrict__ V, long long ldv, const int* __restrict__ jp,
                               const double2* __restrict__ w, long long n, double2* __restrict__ h) {
    const int j = blockIdx.x;
    if (j > *jp) return;
    const double2* v = V + (long long)j * ldv;
    double re = 0.0, im = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 a = v[i], b = w[i];
        re = fma(a.x, b.x, fma(a.y, b.y, re));
        im = fma(a.x, b.y, fma(-a.y, b.x, im));
    }
    __shared__ double sr[32], si[32];
    re = warp_sum(re); im = warp_sum(im);
    if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = re; si[threadIdx.x >> 5] = im; }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x >> 5;
        re = threadIdx.x < nw ? sr[threadIdx.x] : 0.0; im = threadIdx.x < nw ? si[threadIdx.x] : 0.0;
        re = warp_sum(re); im = warp_sum(im);
        if (threadIdx.x == 0) h[j] = make_double2(re, im);
    }
}
// w -= V[:, 0..j] h: 64 rows per block, four threads per row split the columns (j = part mod 4);
// block 0 also writes (add = 0) or adds (add = 1) h into the Hessenberg column j.
__global__ void __launch_bounds__(256) k_cgs_update_dyn(const double2* __restrict__ V, long long ldv, const int* __restrict__ jp,
                                                        const double2* __restrict__ h, long long n, double2* __restrict__ w,
                                                        double2* __restrict__ H, int ldh, int add, double* __restrict__ nrm2) {
    __shared__ double2 part[4][64];
    __shared__ double npart[2];
    const int r = threadIdx.x & 63, q = threadIdx.x >> 6;
    const long long i = (long long)blockIdx.x * 64 + r;
    const int j = *jp;
    double2 acc = make_double2(0.0, 0.0);
    if (i < n)
        for (int c = q; c <= j; c += 4) cfma(acc, V[(long long)c * ldv + i], h[c]);
    part[q][r] = acc;
    __syncthreads();
    double sq = 0.0;
    if (q == 0 && i < n) {
        double2 v = w[i];
        v.x -= part[0][r].x + part[1][r].x + part[2][r].x + part[3][r].x;
        v.y -= part[0][r].y + part[1][r].y + part[2][r].y + part[3][r].y;
        w[i] = v;
        sq = v.x * v.x + v.y * v.y;
    }
    if (nrm2 && q == 0) {   // ||w||^2 of the updated vector: warps 0 and 1 hold the 64 rows
        sq = warp_sum(sq);
        if ((threadIdx.x & 31) == 0) npart[threadIdx.x >> 5] = sq;
    }
    __syncthreads();
    if (nrm2 && threadIdx.x == 0) atomicAdd(nrm2, npart[0] + npart[1]);
    if (blockIdx.x == 0)
        for (int c = threadIdx.x; c <= j; c += blockDim.x) {
            double2* col = H + (long long)j * ldh;
            if (add) { col[c].x += h[c].x; col[c].y += h[c].y; } else col[c] = h[c];
        }
}
// h_{j+1,j} = ||w|| from the accumulated square; V[:, j+1] = w / h_{j+1,j}; block 0 stores
// h_{j+1,j} in the Hessenberg matrix (j is advanced by the next kernel)
__global__ void k_scale_next(const double2* __restrict__ w, const double* __restrict__ nrm2, long long n,
                             double2* __restrict__ V, const int* __restrict__ jp, double2* __restrict__ H, int ldh) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = *jp;
    const double hn = sqrt(fmax(*nrm2, 0.0));
    const double a = hn != 0.0 ? 1.0 / hn : 0.0;
    if (i < n) V[(long long)(j + 1) * n + i] = make_double2(w[i].x * a, w[i].y * a);
    if (i == 0) H[(long long)j * ldh + j + 1] = make_double2(hn, 0.0);
}
__global__ void k_advance(int* __restrict__ jp) { if (threadIdx.x == 0 && blockIdx.x == 0) *jp += 1; }

// dependent FP64 FMA chains, 8 independent chains per thread
__global__ void k_fp64_peak(double* out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = threadIdx.x * 1e-9 + q;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < 8; ++q) x[q] = fma(x[q], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += x[q];
    if (s == 12345.678) out[0] = s;   // keeps the chains alive
}

// ------------------------------------------------------------------ launchers
static inline unsigned nblk(long long n, int b) { return (unsigned)((n + b - 1) / b); }

void launch_near_setup(const int* leaf_start, const int* leaf_count, const int* nbr_ptr, const int* nbr_box,
                       const long long* near_off, int nleaf, const double* xs, const double* ys, const double* nxs,
                       const double* nys, const int* patch_s, const int* nsp_ptr, const int* nsp, double k, int form,
                       double eta, double2* near, cudaStream_t s, const double2* keta) {
    if (nleaf <= 0) return;
    k_near_setup<<<nleaf, 256, 0, s>>>(leaf_start, leaf_count, nbr_ptr, nbr_box, near_off, xs, ys, nxs, nys, patch_s, nsp_ptr,
                                       nsp, k, form, eta, keta, near);
}
void launch_leaf_setup(const int* cone_box, int ncones, const int* leaf_start, const int* leaf_count, const long long* leaf_off,
                       const LeafNode* nodes, const double* xs, const double* ys, const double* nxs, const double* nys, int Ps,
                       int Pang, double k, int form, double eta, const double* Gsep, double2* L, cudaStream_t s,
                       const double2* keta) {
    if (ncones <= 0 || Ps * Pang > 64 || Ps * Ps + Pang * Pang > 128) return;
    k_leaf_setup<<<ncones, kLeafSetupWarps * 32, 0, s>>>(cone_box, ncones, leaf_start, leaf_count, leaf_off, nodes, xs, ys, nxs, nys, Ps, Pang, k,
                                        form, eta, keta, Gsep, L);
}
void launch_sing_apply(const double2* x, const double2* W, const int* row_ptr, const int* row_col, const RPColumn* cols,
                       int N, int Np, double half, double2* y, cudaStream_t s) {
    k_sing_apply<double2><<<nblk((long long)N * 8, 256), 256, 0, s>>>(x, W, row_ptr, row_col, cols, N, Np, half, y, nullptr,
                                                                       nullptr, (double2*)nullptr);
}
void launch_sing_intens(const double2* x, const double2* W, const int* row_ptr, const int* row_col, const RPColumn* cols,
                        int N, int Np, double half, double2* y, const double* wq, const long long* inv, double2* rho64,
                        float2* rho32, cudaStream_t s) {
    if (rho32)
        k_sing_apply<float2><<<nblk((long long)N * 8, 256), 256, 0, s>>>(x, W, row_ptr, row_col, cols, N, Np, half, y, wq, inv, rho32);
    else
        k_sing_apply<double2><<<nblk((long long)N * 8, 256), 256, 0, s>>>(x, W, row_ptr, row_col, cols, N, Np, half, y, wq, inv, rho64);
}
void launch_direct_far(const double* tx, const double* ty, int nt, const int* t_patch, const int* t_nsp_ptr, const int* t_nsp,
                       const double* sx, const double* sy, const double* snx, const double* sny, const int* s_patch,
                       const double2* rho, int ns, double k, int form, double eta, double2* y, int accumulate, cudaStream_t s) {
    if (nt <= 0) return;
    if (nt < kDirectSplitBelow)
        k_direct_far_split<<<nt, kTile, 0, s>>>(tx, ty, t_patch, t_nsp_ptr, t_nsp, sx, sy, snx, sny, s_patch, rho, ns, k, form, eta,
                                                y, accumulate);
    else
        k_direct_far<<<nblk(nt, kTile), kTile, 0, s>>>(tx, ty, nt, t_patch, t_nsp_ptr, t_nsp, sx, sy, snx, sny, s_patch, rho, ns, k,
                                                       form, eta, y, accumulate);
}
cudaError_t preload_direct_kernels() {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, k_sing_apply<double2>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_direct_far_split);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_direct_far);
    return e;
}
void launch_hankel(int order, const double* x, int n, double2* out, cudaStream_t s) {
    if (n <= 0) return;
    k_hankel<<<nblk(n, 256), 256, 0, s>>>(order, x, n, out);
}
void launch_multidot(const double2* V, long long ldv, int ncols, const double2* w, long long n, double2* h, cudaStream_t s) {
    if (ncols <= 0) return;
    k_multidot<<<ncols, 256, 0, s>>>(V, ldv, w, n, h);
}
void launch_multi_axpy(const double2* V, long long ldv, int ncols, const double2* h, double sign, long long n, double2* w, cudaStream_t s) {
    k_multi_axpy<<<nblk(n, 256), 256, 0, s>>>(V, ldv, ncols, h, sign, n, w);
}
void launch_scale(const double2* w, double2 a, long long n, double2* out, cudaStream_t s) {
    k_scale<<<nblk(n, 256), 256, 0, s>>>(w, a, n, out);
}
void launch_sub(const double2* a, const double2* b, long long n, double2* out, cudaStream_t s) {
    k_sub<<<nblk(n, 256), 256, 0, s>>>(a, b, n, out);
}
int arnoldi_part_size(long long n, int m) { return (int)(((n + kDotChunk - 1) / kDotChunk) * (m + 1)); }
void launch_arnoldi_step(double2* V, long long n, int m, int* jp, double2* w, double2* h, double2* H, double* nrm2,
                         double2* part, cudaStream_t s, int passes, const LsqDev* lsq, cudaGraphConditionalHandle cond,
                         bool use_cond) {
    // w holds A v_j on entry (the apply ran between k_copy_col and this call)
    const int ldh = m + 1;
    for (int pass = 0; pass < passes; ++pass) {   // classical Gram-Schmidt; the last pass sums ||w||^2
        const int nchunk = (int)((n + kDotChunk - 1) / kDotChunk);
        k_multidot_part<<<dim3(nchunk, m + 1), 256, 0, s>>>(V, n, jp, w, n, part);
        k_multidot_fin<<<nblk(m + 1, 128), 128, 0, s>>>(part, nchunk, jp, m + 1, h);
        k_cgs_update_dyn<<<nblk(n, 64), 256, 0, s>>>(V, n, jp, h, n, w, H, ldh, pass, pass == passes - 1 ? nrm2 : nullptr);
    }
    k_scale_next<<<nblk(n, 256), 256, 0, s>>>(w, nrm2, n, V, jp, H, ldh);
    if (lsq) launch_lsq_givens(H, ldh, jp, *lsq, cond, use_cond, s);
    else k_advance<<<1, 32, 0, s>>>(jp);
}
void launch_store_col(const double2* z, long long n, const int* jp, double2* Z, cudaStream_t s) {
    k_store_col<<<nblk(n, 256), 256, 0, s>>>(z, n, jp, Z);
}
void launch_copy_col(const double2* V, long long n, const int* jp, double2* out, double* nrm2, cudaStream_t s) {
    k_copy_col<<<nblk(n, 256), 256, 0, s>>>(V, n, jp, out, nrm2);
}
bool launch_fp64_peak(double* tflops) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return false;
    const int blocks = sms * 8, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    k_fp64_peak<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);   // warm-up
    cudaEventRecord(e0);
    k_fp64_peak<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    const bool ok = cudaEventSynchronize(e1) == cudaSuccess && cudaGetLastError() == cudaSuccess;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaFree(out);
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    return ok;
}
void launch_nonfinite_check(const double2* v, long long n, int* flag, cudaStream_t s) {
    k_nonfinite<<<nblk(n, 256), 256, 0, s>>>(v, n, flag);
}

}  // namespace ifgf
