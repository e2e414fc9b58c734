// gmres_device.cu -- the least-squares half of GMRES on the device.
//
// The reference's opgmres (ForwardMap/opGMRES.hpp:183-218) applies the Givens rotations of the
// earlier columns to each new Hessenberg column, forms the next rotation, updates the rotated
// right-hand side g and tests |g_{k}| / ||r0|| against the tolerance; at the end of a cycle it
// solves the triangular system R y = g.  Here that work runs in small kernels on the context's
// stream, so an iteration needs nothing from the host:
// * k_lsq_givens (one thread) after each Arnoldi step, inside the captured iteration graph.
//   It also sets the condition of the CUDA graph while-loop that repeats the iteration, so one
//   graph launch runs a whole restart cycle with no host round trip.
// * k_lsq_solve (one warp) once per cycle: column-oriented back-substitution.
// * batched forms for B right-hand sides in lock step: one thread (rotations) or one warp
//   (back-substitution) per right-hand side.
// The rotations are Eigen's JacobiRotation::makeGivens, complex case, which the reference's
// opgmres calls (opGMRES.hpp:193), written on double2.
#include "ifgf2d_kernels.cuh"

namespace ifgf {
namespace {

__device__ __forceinline__ double2 c_mul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 c_conj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 c_scale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double c_abs(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ double c_norm(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ bool c_zero(double2 a) { return a.x == 0.0 && a.y == 0.0; }
__device__ __forceinline__ double2 c_div(double2 a, double2 b) {
    const double d = 1.0 / c_norm(b);
    return c_scale(c_mul(a, c_conj(b)), d);
}

// Givens rotation G = [c, conj(s); -s, c] (c real) with G^* [p; q] = [r; 0]
__device__ void make_givens(double2 p, double2 q, double& c, double2& s) {
    if (c_zero(q)) {
        c = p.x < 0 ? -1.0 : 1.0;
        s = make_double2(0.0, 0.0);
        return;
    }
    if (c_zero(p)) {
        c = 0.0;
        s = c_scale(q, -1.0 / c_abs(q));
        return;
    }
    const double p1 = fabs(p.x) + fabs(p.y), q1 = fabs(q.x) + fabs(q.y);
    if (p1 >= q1) {
        const double2 ps = c_scale(p, 1.0 / p1), qs = c_scale(q, 1.0 / p1);
        const double p2 = c_norm(ps), q2 = c_norm(qs);
        double u = sqrt(1.0 + q2 / p2);
        if (p.x < 0) u = -u;
        c = 1.0 / u;
        s = c_scale(c_mul(qs, c_conj(ps)), -c / p2);
    } else {
        double2 ps = c_scale(p, 1.0 / q1);
        const double2 qs = c_scale(q, 1.0 / q1);
        const double p2 = c_norm(ps), q2 = c_norm(qs);
        double u = q1 * sqrt(p2 + q2);
        if (p.x < 0) u = -u;
        const double pa = c_abs(p);
        ps = c_scale(p, 1.0 / pa);
        c = pa / u;
        s = c_scale(c_mul(c_conj(ps), c_scale(q, 1.0 / u)), -1.0);
    }
}
// (x, y) <- G^* (x, y)
__device__ __forceinline__ void rotate(double c, double2 s, double2& x, double2& y) {
    const double2 nx = make_double2(c * x.x - (s.x * y.x + s.y * y.y), c * x.y - (s.x * y.y - s.y * y.x));
    const double2 sx = c_mul(s, x);
    y = make_double2(sx.x + c * y.x, sx.y + c * y.y);
    x = nx;
}

// One column: rotate H column j (rows 0..j+1, stride hs) into R column j, update g, and
// return the new residual estimate.  gc / gs hold the rotations, g the rotated right-hand side.
__device__ double givens_column(const double2* h, long long hs, int j, double2* col, double* gc, double2* gs, double2* g,
                                double r0n, double& hn) {
    for (int i = 0; i <= j; ++i) col[i] = h[(long long)i * hs];
    double2 sub = h[(long long)(j + 1) * hs];
    hn = c_abs(sub);
    for (int i = 0; i < j; ++i) rotate(gc[i], gs[i], col[i], col[i + 1]);
    double c = 1.0;
    double2 s = make_double2(0.0, 0.0);
    if (!c_zero(sub)) {
        make_givens(col[j], sub, c, s);
        rotate(c, s, col[j], sub);
        rotate(c, s, g[j], g[j + 1]);
    }
    col[j + 1] = sub;
    gc[j] = c;
    gs[j] = s;
    return c_abs(g[j + 1]) / r0n;
}

__global__ void k_lsq_init(LsqDev L, int* jp, double beta, double r0n, double tol, int limit) {
    for (int i = threadIdx.x; i <= L.m; i += blockDim.x) L.g[i] = make_double2(i == 0 ? beta : 0.0, 0.0);
    if (threadIdx.x == 0) {
        *jp = 0;
        L.st[0] = 0; L.st[1] = 0; L.st[2] = limit; L.st[3] = 0;
        L.sc[0] = 1.0; L.sc[1] = r0n; L.sc[2] = tol;
    }
}

__global__ void k_lsq_givens(const double2* __restrict__ H, int ldh, int* __restrict__ jp, LsqDev L,
                             cudaGraphConditionalHandle cond, int use_cond) {
    if (threadIdx.x != 0) return;
    const int j = *jp;
    int* st = L.st;
    if (st[0] || j >= L.m) {   // a stopped cycle stays stopped
        if (use_cond) cudaGraphSetConditional(cond, 0);
        return;
    }
    double hn = 0.0;
    const double est = givens_column(H + (long long)j * ldh, 1, j, L.R + (long long)j * ldh, L.gc, L.gs, L.g, L.sc[1], hn);
    const int it = st[3] + 1;
    st[3] = it;
    L.sc[0] = est;
    // converged (a NaN estimate stops too), out of iterations, or an exact Krylov subspace
    const bool stop = !(est >= L.sc[2]) || it >= st[2] || hn == 0.0;
    st[1] = j + 1;
    if (stop) st[0] = 1;
    *jp = j + 1;
    if (use_cond) cudaGraphSetConditional(cond, (stop || j + 1 >= L.m) ? 0u : 1u);
}

// y = R^{-1} g over the first st[1] columns, one warp: for i from the last column down, y_i =
// t_i / R_ii, then t_q -= R_qi y_i for q < i (t starts as g and is kept in y)
__global__ void k_lsq_solve(LsqDev L, int ldh, double2* __restrict__ y) {
    const int lane = threadIdx.x;
    const int k = L.st[1];
    for (int q = lane; q < k; q += 32) y[q] = L.g[q];
    __syncwarp();
    for (int i = k - 1; i >= 0; --i) {
        const double2* Ri = L.R + (long long)i * ldh;
        double2 yi = make_double2(0.0, 0.0);
        if (lane == 0) {
            yi = c_div(y[i], Ri[i]);
            y[i] = yi;
        }
        yi.x = __shfl_sync(0xffffffffu, yi.x, 0);
        yi.y = __shfl_sync(0xffffffffu, yi.y, 0);
        for (int q = lane; q < i; q += 32) {
            const double2 t = c_mul(Ri[q], yi);
            y[q] = make_double2(y[q].x - t.x, y[q].y - t.y);
        }
        __syncwarp();
    }
}

// w += sum_{c < *ncols} V[:, c] y[c]
__global__ void k_multi_axpy_dyn(const double2* __restrict__ V, long long ldv, const int* __restrict__ ncols,
                                 const double2* __restrict__ y, long long n, double2* __restrict__ w) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nc = *ncols;
    double2 acc = make_double2(0.0, 0.0);
    for (int c = 0; c < nc; ++c) {
        const double2 v = V[(long long)c * ldv + i], a = y[c];
        acc.x = fma(v.x, a.x, fma(-v.y, a.y, acc.x));
        acc.y = fma(v.x, a.y, fma(v.y, a.x, acc.y));
    }
    double2 o = w[i];
    w[i] = make_double2(o.x + acc.x, o.y + acc.y);
}

// ---- B right-hand sides in lock step: state of right-hand side r at R + r * ldh * m,
// g + r * (m + 1), gc / gs + r * m, st + 4 r, sc + 3 r
__global__ void k_lsq_init_batch(LsqBatchDev L, const double2* __restrict__ beta, const double* __restrict__ par) {
    const int r = blockIdx.x;
    if (r >= L.B) return;
    // par per right-hand side: r0n, tol, limit (iterations allowed this cycle; <= 0: frozen)
    const double r0n = par[3 * r], tol = par[3 * r + 1];
    const int limit = (int)par[3 * r + 2];
    double2* g = L.g + (long long)r * (L.m + 1);
    for (int i = threadIdx.x; i <= L.m; i += blockDim.x) g[i] = make_double2(i == 0 ? beta[r].x : 0.0, 0.0);
    if (threadIdx.x == 0) {
        int* st = L.st + 4 * r;
        st[0] = limit <= 0 ? 1 : 0; st[1] = 0; st[2] = limit; st[3] = 0;
        double* sc = L.sc + 3 * r;
        sc[0] = limit <= 0 ? 0.0 : 1.0; sc[1] = r0n; sc[2] = tol;
    }
}

// column j of every active right-hand side; Hcol is the interleaved column, entry (i, r) at
// Hcol[i * B + r].  active[j] receives the number of right-hand sides still running.
__global__ void k_lsq_givens_batch(const double2* __restrict__ Hcol, int j, LsqBatchDev L, int* __restrict__ active) {
    const int r = threadIdx.x;
    bool run = false;
    if (r < L.B && j < L.m) {
        int* st = L.st + 4 * r;
        if (!st[0]) {
            double* sc = L.sc + 3 * r;
            const int ldh = L.m + 1;
            double hn = 0.0;
            const double est = givens_column(Hcol + r, L.B, j, L.R + (long long)r * ldh * L.m + (long long)j * ldh,
                                             L.gc + (long long)r * L.m, L.gs + (long long)r * L.m, L.g + (long long)r * (L.m + 1),
                                             sc[1], hn);
            const int it = st[3] + 1;
            st[3] = it;
            sc[0] = est;
            st[1] = j + 1;
            if (!(est >= sc[2]) || it >= st[2] || hn == 0.0) st[0] = 1;
            else run = true;
        }
    }
    const int n = __syncthreads_count(run);
    if (threadIdx.x == 0) active[j] = n;
}

// Y[i * B + r] = (R_r^{-1} g_r)_i for i < st[4 r + 1], 0 up to ncols: one warp per right-hand side
__global__ void k_lsq_solve_batch(LsqBatchDev L, int ncols, double2* __restrict__ Y) {
    const int r = blockIdx.x, lane = threadIdx.x;
    if (r >= L.B) return;
    const int ldh = L.m + 1, B = L.B;
    const int k = L.st[4 * r + 1];
    const double2* R = L.R + (long long)r * ldh * L.m;
    const double2* g = L.g + (long long)r * (L.m + 1);
    for (int q = lane; q < ncols; q += 32) Y[(long long)q * B + r] = q < k ? g[q] : make_double2(0.0, 0.0);
    __syncwarp();
    for (int i = k - 1; i >= 0; --i) {
        const double2* Ri = R + (long long)i * ldh;
        double2 yi = make_double2(0.0, 0.0);
        if (lane == 0) {
            yi = c_div(Y[(long long)i * B + r], Ri[i]);
            Y[(long long)i * B + r] = yi;
        }
        yi.x = __shfl_sync(0xffffffffu, yi.x, 0);
        yi.y = __shfl_sync(0xffffffffu, yi.y, 0);
        for (int q = lane; q < i; q += 32) {
            const double2 t = c_mul(Ri[q], yi);
            const double2 o = Y[(long long)q * B + r];
            Y[(long long)q * B + r] = make_double2(o.x - t.x, o.y - t.y);
        }
        __syncwarp();
    }
}

// column j = *jp of every running right-hand side (Hcol = H + j * (m + 1) * B), for a captured
// iteration graph: as k_lsq_givens_batch, then j += 1 and the while-loop condition (0 once no
// right-hand side runs or the cycle is full)
__global__ void k_lsq_givens_batch_dev(const double2* __restrict__ H, int* __restrict__ jp, LsqBatchDev L,
                                       int* __restrict__ active, cudaGraphConditionalHandle cond) {
    const int r = threadIdx.x;
    const int j = *jp;
    bool run = false;
    if (r < L.B && j < L.m) {
        int* st = L.st + 4 * r;
        if (!st[0]) {
            double* sc = L.sc + 3 * r;
            const int ldh = L.m + 1;
            double hn = 0.0;
            const double2* Hcol = H + (long long)j * ldh * L.B;
            const double est = givens_column(Hcol + r, L.B, j, L.R + (long long)r * ldh * L.m + (long long)j * ldh,
                                             L.gc + (long long)r * L.m, L.gs + (long long)r * L.m, L.g + (long long)r * (L.m + 1),
                                             sc[1], hn);
            const int it = st[3] + 1;
            st[3] = it;
            sc[0] = est;
            st[1] = j + 1;
            if (!(est >= sc[2]) || it >= st[2] || hn == 0.0) st[0] = 1;
            else run = true;
        }
    }
    const int n = __syncthreads_count(run);
    if (threadIdx.x == 0) {
        if (j < L.m) active[j] = n;
        *jp = j + 1;
        cudaGraphSetConditional(cond, (n > 0 && j + 1 < L.m) ? 1u : 0u);
    }
}

// ---- segmented vectors: B segments (one per obstacle of a group) side by side in one vector;
// chunk c covers [chunk_lo[c], chunk_lo[c + 1]) inside one segment, segment s owns chunks
// [seg_chunk[s], seg_chunk[s + 1])
constexpr int kSegThreads = 256;
// part[col * nchunk + c] = V[:, col]^H w over chunk c, for col <= *jp (jp NULL: col 0 only, V = v)
__global__ void __launch_bounds__(kSegThreads) k_seg_dot_part(const double2* __restrict__ V, long long ldv, const int* __restrict__ jp,
                                                              const double2* __restrict__ w, const long long* __restrict__ chunk_lo,
                                                              int nchunk, double2* __restrict__ part) {
    const int c = blockIdx.x, col = blockIdx.y;
    if (jp ? col > *jp : col > 0) return;
    const double2* v = V + (long long)col * ldv;
    double re = 0.0, im = 0.0;
    for (long long i = chunk_lo[c] + threadIdx.x; i < chunk_lo[c + 1]; i += kSegThreads) {
        const double2 a = v[i], b = w[i];
        re = fma(a.x, b.x, fma(a.y, b.y, re));
        im = fma(a.x, b.y, fma(-a.y, b.x, im));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { re += __shfl_xor_sync(0xffffffffu, re, o); im += __shfl_xor_sync(0xffffffffu, im, o); }
    __shared__ double sr[kSegThreads / 32], si[kSegThreads / 32];
    if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = re; si[threadIdx.x >> 5] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < kSegThreads / 32; ++q) { a += sr[q]; b += si[q]; }
        part[(long long)col * nchunk + c] = make_double2(a, b);
    }
}
// per (column, segment): the segment's chunks summed in order.  mode 0: hh[col * B + s] and the
// Hessenberg column j (add: accumulate, for a second Gram-Schmidt pass); mode 1 (norms, col 0):
// nrm[s] = (sqrt(sum), 0), and with H also the subdiagonal entry H[j][j+1] of segment s
__global__ void k_seg_dot_fin(const double2* __restrict__ part, int nchunk, const int* __restrict__ seg_chunk, int B,
                              const int* __restrict__ jp, int ncol, int mode, int add, double2* __restrict__ hh,
                              double2* __restrict__ H, int ldh) {
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)ncol * B) return;
    const int col = (int)(id / B), s = (int)(id - (long long)col * B);
    const int j = jp ? *jp : 0;
    if (mode == 0 && col > j) return;
    double a = 0.0, b = 0.0;
    for (int c = seg_chunk[s]; c < seg_chunk[s + 1]; ++c) { const double2 v = part[(long long)col * nchunk + c]; a += v.x; b += v.y; }
    if (mode == 0) {
        hh[(long long)col * B + s] = make_double2(a, b);
        double2* e = H + (long long)j * ldh * B + (long long)col * B + s;
        if (add) { e->x += a; e->y += b; } else *e = make_double2(a, b);
    } else {
        const double nv = sqrt(fmax(a, 0.0));
        hh[s] = make_double2(nv, 0.0);
        if (H) H[(long long)j * ldh * B + (long long)(j + 1) * B + s] = make_double2(nv, 0.0);
    }
}
// w[i] -= sum_{c <= *jp} V[:, c][i] hh[c * B + seg(i)]
__global__ void k_seg_update(const double2* __restrict__ V, long long ldv, const int* __restrict__ jp,
                             const double2* __restrict__ hh, int B, const int* __restrict__ seg_of, long long n,
                             double2* __restrict__ w) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = *jp, s = seg_of[i];
    double2 acc = make_double2(0.0, 0.0);
    for (int c = 0; c <= j; ++c) {
        const double2 v = V[(long long)c * ldv + i], h = hh[(long long)c * B + s];
        acc.x = fma(v.x, h.x, fma(-v.y, h.y, acc.x));
        acc.y = fma(v.x, h.y, fma(v.y, h.x, acc.y));
    }
    const double2 o = w[i];
    w[i] = make_double2(o.x - acc.x, o.y - acc.y);
}
// V[:, col][i] = w[i] / nrm[seg(i)] (0 for a zero norm); col = *jp + 1, or 0 without jp
__global__ void k_seg_scale(const double2* __restrict__ w, const double2* __restrict__ nrm, const int* __restrict__ seg_of,
                            const int* __restrict__ jp, long long n, double2* __restrict__ V) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int col = jp ? *jp + 1 : 0;
    const double h = nrm[seg_of[i]].x;
    const double a = h != 0.0 ? 1.0 / h : 0.0;
    V[(long long)col * n + i] = make_double2(w[i].x * a, w[i].y * a);
}
// x[i] += sum_{c < ncols} V[:, c][i] Y[c * B + seg(i)]
__global__ void k_seg_axpy(const double2* __restrict__ V, long long ldv, int ncols, const double2* __restrict__ Y, int B,
                           const int* __restrict__ seg_of, long long n, double2* __restrict__ x) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = seg_of[i];
    double2 acc = make_double2(0.0, 0.0);
    for (int c = 0; c < ncols; ++c) {
        const double2 v = V[(long long)c * ldv + i], y = Y[(long long)c * B + s];
        acc.x = fma(v.x, y.x, fma(-v.y, y.y, acc.x));
        acc.y = fma(v.x, y.y, fma(v.y, y.x, acc.y));
    }
    const double2 o = x[i];
    x[i] = make_double2(o.x + acc.x, o.y + acc.y);
}

inline unsigned nblocks(long long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

void launch_lsq_init(LsqDev L, int* jp, double beta, double r0n, double tol, int limit, cudaStream_t s) {
    k_lsq_init<<<1, 128, 0, s>>>(L, jp, beta, r0n, tol, limit);
}
void launch_lsq_givens(const double2* H, int ldh, int* jp, LsqDev L, cudaGraphConditionalHandle cond, bool use_cond,
                       cudaStream_t s) {
    k_lsq_givens<<<1, 32, 0, s>>>(H, ldh, jp, L, cond, use_cond ? 1 : 0);
}
void launch_lsq_solve(LsqDev L, int ldh, double2* y, cudaStream_t s) { k_lsq_solve<<<1, 32, 0, s>>>(L, ldh, y); }
void launch_multi_axpy_dyn(const double2* V, long long ldv, const int* ncols, const double2* y, long long n, double2* w,
                           cudaStream_t s) {
    k_multi_axpy_dyn<<<nblocks(n, 256), 256, 0, s>>>(V, ldv, ncols, y, n, w);
}
void launch_lsq_init_batch(LsqBatchDev L, const double2* beta, const double* par, cudaStream_t s) {
    k_lsq_init_batch<<<L.B, 128, 0, s>>>(L, beta, par);
}
void launch_lsq_givens_batch(const double2* Hcol, int j, LsqBatchDev L, int* active, cudaStream_t s) {
    k_lsq_givens_batch<<<1, ((L.B + 31) / 32) * 32, 0, s>>>(Hcol, j, L, active);
}
void launch_lsq_solve_batch(LsqBatchDev L, int ncols, double2* Y, cudaStream_t s) {
    k_lsq_solve_batch<<<L.B, 32, 0, s>>>(L, ncols, Y);
}
void launch_lsq_givens_batch_dev(const double2* H, int* jp, LsqBatchDev L, int* active, cudaGraphConditionalHandle cond,
                                 cudaStream_t s) {
    k_lsq_givens_batch_dev<<<1, ((L.B + 31) / 32) * 32, 0, s>>>(H, jp, L, active, cond);
}
void launch_seg_arnoldi(const SegDesc& S, double2* V, int m, int* jp, double2* w, double2* hh, double2* H, double2* nrm,
                        int passes, cudaStream_t s) {
    const int ldh = m + 1;
    for (int pass = 0; pass < passes; ++pass) {
        k_seg_dot_part<<<dim3(S.nchunk, m + 1), kSegThreads, 0, s>>>(V, S.n, jp, w, S.chunk_lo, S.nchunk, S.part);
        k_seg_dot_fin<<<nblocks((long long)(m + 1) * S.B, 128), 128, 0, s>>>(S.part, S.nchunk, S.seg_chunk, S.B, jp, m + 1, 0, pass,
                                                                              hh, H, ldh);
        k_seg_update<<<nblocks(S.n, 256), 256, 0, s>>>(V, S.n, jp, hh, S.B, S.seg_of, S.n, w);
    }
    k_seg_dot_part<<<dim3(S.nchunk, 1), kSegThreads, 0, s>>>(w, 0, nullptr, w, S.chunk_lo, S.nchunk, S.part);
    k_seg_dot_fin<<<nblocks(S.B, 128), 128, 0, s>>>(S.part, S.nchunk, S.seg_chunk, S.B, jp, 1, 1, 0, nrm, H, ldh);
    k_seg_scale<<<nblocks(S.n, 256), 256, 0, s>>>(w, nrm, S.seg_of, jp, S.n, V);
}
void launch_seg_norms(const SegDesc& S, const double2* v, double2* nrm, cudaStream_t s) {
    k_seg_dot_part<<<dim3(S.nchunk, 1), kSegThreads, 0, s>>>(v, 0, nullptr, v, S.chunk_lo, S.nchunk, S.part);
    k_seg_dot_fin<<<nblocks(S.B, 128), 128, 0, s>>>(S.part, S.nchunk, S.seg_chunk, S.B, nullptr, 1, 1, 0, nrm, nullptr, 0);
}
void launch_seg_scale0(const SegDesc& S, const double2* w, const double2* nrm, double2* V, cudaStream_t s) {
    k_seg_scale<<<nblocks(S.n, 256), 256, 0, s>>>(w, nrm, S.seg_of, nullptr, S.n, V);
}
void launch_seg_axpy(const SegDesc& S, const double2* V, int ncols, const double2* Y, double2* x, cudaStream_t s) {
    if (ncols <= 0) return;
    k_seg_axpy<<<nblocks(S.n, 256), 256, 0, s>>>(V, S.n, ncols, Y, S.B, S.seg_of, S.n, x);
}

}  // namespace ifgf
