// ifgf_batch.cu -- the IFGF forward map applied to a batch of right-hand sides at once.
//
// Every table of the single-vector apply (near-field Green values, leaf-cone values,
// propagation and interpolation plans) depends on the geometry and k only, so B right-hand
// sides (plane waves of different incidence, ForwardMap::solve called B times) can share one
// pass over them.  The batch lives interleaved, [N][B] with the RHS index fastest, and one warp
// serves 32 right-hand sides: table entries become warp-uniform broadcast loads and the
// density / coefficient accesses are 256-byte coalesced rows.
//
//   k_sing_b   singular correction + jump term + intensities     ForwardMap.tpp:425-435, 481-515
//              (FP32 weights in the mixed form)
//   k_leaf_b   leaf cone coefficients, table rows staged in shared
//              memory by cp.async, 25 accumulators per RHS          BoxTree.h:685-762
//   k_prop_b   child -> parent, per parent cone one warp; the
//              parent's terms sorted by child cone so each child
//              cone's coefficients are loaded once                 BoxTree.h:767-868, Interpolator.h:81-120
//   k_final_b  near field + cousin interpolation per target       BoxTree.h:614-683, 876-937
//
// plus the batched GMRES vector kernels (per-RHS dot products, CGS updates, scaling).
#include "ifgf_device.cuh"
#include "tcgen05.cuh"

namespace ifgf {

static inline unsigned nblk_b(long long n, int b) { return (unsigned)((n + b - 1) / b); }

// ------------------------------------------------------------------ layout changes
__global__ void k_interleave(const double2* __restrict__ x, long long N, int B, double2* __restrict__ xt) {
    __shared__ double2 t[32][33];
    const long long i0 = (long long)blockIdx.x * 32;
    const int r0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int r = r0 + k;
        const long long i = i0 + threadIdx.x;
        if (r < B && i < N) t[k][threadIdx.x] = x[(long long)r * N + i];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        const long long i = i0 + k;
        const int r = r0 + threadIdx.x;
        if (r < B && i < N) xt[i * B + r] = t[threadIdx.x][k];
    }
}
__global__ void k_deinterleave(const double2* __restrict__ xt, long long N, int B, double2* __restrict__ x) {
    __shared__ double2 t[32][33];
    const long long i0 = (long long)blockIdx.x * 32;
    const int r0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const long long i = i0 + k;
        const int r = r0 + threadIdx.x;
        if (r < B && i < N) t[k][threadIdx.x] = xt[i * B + r];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int r = r0 + k;
        const long long i = i0 + threadIdx.x;
        if (r < B && i < N) x[(long long)r * N + i] = t[threadIdx.x][k];
    }
}

// ------------------------------------------------------------------ singular correction
// warp = one output row, lane = one right-hand side.  WT = double2: FP64 weights, densities and
// arithmetic (the plain form; xw = xt); WT = float2: complex64 copies of the FP64-computed
// weights and of the densities (xw), FP32 sums (the mixed form).  The jump term and the
// intensities take the FP64 densities xt.
template <typename WT, typename RhoT>
__global__ void __launch_bounds__(256) k_sing_b(const double2* __restrict__ xt, const WT* __restrict__ xw,
                                                const WT* __restrict__ W, const int* __restrict__ row_ptr,
                                                const int* __restrict__ row_col, const RPColumn* __restrict__ cols, int N,
                                                int Np, int B, double half, double2* __restrict__ yt,
                                                const double* __restrict__ wq, const long long* __restrict__ inv,
                                                RhoT* __restrict__ rho) {
    using A = decltype(WT{}.x);
    const int o = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int r = blockIdx.y * 32 + (threadIdx.x & 31);
    if (o >= N || r >= B) return;
    A ax = A(0), ay = A(0);
    for (int q = row_ptr[o]; q < row_ptr[o + 1]; ++q) {
        const int col = row_col[q];
        const WT* w = W + (long long)col * Np;
        const WT* d = xw + (long long)cols[col].patch * Np * B + r;
        int kk = 0;
        for (; kk + 4 <= Np; kk += 4) {         // four nodes' loads in flight at once
            WT a[4], bw[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { a[u] = d[(long long)(kk + u) * B]; bw[u] = w[kk + u]; }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                ax = fma(a[u].x, bw[u].x, fma(-a[u].y, bw[u].y, ax));
                ay = fma(a[u].x, bw[u].y, fma(a[u].y, bw[u].x, ay));
            }
        }
        for (; kk < Np; ++kk) {
            const WT a = d[(long long)kk * B], b = w[kk];
            ax = fma(a.x, b.x, fma(-a.y, b.y, ax));
            ay = fma(a.x, b.y, fma(a.y, b.x, ay));
        }
    }
    const double2 v = xt[(long long)o * B + r];
    double2 acc = make_double2((double)ax, (double)ay);
    if (half != 0.0) { acc.x += half * v.x; acc.y += half * v.y; }   // jump term
    yt[(long long)o * B + r] = acc;
    if (rho) {
        const double wv = wq[o];
        RhoT q; q.x = v.x * wv; q.y = v.y * wv;
        rho[inv[o] * B + r] = q;
    }
}

// ------------------------------------------------------------------ asynchronous copies
// cp.async (global -> shared without a register round trip) of one 8- or 16-byte element
template <int BYTES>
__device__ __forceinline__ void cp_async_el(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory"); }

// right-hand sides per lane: two for the complex64 form (a warp covers a 64-wide batch, so
// every table entry is read once per batch), one for FP64 (register budget)
template <typename R> struct Rpl { static constexpr int v = sizeof(R) == 4 ? 2 : 1; };

// ------------------------------------------------------------------ leaf cones
// warp = one leaf cone x 32*RPL right-hand sides, P accumulators per (lane, RHS).  The cone's
// table rows stream through shared memory in tiles of TS sources (cp.async, double-buffered)
// and every lane reads them as broadcasts; densities are prefetched one source ahead.
constexpr int kLeafWarps = 4;
template <typename R, int P, int RPL>
__global__ void __launch_bounds__(kLeafWarps * 32) k_leaf_b(const int* __restrict__ cone_box, int ncones, int cone_base,
                                                            const int* __restrict__ leaf_start,
                                                            const int* __restrict__ leaf_count,
                                                            const long long* __restrict__ leaf_off,
                                                            const V2<R>* __restrict__ L, const V2<R>* __restrict__ rho, int B,
                                                            V2<R>* __restrict__ coef) {
    constexpr int TS = sizeof(R) == 4 ? 16 : 8;
    __shared__ V2<R> tile[kLeafWarps][2][TS * P];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * kLeafWarps + w;
    if (c >= ncones) return;                 // warps are independent: no block-wide barrier below
    int rr[RPL];
    bool act[RPL];
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
        const int r = blockIdx.y * 32 * RPL + 32 * k + lane;
        act[k] = r < B;
        rr[k] = act[k] ? r : 0;
    }
    const int b = cone_box[c];
    const int n = leaf_count[b], s0 = leaf_start[b];
    const V2<R>* Lc = L + leaf_off[c];
    auto load_tile = [&](int t) {
        const int sb = t * TS;
        const int cnt = (n - sb < TS ? n - sb : TS) * P;
        const V2<R>* src = Lc + (long long)sb * P;
        V2<R>* dst = tile[w][t & 1];
        for (int q = lane; q < cnt; q += 32) cp_async_el<(int)sizeof(V2<R>)>(dst + q, src + q);
        cp_async_commit();
    };
    V2<R> acc[RPL][P];
#pragma unroll
    for (int k = 0; k < RPL; ++k)
#pragma unroll
        for (int m = 0; m < P; ++m) { acc[k][m].x = R(0); acc[k][m].y = R(0); }
    const V2<R>* rh = rho + (long long)s0 * B;
    V2<R> vn[RPL];
#pragma unroll
    for (int k = 0; k < RPL; ++k) vn[k] = rh[rr[k]];
    const int nt = (n + TS - 1) / TS;
    load_tile(0);
    for (int t = 0; t < nt; ++t) {
        if (t + 1 < nt) { load_tile(t + 1); cp_async_wait<1>(); }
        else cp_async_wait<0>();
        __syncwarp();
        const V2<R>* Lt = tile[w][t & 1];
        const int sb = t * TS;
        const int cnt = n - sb < TS ? n - sb : TS;
        for (int s = 0; s < cnt; ++s) {
            V2<R> v[RPL];
#pragma unroll
            for (int k = 0; k < RPL; ++k) v[k] = vn[k];
            if (sb + s + 1 < n) {
#pragma unroll
                for (int k = 0; k < RPL; ++k) vn[k] = rh[(long long)(sb + s + 1) * B + rr[k]];
            }
#pragma unroll
            for (int m = 0; m < P; ++m) {
                const V2<R> l = Lt[s * P + m];
#pragma unroll
                for (int k = 0; k < RPL; ++k) cmac<R>(acc[k][m], l, v[k]);
            }
        }
        __syncwarp();                        // the buffer is refilled two tiles later
    }
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
        if (!act[k]) continue;
        V2<R>* out = coef + (long long)(cone_base + c) * P * B + rr[k];
#pragma unroll
        for (int m = 0; m < P; ++m) out[(long long)m * B] = acc[k][m];
    }
}

// ------------------------------------------------------------------ propagation
// warp = one parent cone x 32*RPL right-hand sides.  Node values accumulate in the lane's own
// shared-memory columns; the values -> coefficients map then runs in the lane's registers.
template <typename R, int P, int RPL>
struct PropBlock {
    static constexpr int bytes_per_warp = P * 32 * RPL * (int)sizeof(V2<R>);
    static constexpr int W = 32768 / bytes_per_warp >= 4 ? 4 : (32768 / bytes_per_warp >= 2 ? 2 : 1);
};
template <typename R, int PS, int PA, int WPB, int RPL, bool ROWS = false>
__global__ void __launch_bounds__(WPB * 32) k_prop_b(int pbegin, int pend, const long long* __restrict__ pp_ptr,
                                                     const int* __restrict__ pp_nchild, const PropB<R>* __restrict__ pb,
                                                     const R* __restrict__ Gsep, int B, V2<R>* __restrict__ coef,
                                                     const R* __restrict__ rows = nullptr) {
    constexpr int P = PS * PA;
    __shared__ V2<R> sv[WPB][P][32 * RPL];
    __shared__ R sG[PS * PS + PA * PA];
    for (int i = threadIdx.x; i < PS * PS + PA * PA; i += blockDim.x) sG[i] = Gsep[i];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pc = pbegin + blockIdx.x * WPB + w;
    if (pc >= pend) return;
    int rr[RPL];
    bool act[RPL];
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
        const int r = blockIdx.y * 32 * RPL + 32 * k + lane;
        act[k] = r < B;
        rr[k] = act[k] ? r : 0;
    }
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
        for (int k = 0; k < RPL; ++k) { sv[w][q][32 * k + lane].x = R(0); sv[w][q][32 * k + lane].y = R(0); }
    const long long e0 = pp_ptr[pc];
    const int ne = pp_nchild[pc] * P;
    V2<R> cc[RPL][P];
    int cur = -1;
    PropB<R> En{};
    if (ne > 0) En = pb[e0];
    for (int e = 0; e < ne; ++e) {
        const PropB<R> E = En;
        if (e + 1 < ne) En = pb[e0 + e + 1];   // next term in flight during this one
        if (E.child_cone != cur) {             // warp-uniform: E is the same for every lane
            cur = E.child_cone;
            const V2<R>* src = coef + (long long)cur * P * B;
#pragma unroll
            for (int k = 0; k < RPL; ++k)
#pragma unroll
                for (int q = 0; q < P; ++q) cc[k][q] = src[(long long)q * B + rr[k]];
        }
        R Ts[PS], Tt[PA];
        if constexpr (ROWS) {   // the same rows, computed once per term by k_plan_rows
            const R* rw = rows + (e0 + e) * (PS + PA);
#pragma unroll
            for (int q = 0; q < PS; ++q) Ts[q] = rw[q];
#pragma unroll
            for (int q = 0; q < PA; ++q) Tt[q] = rw[PS + q];
        } else {
            cheb_row<R, PS>(E.s, Ts);
            cheb_row<R, PA>(E.th, Tt);
        }
        V2<R> wv; wv.x = E.wr; wv.y = E.wi;
#pragma unroll
        for (int k = 0; k < RPL; ++k) {
            const V2<R> it = interp_eval_tt<R, PS, PA>(cc[k], Ts, Tt);
            V2<R> a = sv[w][E.pt][32 * k + lane];
            cmac<R>(a, it, wv);
            sv[w][E.pt][32 * k + lane] = a;
        }
    }
    // u[l][m] = sum_k Gs[m][k] v[l][k];  c[n][m] = sum_l Ga[n][l] u[l][m], stored at n*PS + m
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
        V2<R> u[P];
#pragma unroll
        for (int l = 0; l < PA; ++l) {
            V2<R> v[PS];
#pragma unroll
            for (int q = 0; q < PS; ++q) v[q] = sv[w][l * PS + q][32 * k + lane];
#pragma unroll
            for (int m = 0; m < PS; ++m) {
                V2<R> a; a.x = R(0); a.y = R(0);
#pragma unroll
                for (int q = 0; q < PS; ++q) { const R g = sG[m * PS + q]; a.x = rfma(g, v[q].x, a.x); a.y = rfma(g, v[q].y, a.y); }
                u[l * PS + m] = a;
            }
        }
        if (!act[k]) continue;
        V2<R>* out = coef + (long long)pc * P * B + rr[k];
#pragma unroll
        for (int n = 0; n < PA; ++n)
#pragma unroll
            for (int m = 0; m < PS; ++m) {
                V2<R> a; a.x = R(0); a.y = R(0);
#pragma unroll
                for (int l = 0; l < PA; ++l) {
                    const R g = sG[PS * PS + n * PA + l];
                    a.x = rfma(g, u[l * PS + m].x, a.x); a.y = rfma(g, u[l * PS + m].y, a.y);
                }
                out[(long long)(n * PS + m) * B] = a;
            }
    }
}

// the Chebyshev rows T_q(s), T_a(th) of every batched plan term, [term][PS + PA]: the propagation
// reads them once per warp instead of computing them in every lane (they are the same for all
// the warp's right-hand sides), with the same cheb_row arithmetic
template <typename R, int PS, int PA>
__global__ void k_plan_rows(const PropB<R>* __restrict__ pb, long long n, R* __restrict__ rows) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const PropB<R> E = pb[e];
    R Ts[PS], Tt[PA];
    cheb_row<R, PS>(E.s, Ts);
    cheb_row<R, PA>(E.th, Tt);
    R* rw = rows + e * (PS + PA);
#pragma unroll
    for (int q = 0; q < PS; ++q) rw[q] = Ts[q];
#pragma unroll
    for (int q = 0; q < PA; ++q) rw[PS + q] = Tt[q];
}

// ------------------------------------------------------------------ propagation, TMA-staged
// k_prop_b (complex64) with its loads taken off the FMA loop: the parent's terms are staged in
// shared memory at the start, and the child cones' coefficient blocks by the tensor memory
// accelerator.  When the block starts a group of terms, thread 0 issues a bulk copy
// (cp.async.bulk, completion counted on an mbarrier) of the NEXT group's 25 x B block into
// shared memory, so it has landed by the time the FMA loop needs it.  Two warps share one parent
// cone and one staging buffer, 32 right-hand sides each (half the shared memory per warp of a
// warp per cone, twice the resident warps).  B must be even (the block is a multiple of 16
// bytes).  Waits are bounded; one that runs out sets *err and the block stops.
constexpr int kPropBkWarps = 2;
template <int PS, int PA>
__global__ void __launch_bounds__(32 * kPropBkWarps) k_prop_bk(int pbegin, int pend, const long long* __restrict__ pp_ptr,
                                                               const int* __restrict__ pp_nchild, const PropB<float>* __restrict__ pb,
                                                               const float* __restrict__ Gsep, int B, float2* __restrict__ coef,
                                                               int* __restrict__ err) {
    constexpr int P = PS * PA;
    __shared__ __align__(128) float2 buf[P * 32 * kPropBkWarps];
    __shared__ float2 sv[P][32 * kPropBkWarps];
    __shared__ float sG[PS * PS + PA * PA];
    __shared__ PropB<float> st[4 * P];
    __shared__ __align__(8) unsigned long long mbar;
    const int tid = threadIdx.x, lane = tid & 31;
    const int pc = pbegin + blockIdx.x;
    if (pc >= pend) return;
    for (int i = tid; i < PS * PS + PA * PA; i += blockDim.x) sG[i] = Gsep[i];
    const uint32_t bar = tc5::smem_u32(&mbar), sbuf = tc5::smem_u32(buf);
    const int r = tid;                        // this thread's right-hand side
    const bool act = r < B;
    const int rr = act ? r : 0;
#pragma unroll
    for (int q = 0; q < P; ++q) sv[q][tid] = make_float2(0.f, 0.f);
    const long long e0 = pp_ptr[pc];
    const int ne = pp_nchild[pc] * P;   // at most four children
    const uint32_t bytes = (uint32_t)(P * B * sizeof(float2));
    if (tid == 0) {
        tc5::mbar_init(bar, 1);
        if (ne > 0) tc5::bulk_g2s(sbuf, coef + (long long)pb[e0].child_cone * P * B, bytes, bar);
    }
    for (int i = tid; i < ne; i += blockDim.x) st[i] = pb[e0 + i];   // the parent's terms
    __syncthreads();
    uint32_t phase = 0;
    bool ok = true;
    float2 cc[P];
    int cur = -1;
    for (int e = 0; e < ne; ++e) {
        const PropB<float> E = st[e];
        if (E.child_cone != cur) {             // block-uniform
            cur = E.child_cone;
            ok = __syncthreads_and(tc5::mbar_wait(bar, phase & 1u, 2000000000ll));
            ++phase;
            if (!ok) break;
#pragma unroll
            for (int q = 0; q < P; ++q) cc[q] = buf[q * B + rr];
            __syncthreads();                   // every thread has read the block before it is overwritten
            if (tid < 32) {                    // the next group: the first later term with another child cone
                int nxt = -1;
                for (int base = e + 1; base < ne && nxt < 0; base += 32) {
                    const int idx = base + lane;
                    const int cn = idx < ne ? st[idx].child_cone : cur;
                    const unsigned m = __ballot_sync(0xffffffffu, cn != cur);
                    if (m) nxt = __shfl_sync(0xffffffffu, cn, __ffs(m) - 1);
                }
                if (nxt >= 0 && tid == 0) tc5::bulk_g2s(sbuf, coef + (long long)nxt * P * B, bytes, bar);
            }
        }
        float Ts[PS], Tt[PA];
        cheb_row<float, PS>(E.s, Ts);
        cheb_row<float, PA>(E.th, Tt);
        const float2 it = interp_eval_tt<float, PS, PA>(cc, Ts, Tt);
        float2 a = sv[E.pt][tid];
        cmac<float>(a, it, make_float2(E.wr, E.wi));
        sv[E.pt][tid] = a;
    }
    if (!ok) {   // the copy of the group that timed out may still land: one more bounded wait
        if (tid == 0) { atomicExch(err, 1); tc5::mbar_wait(bar, (phase - 1u) & 1u, 2000000000ll); }
        return;
    }
    // u[l][m] = sum_k Gs[m][k] v[l][k];  c[n][m] = sum_l Ga[n][l] u[l][m], stored at n*PS + m
    float2 u[P];
#pragma unroll
    for (int l = 0; l < PA; ++l) {
        float2 v[PS];
#pragma unroll
        for (int q = 0; q < PS; ++q) v[q] = sv[l * PS + q][tid];
#pragma unroll
        for (int m = 0; m < PS; ++m) {
            float2 a = make_float2(0.f, 0.f);
#pragma unroll
            for (int q = 0; q < PS; ++q) { const float g = sG[m * PS + q]; a.x = fmaf(g, v[q].x, a.x); a.y = fmaf(g, v[q].y, a.y); }
            u[l * PS + m] = a;
        }
    }
    if (!act) return;
    float2* out = coef + (long long)pc * P * B + r;
#pragma unroll
    for (int n = 0; n < PA; ++n)
#pragma unroll
        for (int m = 0; m < PS; ++m) {
            float2 a = make_float2(0.f, 0.f);
#pragma unroll
            for (int l = 0; l < PA; ++l) {
                const float g = sG[PS * PS + n * PA + l];
                a.x = fmaf(g, u[l * PS + m].x, a.x); a.y = fmaf(g, u[l * PS + m].y, a.y);
            }
            out[(long long)(n * PS + m) * B] = a;
        }
}

// ------------------------------------------------------------------ near field + interpolation
// warp = one Morton-sorted target x 32*RPL right-hand sides; y accumulated at the original index
template <typename R, int PS, int PA, int RPL>
__global__ void __launch_bounds__(256) k_final_b(int N, const int* __restrict__ point_leaf, const int* __restrict__ leaf_start,
                                                 const int* __restrict__ leaf_count, const int* __restrict__ nbr_ptr,
                                                 const int* __restrict__ nbr_box, const int* __restrict__ near_rowlen,
                                                 const long long* __restrict__ near_off, const V2<R>* __restrict__ near,
                                                 const V2<R>* __restrict__ rho, const int* __restrict__ ip_ptr,
                                                 const InterpE<R>* __restrict__ ip, const V2<R>* __restrict__ coef,
                                                 const long long* __restrict__ sorting, int B, double2* __restrict__ yt) {
    constexpr int P = PS * PA;
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= N) return;
    int rr[RPL];
    bool act[RPL];
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
        const int r = blockIdx.y * 32 * RPL + 32 * k + lane;
        act[k] = r < B;
        rr[k] = act[k] ? r : 0;
    }
    const int b = point_leaf[i];
    const int t = i - leaf_start[b];
    const V2<R>* row = near + near_off[b] + (long long)t * near_rowlen[b];
    V2<R> acc[RPL];
#pragma unroll
    for (int k = 0; k < RPL; ++k) { acc[k].x = R(0); acc[k].y = R(0); }
    int sg = 0;
    for (int q = nbr_ptr[b]; q < nbr_ptr[b + 1]; ++q) {
        const int bb = nbr_box[q];
        const int c = leaf_count[bb];
        const V2<R>* rh = rho + (long long)leaf_start[bb] * B;
        int s = 0;
        for (; s + 4 <= c; s += 4) {           // four sources' loads in flight at once
            V2<R> nv[4], rv[4][RPL];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                nv[u] = row[sg + s + u];
#pragma unroll
                for (int k = 0; k < RPL; ++k) rv[u][k] = rh[(long long)(s + u) * B + rr[k]];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int k = 0; k < RPL; ++k) cmac<R>(acc[k], nv[u], rv[u][k]);
        }
        for (; s < c; ++s) {
            const V2<R> nv = row[sg + s];
#pragma unroll
            for (int k = 0; k < RPL; ++k) cmac<R>(acc[k], nv, rh[(long long)s * B + rr[k]]);
        }
        sg += c;
    }
    for (int e = ip ? ip_ptr[i] : 0; ip && e < ip_ptr[i + 1]; ++e) {   // ip null: near field only
        const InterpE<R> E = ip[e];
        R Ts[PS], Tt[PA];
        cheb_row<R, PS>(E.s, Ts);
        cheb_row<R, PA>(E.th, Tt);
        V2<R> f; f.x = E.fr; f.y = E.fi;
        const V2<R>* src = coef + (long long)E.cone * P * B;
#pragma unroll
        for (int k = 0; k < RPL; ++k) {
            V2<R> cc[P];
#pragma unroll
            for (int q = 0; q < P; ++q) cc[q] = src[(long long)q * B + rr[k]];
            cmac<R>(acc[k], interp_eval_tt<R, PS, PA>(cc, Ts, Tt), f);
        }
    }
    const long long o = sorting[i];
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
        if (!act[k]) continue;
        double2* yo = yt + o * B + rr[k];
        double2 v = *yo;
        v.x += (double)acc[k].x; v.y += (double)acc[k].y;
        *yo = v;
    }
}

// ------------------------------------------------------------------ interpolation grouped by cone
// Two warps = one work item (up to kInterpGrpTargets targets of one leaf box), 32 right-hand
// sides each.  The item's terms are sorted by cone, so each cone's 25 x B coefficient block is
// loaded once for every target of the item that reads it (k_final_b loads it once per target);
// per-target sums accumulate in shared memory, then are added into yt.
template <int PS, int PA>
__global__ void __launch_bounds__(64) k_interp_grp(const int4* __restrict__ items, int nitems, const InterpG* __restrict__ terms,
                                                   const float2* __restrict__ coef, const long long* __restrict__ sorting, int B,
                                                   double2* __restrict__ yt) {
    constexpr int P = PS * PA;
    __shared__ float2 acc[kInterpGrpTargets][64];
    const int it = blockIdx.x;
    if (it >= nitems) return;
    const int4 I = items[it];   // terms [x, y), targets [z, z + w)
    const int r = threadIdx.x;  // this thread's right-hand side
    const bool act = r < B;
    const int rr = act ? r : 0;
    for (int t = 0; t < I.w; ++t) acc[t][r] = make_float2(0.f, 0.f);   // each thread its own column
    float2 cc[P];
    int cur = -1;
    InterpG En{};
    if (I.x < I.y) En = terms[I.x];
    for (int e = I.x; e < I.y; ++e) {
        const InterpG E = En;
        if (e + 1 < I.y) En = terms[e + 1];     // next term in flight during this one
        if (E.cone != cur) {                    // uniform over the block
            cur = E.cone;
            const float2* src = coef + (long long)cur * P * B;
#pragma unroll
            for (int q = 0; q < P; ++q) cc[q] = src[(long long)q * B + rr];
        }
        float Ts[PS], Tt[PA];
        cheb_row<float, PS>(E.s, Ts);
        cheb_row<float, PA>(E.th, Tt);
        float2 a = acc[E.t - I.z][r];
        cmac<float>(a, interp_eval_tt<float, PS, PA>(cc, Ts, Tt), make_float2(E.fr, E.fi));
        acc[E.t - I.z][r] = a;
    }
    if (!act) return;
    for (int t = 0; t < I.w; ++t) {
        double2* yo = yt + sorting[I.z + t] * B + r;
        const float2 a = acc[t][r];
        double2 v = *yo;
        v.x += (double)a.x; v.y += (double)a.y;
        *yo = v;
    }
}

// ------------------------------------------------------------------ batched GMRES vector kernels
constexpr int kRowsPerChunk = 512;
int bdot_chunks(long long N) { return (int)((N + kRowsPerChunk - 1) / kRowsPerChunk); }

// block (chunk, column c): partial sums of conj(V_c) w over the chunk's rows, per RHS
__global__ void __launch_bounds__(256) k_bdot_part(const double2* __restrict__ V, long long ldc, const double2* __restrict__ w,
                                                   long long N, int B, double2* __restrict__ part) {
    __shared__ double2 sm[256];
    const int c = blockIdx.y, chunk = blockIdx.x, nchunk = gridDim.x;
    const int RP = 256 / B;
    const int t = threadIdx.x, g = t / B, r = t - g * B;
    double2 acc = make_double2(0.0, 0.0);
    if (g < RP) {
        const long long i0 = (long long)chunk * kRowsPerChunk;
        const long long i1 = i0 + kRowsPerChunk < N ? i0 + kRowsPerChunk : N;
        const double2* v = V + (long long)c * ldc;
        for (long long i = i0 + g; i < i1; i += RP) {
            const double2 a = v[i * B + r], b = w[i * B + r];
            acc.x = fma(a.x, b.x, fma(a.y, b.y, acc.x));
            acc.y = fma(a.x, b.y, fma(-a.y, b.x, acc.y));
        }
    }
    sm[t] = acc;
    __syncthreads();
    if (t < B) {
        double2 s = sm[t];
        for (int q = 1; q < RP; ++q) { s.x += sm[q * B + t].x; s.y += sm[q * B + t].y; }
        part[((long long)c * nchunk + chunk) * B + t] = s;
    }
}
__global__ void k_bdot_reduce(const double2* __restrict__ part, int nchunk, int ncols, int B, double2* __restrict__ h,
                              double2* __restrict__ Hcol, int add, int sqrt_row) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncols * B) return;
    const int c = idx / B, r = idx - c * B;
    double2 s = make_double2(0.0, 0.0);
    const double2* p = part + (long long)c * nchunk * B + r;
    for (int q = 0; q < nchunk; ++q) { s.x += p[(long long)q * B].x; s.y += p[(long long)q * B].y; }
    if (sqrt_row >= 0) {
        Hcol[(long long)sqrt_row * B + r] = make_double2(sqrt(s.x > 0.0 ? s.x : 0.0), 0.0);
        return;
    }
    if (h) h[idx] = s;
    if (Hcol) {
        double2 v = s;
        if (add) { v.x += Hcol[idx].x; v.y += Hcol[idx].y; }
        Hcol[idx] = v;
    }
}
__global__ void __launch_bounds__(256) k_bupdate(const double2* __restrict__ V, long long ldc, int ncols,
                                                 const double2* __restrict__ h, double sign, long long n, int B,
                                                 double2* __restrict__ w) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const int r = (int)(e % B);
    double2 acc = make_double2(0.0, 0.0);
    for (int c = 0; c < ncols; ++c) {
        const double2 a = V[(long long)c * ldc + e], b = h[c * B + r];
        acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
        acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
    }
    double2 v = w[e];
    v.x = fma(sign, acc.x, v.x); v.y = fma(sign, acc.y, v.y);
    w[e] = v;
}
__global__ void k_bscale(const double2* __restrict__ w, const double2* __restrict__ hn, long long n, int B,
                         double2* __restrict__ out) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const double h = hn[e % B].x;
    const double s = h > 0.0 ? 1.0 / h : 0.0;
    const double2 v = w[e];
    out[e] = make_double2(v.x * s, v.y * s);
}

// columns act[0..Bc) of an interleaved [N][B] array <-> a compact [N][Bc] one
__global__ void k_gather_cols(const double2* __restrict__ in, int B, const int* __restrict__ act, int Bc, long long N,
                              double2* __restrict__ out) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N * Bc) return;
    const long long i = e / Bc;
    out[e] = in[i * B + act[e - i * Bc]];
}
__global__ void k_scatter_cols(const double2* __restrict__ in, int Bc, const int* __restrict__ act, int B, long long N, int add,
                               double2* __restrict__ out) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N * Bc) return;
    const long long i = e / Bc;
    double2& o = out[i * B + act[e - i * Bc]];
    const double2 v = in[e];
    if (add) { o.x += v.x; o.y += v.y; } else o = v;
}

// ------------------------------------------------------------------ launchers
void launch_gather_cols(const double2* in, int B, const int* act, int Bc, long long N, double2* out, cudaStream_t s) {
    if (N * Bc > 0) k_gather_cols<<<nblk_b(N * Bc, 256), 256, 0, s>>>(in, B, act, Bc, N, out);
}
void launch_scatter_cols(const double2* in, int Bc, const int* act, int B, long long N, bool add, double2* out, cudaStream_t s) {
    if (N * Bc > 0) k_scatter_cols<<<nblk_b(N * Bc, 256), 256, 0, s>>>(in, Bc, act, B, N, add ? 1 : 0, out);
}
void launch_interleave(const double2* x, long long N, int B, double2* xt, cudaStream_t s) {
    if (N <= 0 || B <= 0) return;
    k_interleave<<<dim3(nblk_b(N, 32), nblk_b(B, 32)), dim3(32, 8), 0, s>>>(x, N, B, xt);
}
void launch_deinterleave(const double2* xt, long long N, int B, double2* x, cudaStream_t s) {
    if (N <= 0 || B <= 0) return;
    k_deinterleave<<<dim3(nblk_b(N, 32), nblk_b(B, 32)), dim3(32, 8), 0, s>>>(xt, N, B, x);
}
void launch_sing_b(const double2* xt, const float2* xt32, const double2* W, const float2* W32, const int* row_ptr,
                   const int* row_col, const RPColumn* cols, int N, int Np, int B, double half, double2* yt,
                   const double* wq, const long long* inv, double2* rho64, float2* rho32, cudaStream_t s) {
    const dim3 grid(nblk_b(N, 8), nblk_b(B, 32));
    if (rho32)
        k_sing_b<float2, float2><<<grid, 256, 0, s>>>(xt, xt32, W32, row_ptr, row_col, cols, N, Np, B, half, yt, wq, inv, rho32);
    else
        k_sing_b<double2, double2><<<grid, 256, 0, s>>>(xt, xt, W, row_ptr, row_col, cols, N, Np, B, half, yt, wq, inv, rho64);
}
template <typename R>
void launch_leaf_b(const int* cone_box, int ncones, int cone_base, const int* leaf_start, const int* leaf_count,
                   const long long* leaf_off, const V2<R>* L, const V2<R>* rho, int Ps, int Pang, int B, V2<R>* coef,
                   cudaStream_t s) {
    if (ncones <= 0) return;
    constexpr int RPL = Rpl<R>::v;
    const dim3 grid(nblk_b(ncones, kLeafWarps), nblk_b(B, 32 * RPL));
    IFGF_DISPATCH_P(Ps, Pang, (k_leaf_b<R, PS * PA, RPL><<<grid, kLeafWarps * 32, 0, s>>>(
                                   cone_box, ncones, cone_base, leaf_start, leaf_count, leaf_off, L, rho, B, coef)));
}
template <typename R>
void launch_prop_b(int pbegin, int pend, const long long* pp_ptr, const int* pp_nchild, const PropB<R>* pb, int Ps, int Pang,
                   const R* Gsep, int B, V2<R>* coef, cudaStream_t s, const R* rows) {
    if (pend <= pbegin) return;
    constexpr int RPL = Rpl<R>::v;
    IFGF_DISPATCH_P(Ps, Pang, {
        constexpr int WPB = PropBlock<R, PS * PA, RPL>::W;
        const dim3 grid(nblk_b(pend - pbegin, WPB), nblk_b(B, 32 * RPL));
        if (rows)
            k_prop_b<R, PS, PA, WPB, RPL, true><<<grid, WPB * 32, 0, s>>>(pbegin, pend, pp_ptr, pp_nchild, pb, Gsep, B, coef, rows);
        else
            k_prop_b<R, PS, PA, WPB, RPL><<<grid, WPB * 32, 0, s>>>(pbegin, pend, pp_ptr, pp_nchild, pb, Gsep, B, coef);
    });
}
template <typename R>
void launch_plan_rows(const PropB<R>* pb, long long n, int Ps, int Pang, R* rows, cudaStream_t s) {
    if (n <= 0) return;
    IFGF_DISPATCH_P(Ps, Pang, (k_plan_rows<R, PS, PA><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(pb, n, rows)));
}
bool launch_interp_grp(const int4* items, int nitems, const InterpG* terms, const float2* coef, int Ps, int Pang,
                       const long long* sorting, int B, double2* yt, cudaStream_t s) {
    if (Ps != 5 || Pang != 5 || B > 64 || B <= 0) return false;
    if (nitems <= 0) return true;
    k_interp_grp<5, 5><<<nitems, 64, 0, s>>>(items, nitems, terms, coef, sorting, B, yt);
    return true;
}
bool launch_prop_bk(int pbegin, int pend, const long long* pp_ptr, const int* pp_nchild, const PropB<float>* pb, int Ps, int Pang,
                    const float* Gsep, int B, float2* coef, int* err, cudaStream_t s) {
    if (Ps != 5 || Pang != 5 || B > 64 || B <= 0 || (B & 1)) return false;
    if (pend <= pbegin) return true;
    k_prop_bk<5, 5><<<pend - pbegin, 32 * kPropBkWarps, 0, s>>>(pbegin, pend, pp_ptr, pp_nchild, pb, Gsep, B, coef, err);
    return true;
}
template <typename R>
void launch_final_b(int N, const int* point_leaf, const int* leaf_start, const int* leaf_count, const int* nbr_ptr,
                    const int* nbr_box, const int* near_rowlen, const long long* near_off, const V2<R>* near,
                    const V2<R>* rho, const int* ip_ptr, const InterpE<R>* ip, const V2<R>* coef, int Ps, int Pang,
                    const long long* sorting, int B, double2* yt, cudaStream_t s) {
    constexpr int RPL = Rpl<R>::v;
    const dim3 grid(nblk_b(N, 8), nblk_b(B, 32 * RPL));
    IFGF_DISPATCH_P(Ps, Pang, (k_final_b<R, PS, PA, RPL><<<grid, 256, 0, s>>>(N, point_leaf, leaf_start, leaf_count,
                                                                             nbr_ptr, nbr_box, near_rowlen, near_off, near,
                                                                             rho, ip_ptr, ip, coef, sorting, B, yt)));
}
void launch_bdot(const double2* V, long long ldc, int ncols, const double2* w, long long N, int B, double2* part,
                 double2* h, double2* Hcol, int add, int sqrt_row, cudaStream_t s) {
    if (ncols <= 0) return;
    const int nchunk = bdot_chunks(N);
    k_bdot_part<<<dim3(nchunk, ncols), 256, 0, s>>>(V, ldc, w, N, B, part);
    k_bdot_reduce<<<nblk_b((long long)ncols * B, 256), 256, 0, s>>>(part, nchunk, ncols, B, h, Hcol, add, sqrt_row);
}
void launch_bupdate(const double2* V, long long ldc, int ncols, const double2* h, double sign, long long N, int B, double2* w,
                    cudaStream_t s) {
    if (ncols <= 0) return;
    k_bupdate<<<nblk_b(N * B, 256), 256, 0, s>>>(V, ldc, ncols, h, sign, N * B, B, w);
}
void launch_bscale(const double2* w, const double2* hn, long long N, int B, double2* out, cudaStream_t s) {
    k_bscale<<<nblk_b(N * B, 256), 256, 0, s>>>(w, hn, N * B, B, out);
}

#define IFGF_BATCH_INSTANTIATE(R)                                                                                       \
    template void launch_leaf_b<R>(const int*, int, int, const int*, const int*, const long long*, const V2<R>*,        \
                                   const V2<R>*, int, int, int, V2<R>*, cudaStream_t);                                  \
    template void launch_prop_b<R>(int, int, const long long*, const int*, const PropB<R>*, int, int, const R*, int,    \
                                   V2<R>*, cudaStream_t, const R*);                                                     \
    template void launch_plan_rows<R>(const PropB<R>*, long long, int, int, R*, cudaStream_t);                         \
    template void launch_final_b<R>(int, const int*, const int*, const int*, const int*, const int*, const int*,        \
                                    const long long*, const V2<R>*, const V2<R>*, const int*, const InterpE<R>*,        \
                                    const V2<R>*, int, int, const long long*, int, double2*, cudaStream_t);
IFGF_BATCH_INSTANTIATE(double)
IFGF_BATCH_INSTANTIATE(float)

}  // namespace ifgf
