// ifgf_apply.cu -- per-apply IFGF kernels, templated on the arithmetic type.
//
// R = double: the plain form (complex128 tables, FP64 arithmetic).
// R = float : the mixed form (complex64 copies of the same FP64-computed tables, FP32
//             arithmetic; the rectangular-polar correction stays FP64).
//
//   k_intensities  density * quadrature weight, Morton permutation   ForwardMap.tpp:425-435, BoxTree.h:954-963
//   k_leaf_apply   leaf cone coefficients (one thread per cone x coefficient)      BoxTree.h:685-762
//   k_propagate    child -> parent coefficients (one thread per cone x node),
//                  separable values->coefficients map                             BoxTree.h:767-868, Interpolator.h:81-120
//   k_final        near field + every level's cousin interpolants, one warp per target,
//                  result added to y at the target's original index               BoxTree.h:614-683, 876-937, 1063-1069
#include "ifgf_device.cuh"
#include "tcgen05.cuh"
#include <type_traits>
#include <algorithm>
#include <atomic>

namespace ifgf {

template <typename R>
__global__ void k_intensities_t(const double2* __restrict__ x, const double* __restrict__ wq, const long long* __restrict__ perm,
                                int N, V2<R>* __restrict__ rho) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const long long o = perm ? perm[i] : i;
    const double2 v = x[o];
    const double w = wq[o];
    V2<R> r; r.x = (R)(v.x * w); r.y = (R)(v.y * w);
    rho[i] = r;
}

// thread = (leaf cone, source chunk, coefficient).  CH threads share one (cone, coefficient):
// chunk ch takes the sources s = ch, ch + CH, ...; the CH partial sums meet in shared memory.
// Boxes hold 10-100 points, so splitting the source walk shortens the latency chain of the
// longest boxes by CH.
template <typename R, int CH>
__global__ void __launch_bounds__(256) k_leaf_apply_t(const int* __restrict__ cone_box, int ncones, int cone_base,
                                                      const int* __restrict__ leaf_start, const int* __restrict__ leaf_count,
                                                      const long long* __restrict__ leaf_off, const V2<R>* __restrict__ L,
                                                      const V2<R>* __restrict__ rho, int P, V2<R>* __restrict__ coef) {
    __shared__ V2<R> part[256];
    const int per_cone = P * CH;
    const int cpb = blockDim.x / per_cone;
    const int local = threadIdx.x / per_cone, r = threadIdx.x - local * per_cone;
    const int ch = r / P, m = r - ch * P;
    const int c = blockIdx.x * cpb + local;
    const bool active = local < cpb && c < ncones;
    V2<R> a0, a1;
    a0.x = a0.y = a1.x = a1.y = R(0);
    if (active) {
        const int b = cone_box[c];
        const int n = leaf_count[b], s0 = leaf_start[b];
        const V2<R>* Lc = L + leaf_off[c] + m;
        const V2<R>* rh = rho + s0;
        int s = ch;
        for (; s + CH < n; s += 2 * CH) {
            const V2<R> l0 = Lc[(long long)s * P], l1 = Lc[(long long)(s + CH) * P];
            const V2<R> r0 = rh[s], r1 = rh[s + CH];
            cmac<R>(a0, l0, r0); cmac<R>(a1, l1, r1);
        }
        if (s < n) cmac<R>(a0, Lc[(long long)s * P], rh[s]);
        a0.x += a1.x; a0.y += a1.y;
    }
    part[threadIdx.x] = a0;
    __syncthreads();
    if (active && ch == 0) {
        V2<R> acc = a0;
        for (int q = 1; q < CH; ++q) { const V2<R> v = part[local * per_cone + q * P + m]; acc.x += v.x; acc.y += v.y; }
        coef[(long long)(cone_base + c) * P + m] = acc;
    }
}

// complex64 leaf cones with the table streamed by the tensor memory accelerator.  A persistent
// CTA walks its cones (blockIdx.x, + gridDim.x, ...) in pieces of at most kLtSrc sources; thread 0
// keeps kLtStages pieces in flight, each two cp.async.bulk copies (the piece's table rows and its
// densities) into a shared-memory ring, counted on the stage's mbarrier.  Each copy starts at the
// 16-byte boundary at or below its data (the table and density arrays carry 16 bytes of padding
// at their ends).  Threads (chunk, m) sum L[s][m] rho[s] over the piece's sources s = chunk mod kLtChunks,
// and a cone's chunk partials are reduced in shared memory.  Waits are bounded: one that runs
// out sets *err, waits once more for the copies in flight and stops the CTA.
constexpr int kLtSrc = 64, kLtStages = 4, kLtChunks = 5, kLtThreads = 128;
template <int P>
struct LeafTma {
    static constexpr int table = (kLtSrc * P * 8 + 16 + 127) / 128 * 128;   // table rows, then the densities
    static constexpr int stage = table + (kLtSrc * 8 + 16 + 127) / 128 * 128;
    static constexpr int part_off = kLtStages * stage;
    static constexpr int bar_off = part_off + kLtChunks * P * 8;
    static constexpr int smem = bar_off + 8 * kLtStages;
};
template <int P>
__global__ void __launch_bounds__(kLtThreads) k_leaf_tma(const int* __restrict__ cone_box, int ncones, int cone_base,
                                                         const int* __restrict__ leaf_start, const int* __restrict__ leaf_count,
                                                         const long long* __restrict__ leaf_off, const float2* __restrict__ L,
                                                         const float2* __restrict__ rho, float2* __restrict__ coef,
                                                         int* __restrict__ err) {
    static_assert(kLtChunks * P <= kLtThreads, "a thread per (chunk, coefficient)");
    using LT = LeafTma<P>;
    extern __shared__ __align__(128) unsigned char sm[];
    const int tid = threadIdx.x;
    const bool comp = tid < kLtChunks * P;
    const int ch = tid / P, m = tid - (tid / P) * P;
    float2* part = reinterpret_cast<float2*>(sm + LT::part_off);
    auto bar = [&](int st) { return tc5::smem_u32(sm + LT::bar_off + 8 * st); };
    // producer cursor (thread 0): the next piece to fetch
    int fc = blockIdx.x, fq = 0;
    auto piece_src = [&](int c, int q, int& n, int& len) {
        n = leaf_count[cone_box[c]];
        len = min(kLtSrc, n - q * kLtSrc);
        return reinterpret_cast<unsigned long long>(L + leaf_off[c] + (long long)q * kLtSrc * P);
    };
    auto fetch = [&](int st) {
        if (fc >= ncones) return;
        int n, len;
        const unsigned long long a = piece_src(fc, fq, n, len);
        const unsigned long long a0 = a & ~15ull;
        const uint32_t bytes = (uint32_t)(((a - a0) + (unsigned long long)len * P * 8 + 15) & ~15ull);
        const unsigned long long r = reinterpret_cast<unsigned long long>(rho + leaf_start[cone_box[fc]] + fq * kLtSrc);
        const unsigned long long r0 = r & ~15ull;
        const uint32_t rbytes = (uint32_t)(((r - r0) + (unsigned long long)len * 8 + 15) & ~15ull);
        tc5::mbar_expect_tx(bar(st), bytes + rbytes);
        tc5::bulk_g2s_counted(tc5::smem_u32(sm + st * LT::stage), reinterpret_cast<const void*>(a0), bytes, bar(st));
        tc5::bulk_g2s_counted(tc5::smem_u32(sm + st * LT::stage + LT::table), reinterpret_cast<const void*>(r0), rbytes, bar(st));
        if (++fq * kLtSrc >= n) { fq = 0; fc += gridDim.x; }
    };
    if (tid == 0) {
        for (int st = 0; st < kLtStages; ++st) tc5::mbar_init(bar(st), 1);
        for (int st = 0; st < kLtStages; ++st) fetch(st);
    }
    __syncthreads();
    long long piece = 0;
    int c = blockIdx.x, q = 0;
    float2 acc = make_float2(0.f, 0.f);
    bool ok = true;
    while (c < ncones) {
        const int st = (int)(piece % kLtStages);
        ok = __syncthreads_and(tc5::mbar_wait(bar(st), (uint32_t)((piece / kLtStages) & 1), 2000000000ll));
        if (!ok) break;
        int n, len;
        const unsigned long long a = piece_src(c, q, n, len);
        const float2* data = reinterpret_cast<const float2*>(sm + st * LT::stage + (a & 15ull));
        if (comp) {
            const unsigned long long r = reinterpret_cast<unsigned long long>(rho + leaf_start[cone_box[c]] + q * kLtSrc);
            const float2* rh = reinterpret_cast<const float2*>(sm + st * LT::stage + LT::table + (r & 15ull));
            for (int s2 = ch; s2 < len; s2 += kLtChunks) cmac<float>(acc, data[s2 * P + m], rh[s2]);
        }
        __syncthreads();                        // the stage has been read
        if (tid == 0) fetch(st);                // refill it with the piece kLtStages ahead
        ++piece;
        if (++q * kLtSrc >= n) {                // the cone is complete
            if (comp) part[ch * P + m] = acc;
            __syncthreads();
            if (comp && ch == 0) {
                float2 t = part[m];
                for (int k2 = 1; k2 < kLtChunks; ++k2) { t.x += part[k2 * P + m].x; t.y += part[k2 * P + m].y; }
                coef[(long long)(cone_base + c) * P + m] = t;
            }
            acc = make_float2(0.f, 0.f);
            q = 0;
            c += gridDim.x;
        }
    }
    if (!ok && tid == 0) {   // the pieces fetched ahead may still land: one more bounded wait each
        atomicExch(err, 1);
        for (int i = 0; i < kLtStages; ++i) {
            const long long p2 = piece + i;
            tc5::mbar_wait(bar((int)(p2 % kLtStages)), (uint32_t)((p2 / kLtStages) & 1), 2000000000ll);
        }
    }
}

// thread = (parent cone, interpolation node); CPB cones per block.  Gsep = [PS x PS radial
// map | PA x PA angular map] of the values->coefficients transform, normalisation included.
template <typename R, int PS, int PA, int CPB>
__global__ void __launch_bounds__(256) k_propagate_t(int pbegin, int pend, const long long* __restrict__ pp_ptr,
                                                     const int* __restrict__ pp_nchild, const PropE<R>* __restrict__ pp,
                                                     const R* __restrict__ Gsep, V2<R>* __restrict__ coef) {
    constexpr int P = PS * PA;
    __shared__ V2<R> sv[CPB][P];
    __shared__ V2<R> su[CPB][P];
    __shared__ R sGs[PS * PS], sGa[PA * PA];
    for (int i = threadIdx.x; i < PS * PS; i += blockDim.x) sGs[i] = Gsep[i];
    for (int i = threadIdx.x; i < PA * PA; i += blockDim.x) sGa[i] = Gsep[PS * PS + i];
    const int local = threadIdx.x / P, pt = threadIdx.x - local * P;
    const int pc = pbegin + blockIdx.x * CPB + local;
    const bool active = local < CPB && pc < pend;
    if (active) {
        const long long e0 = pp_ptr[pc];
        const int nch = pp_nchild[pc];
        V2<R> v; v.x = R(0); v.y = R(0);
        if (sizeof(R) == 4) {
            // all plan entries first, then two children's coefficient gathers before any arithmetic
            PropE<R> E[4];
#pragma unroll
            for (int ch = 0; ch < 4; ++ch) if (ch < nch) E[ch] = pp[e0 + (long long)ch * P + pt];
#pragma unroll
            for (int c0 = 0; c0 < 4; c0 += 2) {
                if (c0 >= nch) break;
                V2<R> ca[P], cb[P];
                const V2<R>* pa = coef + (long long)E[c0].child_cone * P;
                const bool two = c0 + 1 < nch;
                const int cb_cone = two ? E[c0 + 1].child_cone : E[c0].child_cone;
                const V2<R>* pb = coef + (long long)cb_cone * P;
#pragma unroll
                for (int q = 0; q < P; ++q) { ca[q] = pa[q]; cb[q] = pb[q]; }
                V2<R> w; w.x = E[c0].wr; w.y = E[c0].wi;
                cmac<R>(v, interp_eval<R, PS, PA>(ca, E[c0].s, E[c0].th), w);
                if (two) {
                    w.x = E[c0 + 1].wr; w.y = E[c0 + 1].wi;
                    cmac<R>(v, interp_eval<R, PS, PA>(cb, E[c0 + 1].s, E[c0 + 1].th), w);
                }
            }
        } else {
            for (int ch = 0; ch < nch; ++ch) {
                const PropE<R> E = pp[e0 + (long long)ch * P + pt];
                const V2<R> it = interp_eval<R, PS, PA>(coef + (long long)E.child_cone * P, E.s, E.th);
                V2<R> w; w.x = E.wr; w.y = E.wi;
                cmac<R>(v, it, w);
            }
        }
        sv[local][pt] = v;
    }
    __syncthreads();
    const int m = pt % PS, l = pt / PS;
    if (active) {            // u[l][m] = sum_k Gs[m][k] v[l*PS + k]
        V2<R> u; u.x = R(0); u.y = R(0);
#pragma unroll
        for (int k = 0; k < PS; ++k) {
            const R g = sGs[m * PS + k];
            const V2<R> v = sv[local][l * PS + k];
            u.x = rfma(g, v.x, u.x); u.y = rfma(g, v.y, u.y);
        }
        su[local][l * PS + m] = u;
    }
    __syncthreads();
    if (active) {            // c[n][m] = sum_l Ga[n][l] u[l][m], stored at n*PS + m
        const int n = l;
        V2<R> c; c.x = R(0); c.y = R(0);
#pragma unroll
        for (int q = 0; q < PA; ++q) {
            const R g = sGa[n * PA + q];
            const V2<R> u = su[local][q * PS + m];
            c.x = rfma(g, u.x, c.x); c.y = rfma(g, u.y, c.y);
        }
        coef[(long long)pc * P + n * PS + m] = c;
    }
}

// k_propagate_t with the child coefficient blocks staged in shared memory.  A parent cone's 25
// nodes read 1-4 children's blocks each, but the block's ten parent cones touch only about 40
// distinct child cones (3.4-4.3 per parent cone on the kite trees), so the per-thread gathers
// of k_propagate_t read each block about twelve times.  Here the block first collects its
// distinct child cones in a shared hash table (open addressing, at most kStageKeys probes),
// copies each one's block once with coalesced loads, and evaluates from shared memory.  A child
// cone that finds no free key or no data slot is read from global memory.  Each thread's
// arithmetic is that of k_propagate_t in the same order, so the results are bit-identical.
// FP64 gains a few per cent from it (the autotuner takes it on the finer levels); in complex64
// the 25 shared-memory reads per term cost as much as the L1 hits they replace.
constexpr int kStageKeys = 128;
template <typename R, int P>
struct PropStage {
    static constexpr int cap = (size_t)P * sizeof(V2<R>) * 64 <= 26000 ? 64 : (int)(26000 / ((size_t)P * sizeof(V2<R>)));
};
template <typename R, int PS, int PA, int CPB>
__global__ void __launch_bounds__(256) k_propagate_st(int pbegin, int pend, const long long* __restrict__ pp_ptr,
                                                      const int* __restrict__ pp_nchild, const PropE<R>* __restrict__ pp,
                                                      const R* __restrict__ Gsep, V2<R>* __restrict__ coef) {
    constexpr int P = PS * PA;
    constexpr int CAP = PropStage<R, P>::cap;
    __shared__ int key[kStageKeys], slot_of[kStageKeys], ulist[CAP];
    __shared__ int nused;
    __shared__ V2<R> blk[CAP][P];
    __shared__ V2<R> sv[CPB][P];
    __shared__ V2<R> su[CPB][P];
    __shared__ R sGs[PS * PS], sGa[PA * PA];
    for (int i = threadIdx.x; i < PS * PS; i += blockDim.x) sGs[i] = Gsep[i];
    for (int i = threadIdx.x; i < PA * PA; i += blockDim.x) sGa[i] = Gsep[PS * PS + i];
    for (int i = threadIdx.x; i < kStageKeys; i += blockDim.x) key[i] = -1;
    if (threadIdx.x == 0) nused = 0;
    const int local = threadIdx.x / P, pt = threadIdx.x - local * P;
    const int pc = pbegin + blockIdx.x * CPB + local;
    const bool active = local < CPB && pc < pend;
    PropE<R> E[4];
    int nch = 0, pos[4] = {-1, -1, -1, -1};
    if (active) {
        const long long e0 = pp_ptr[pc];
        nch = min(pp_nchild[pc], 4);
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) if (ch < nch) E[ch] = pp[e0 + (long long)ch * P + pt];
    }
    __syncthreads();
    // the distinct child cones of the block: lanes of a warp that share a cone elect one leader,
    // which claims (or finds) the cone's key; the thread that claims a key appends the cone
    const int lane = threadIdx.x & 31;
    const int wsize = min(32, (int)blockDim.x - (int)(threadIdx.x & ~31u));   // the block's last warp may be partial
    const unsigned wmask = wsize == 32 ? 0xffffffffu : (1u << wsize) - 1u;
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
        const int c = ch < nch ? E[ch].child_cone : -1;
        const unsigned peers = __match_any_sync(wmask, c);
        const int leader = __ffs(peers) - 1;
        int h = -1;
        if (c >= 0 && lane == leader) {
            int q = (int)(((unsigned)c * 2654435761u) >> 25) & (kStageKeys - 1);
            for (int probe = 0; probe < kStageKeys; ++probe) {
                const int old = atomicCAS(&key[q], -1, c);
                if (old == -1) {
                    const int id = atomicAdd(&nused, 1);
                    slot_of[q] = id < CAP ? id : -1;
                    if (id < CAP) ulist[id] = c;
                    h = q;
                    break;
                }
                if (old == c) { h = q; break; }
                q = (q + 1) & (kStageKeys - 1);
            }
        }
        h = __shfl_sync(wmask, h, leader);
        if (c >= 0) pos[ch] = h;
    }
    __syncthreads();
    // one coalesced copy of each distinct child block
    {
        const int n = min(nused, CAP) * P;
        for (int i0 = threadIdx.x; i0 < n; i0 += 4 * blockDim.x) {
            V2<R> v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * blockDim.x;
                if (i < n) v[u] = coef[(long long)ulist[i / P] * P + i % P];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * blockDim.x;
                if (i < n) blk[i / P][i % P] = v[u];
            }
        }
    }
    __syncthreads();
    if (active) {
        V2<R> v; v.x = R(0); v.y = R(0);
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
            if (ch >= nch) break;
            const int slot = pos[ch] >= 0 ? slot_of[pos[ch]] : -1;
            const V2<R> it = slot >= 0 ? interp_eval<R, PS, PA>(blk[slot], E[ch].s, E[ch].th)
                                       : interp_eval<R, PS, PA>(coef + (long long)E[ch].child_cone * P, E[ch].s, E[ch].th);
            V2<R> w; w.x = E[ch].wr; w.y = E[ch].wi;
            cmac<R>(v, it, w);
        }
        sv[local][pt] = v;
    }
    __syncthreads();
    const int m = pt % PS, l = pt / PS;
    if (active) {            // u[l][m] = sum_k Gs[m][k] v[l*PS + k]
        V2<R> u; u.x = R(0); u.y = R(0);
#pragma unroll
        for (int k = 0; k < PS; ++k) {
            const R g = sGs[m * PS + k];
            const V2<R> vv = sv[local][l * PS + k];
            u.x = rfma(g, vv.x, u.x); u.y = rfma(g, vv.y, u.y);
        }
        su[local][l * PS + m] = u;
    }
    __syncthreads();
    if (active) {            // c[n][m] = sum_l Ga[n][l] u[l][m], stored at n*PS + m
        const int n = l;
        V2<R> c; c.x = R(0); c.y = R(0);
#pragma unroll
        for (int q = 0; q < PA; ++q) {
            const R g = sGa[n * PA + q];
            const V2<R> u = su[local][q * PS + m];
            c.x = rfma(g, u.x, c.x); c.y = rfma(g, u.y, c.y);
        }
        coef[(long long)pc * P + n * PS + m] = c;
    }
}

// one warp per (leaf box, up to 32 of its targets, kIbPiece of their interpolation terms), one
// lane per target.  The targets of a leaf box share their ancestors, hence the same cousin lists
// in the same order: their j-th terms read the same cousin box, mostly the same cone (2.5-3
// distinct cones per warp step on the kite trees, against up to 32 when a warp walks one target's
// terms), so the coefficient gathers are broadcasts.  The plan is stored box-transposed (term j of
// the box's target t at box base + j n + t) for coalesced entry loads.  Each lane writes its
// piece's sum to part[piece][target]; k_final_t adds the pieces in order.
template <typename R, int PS, int PA>
__global__ void __launch_bounds__(256) k_interp_box(const int4* __restrict__ items, int nitems, int N,
                                                    const int* __restrict__ leaf_start, const int* __restrict__ leaf_count,
                                                    const int* __restrict__ ip_ptr, const InterpE<R>* __restrict__ ipT,
                                                    const V2<R>* __restrict__ coef, V2<R>* __restrict__ part) {
    constexpr int P = PS * PA;
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (w >= nitems) return;
    const int lane = threadIdx.x & 31;
    const int4 I = items[w];   // leaf box, first target, terms [z, w)
    const int s = leaf_start[I.x], n = leaf_count[I.x];
    const int t = I.y + lane;
    if (t >= n) return;
    const InterpE<R>* e = ipT + ip_ptr[s] + t;
    V2<R> acc; acc.x = R(0); acc.y = R(0);
    int j = I.z;
    if constexpr (sizeof(R) == 4) {   // two terms' loads in flight before either is evaluated
        for (; j + 1 < I.w; j += 2) {
            const InterpE<R> E0 = e[(long long)j * n], E1 = e[(long long)(j + 1) * n];
            V2<R> c0[P], c1[P];
            const V2<R>* b0 = coef + (long long)E0.cone * P;
            const V2<R>* b1 = coef + (long long)E1.cone * P;
#pragma unroll
            for (int q = 0; q < P; ++q) { c0[q] = b0[q]; c1[q] = b1[q]; }
            V2<R> f; f.x = E0.fr; f.y = E0.fi;
            cmac<R>(acc, interp_eval<R, PS, PA>(c0, E0.s, E0.th), f);
            f.x = E1.fr; f.y = E1.fi;
            cmac<R>(acc, interp_eval<R, PS, PA>(c1, E1.s, E1.th), f);
        }
    }
    for (; j < I.w; ++j) {
        const InterpE<R> E = e[(long long)j * n];
        V2<R> c[P];
        const V2<R>* cb = coef + (long long)E.cone * P;
#pragma unroll
        for (int q = 0; q < P; ++q) c[q] = cb[q];
        V2<R> f; f.x = E.fr; f.y = E.fi;
        cmac<R>(acc, interp_eval<R, PS, PA>(c, E.s, E.th), f);
    }
    part[(long long)(I.z / kIbPiece) * N + s + t] = acc;
}

// near field by leaf box: one block per (leaf box, up to 32 of its targets).  The box's
// neighbour densities rho[src[e]] are staged in shared memory kNearChunk at a time, once for all
// its targets, and each warp streams its targets' table rows (coalesced) against them; a target's
// chunk sums meet in shared memory in chunk order.  Then the target's interpolation pieces
// (k_interp_box) are added in order and the sum goes to y at the target's original index.
template <typename R>
__global__ void __launch_bounds__(256) k_near_box(const int2* __restrict__ items, const int* __restrict__ leaf_start,
                                                  const int* __restrict__ leaf_count, const int* __restrict__ near_src_off,
                                                  const int* __restrict__ near_src, const int* __restrict__ near_rowlen,
                                                  const long long* __restrict__ near_off, const V2<R>* __restrict__ near,
                                                  const V2<R>* __restrict__ rho, const int* __restrict__ ip_ptr,
                                                  const V2<R>* __restrict__ part, int N, const long long* __restrict__ sorting,
                                                  double2* __restrict__ y) {
    static_assert(kNearTargets == 4 * 8, "eight warps of four targets");
    __shared__ V2<R> srho[kNearChunk];
    __shared__ V2<R> sacc[kNearTargets];
    const int2 I = items[blockIdx.x];   // leaf box, first target
    const int b = I.x, s = leaf_start[b], n = min(kNearTargets, leaf_count[b] - I.y);
    const int rl = near_rowlen[b];
    const int* src = near_src + near_src_off[b];
    const V2<R>* rows = near + near_off[b] + (long long)I.y * rl;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < kNearTargets) { sacc[threadIdx.x].x = R(0); sacc[threadIdx.x].y = R(0); }
    for (int c0 = 0; c0 < rl; c0 += kNearChunk) {
        const int cn = min(kNearChunk, rl - c0);
        __syncthreads();   // the previous chunk has been read
        for (int e = threadIdx.x; e < cn; e += blockDim.x) srho[e] = rho[src[c0 + e]];
        __syncthreads();
        // warp w: targets 4 w .. 4 w + 3 together (four independent row loads per density read)
        const int t0 = 4 * warp;
        if (t0 < n) {
            V2<R> acc[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { acc[u].x = R(0); acc[u].y = R(0); }
            const V2<R>* row = rows + (long long)t0 * rl + c0;
#pragma unroll 2
            for (int e = lane; e < cn; e += 32) {
                const V2<R> r = srho[e];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (t0 + u < n) cmac<R>(acc[u], row[(long long)u * rl + e], r);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const R ax = warp_sum_r<R>(acc[u].x), ay = warp_sum_r<R>(acc[u].y);
                if (lane == 0 && t0 + u < n) { sacc[t0 + u].x += ax; sacc[t0 + u].y += ay; }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < n) {
        const int i = s + I.y + threadIdx.x;
        V2<R> acc = sacc[threadIdx.x];
        if (part) {
            const int npc = (ip_ptr[i + 1] - ip_ptr[i] + kIbPiece - 1) / kIbPiece;
            for (int q = 0; q < npc; ++q) { const V2<R> a = part[(long long)q * N + i]; acc.x += a.x; acc.y += a.y; }
        }
        const long long o = sorting[i];
        double2 v = y[o];
        v.x += (double)acc.x; v.y += (double)acc.y;
        y[o] = v;
    }
}

// the interpolation plan of each leaf box transposed: term j of the box's target t moves from
// ip_ptr[i] + j to ip_ptr[box's first target] + j n + t (every target of a box has as many terms)
template <typename R>
__global__ void k_interp_transpose(int N, const int* __restrict__ point_leaf, const int* __restrict__ leaf_start,
                                   const int* __restrict__ leaf_count, const int* __restrict__ ip_ptr,
                                   const InterpE<double>* __restrict__ in, InterpE<R>* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int b = point_leaf[i], s = leaf_start[b], n = leaf_count[b], t = i - s;
    const int base = ip_ptr[s], nt = ip_ptr[i + 1] - ip_ptr[i];
    for (int j = 0; j < nt; ++j) {
        const InterpE<double> E = in[ip_ptr[i] + j];
        InterpE<R> o{};
        o.cone = E.cone; o.s = (R)E.s; o.th = (R)E.th; o.fr = (R)E.fr; o.fi = (R)E.fi;
        out[base + (long long)j * n + t] = o;
    }
}

// one warp per Morton-sorted target; near row layout [target][neighbour sources], and
// near_src[near_src_off[b] + e] the Morton index of entry e's source in leaf box b's rows, so the
// lanes stride over one flat row with independent loads.  With `part`, the interpolation terms were
// summed by k_interp_box: the target's pieces are added in order instead.
template <typename R, int PS, int PA>
__global__ void __launch_bounds__(256) k_final_t(int N, const int* __restrict__ point_leaf, const int* __restrict__ leaf_start,
                                                 const int* __restrict__ near_src_off, const int* __restrict__ near_src,
                                                 const int* __restrict__ near_rowlen,
                                                 const long long* __restrict__ near_off, const V2<R>* __restrict__ near,
                                                 const V2<R>* __restrict__ rho, const int* __restrict__ ip_ptr,
                                                 const InterpE<R>* __restrict__ ip, const V2<R>* __restrict__ coef,
                                                 const long long* __restrict__ sorting, double2* __restrict__ y,
                                                 const V2<R>* __restrict__ part) {
    constexpr int P = PS * PA;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= N) return;
    const int b = point_leaf[i];
    const int t = i - leaf_start[b];
    const int rl = near_rowlen[b];
    const V2<R>* row = near + near_off[b] + (long long)t * rl;
    const int* src = near_src + near_src_off[b];
    V2<R> acc; acc.x = R(0); acc.y = R(0);
#pragma unroll 4
    for (int e = lane; e < rl; e += 32) cmac<R>(acc, row[e], rho[src[e]]);
    if (!part) {
        for (int e = ip_ptr[i] + lane; e < ip_ptr[i + 1]; e += 32) {
            const InterpE<R> E = ip[e];
            const V2<R> it = interp_eval<R, PS, PA>(coef + (long long)E.cone * P, E.s, E.th);
            V2<R> f; f.x = E.fr; f.y = E.fi;
            cmac<R>(acc, it, f);
        }
    }
    acc.x = warp_sum_r<R>(acc.x);
    acc.y = warp_sum_r<R>(acc.y);
    if (lane == 0) {
        if (part) {
            const int npc = (ip_ptr[i + 1] - ip_ptr[i] + kIbPiece - 1) / kIbPiece;
            for (int q = 0; q < npc; ++q) { const V2<R> a = part[(long long)q * N + i]; acc.x += a.x; acc.y += a.y; }
        }
        const long long o = sorting[i];
        double2 v = y[o];
        v.x += (double)acc.x; v.y += (double)acc.y;
        y[o] = v;
    }
}

__global__ void k_d2f(const double2* __restrict__ a, long long n, float2* __restrict__ b) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

// ------------------------------------------------------------------ launchers
static inline unsigned nblk_a(long long n, int b) { return (unsigned)((n + b - 1) / b); }

template <typename R>
void launch_intensities_t(const double2* x, const double* wq, const long long* perm, int N, V2<R>* rho, cudaStream_t s) {
    k_intensities_t<R><<<nblk_a(N, 256), 256, 0, s>>>(x, wq, perm, N, rho);
}
cudaError_t preload_intensities_kernel() {
    cudaFuncAttributes a;
    return cudaFuncGetAttributes(&a, k_intensities_t<double>);
}
template <typename R>
void launch_leaf_apply_t(const int* cone_box, int ncones, int cone_base, const int* leaf_start, const int* leaf_count,
                         const long long* leaf_off, const V2<R>* L, const V2<R>* rho, int P, V2<R>* coef, cudaStream_t s,
                         int chunks) {
    if (ncones <= 0) return;
    // chunks per coefficient (the tuning variant): 1, 2, 5 or 10; a block holds 256 / (P * CH) cones
    auto go = [&](auto ch_tag) {
        constexpr int CH = decltype(ch_tag)::value;
        const int cpb = 256 / (P * CH);
        k_leaf_apply_t<R, CH><<<nblk_a(ncones, cpb), cpb * P * CH, 0, s>>>(cone_box, ncones, cone_base, leaf_start, leaf_count,
                                                                          leaf_off, L, rho, P, coef);
    };
    if (chunks == 10 && 256 / (P * 10) >= 1) go(std::integral_constant<int, 10>{});
    else if (chunks == 2 && 256 / (P * 2) >= 1) go(std::integral_constant<int, 2>{});
    else if (chunks == 1 || 256 / (P * 5) < 1) go(std::integral_constant<int, 1>{});
    else go(std::integral_constant<int, 5>{});
}
static std::atomic<int> g_leaf_tma_ready{0};
cudaError_t leaf_tma_init() {
    if (g_leaf_tma_ready.load()) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(k_leaf_tma<25>, cudaFuncAttributeMaxDynamicSharedMemorySize, LeafTma<25>::smem);
    if (e == cudaSuccess) g_leaf_tma_ready.store(1);
    return e;
}
bool launch_leaf_tma(const int* cone_box, int ncones, int cone_base, const int* leaf_start, const int* leaf_count,
                     const long long* leaf_off, const float2* L, const float2* rho, int P, float2* coef, int* err, int nsm,
                     cudaStream_t s) {
    if (P != 25) return false;
    if (ncones <= 0) return true;
    if (!g_leaf_tma_ready.load()) return false;   // leaf_tma_init not run on this device
    const int grid = std::min(ncones, 4 * std::max(nsm, 1));
    k_leaf_tma<25><<<grid, kLtThreads, LeafTma<25>::smem, s>>>(cone_box, ncones, cone_base, leaf_start, leaf_count, leaf_off, L,
                                                              rho, coef, err);
    return true;
}
template <typename R>
void launch_propagate_t(int pbegin, int pend, const long long* pp_ptr, const int* pp_nchild, const PropE<R>* pp, int Ps, int Pang,
                        const R* Gsep, V2<R>* coef, cudaStream_t s, int cones_per_block) {
    if (pend <= pbegin) return;
    // cones per block (the tuning variant): 2, 4 or the most that fit 256 threads; kPropStaged:
    // the most that fit, child blocks staged in shared memory
    IFGF_DISPATCH_P(Ps, Pang, {
        constexpr int CPBMAX = 256 / (PS * PA);
        if (cones_per_block == kPropStaged)
            k_propagate_st<R, PS, PA, CPBMAX><<<nblk_a(pend - pbegin, CPBMAX), CPBMAX * PS * PA, 0, s>>>(pbegin, pend, pp_ptr,
                                                                                                      pp_nchild, pp, Gsep, coef);
        else if (cones_per_block == 2 && CPBMAX >= 2)
            k_propagate_t<R, PS, PA, 2><<<nblk_a(pend - pbegin, 2), 2 * PS * PA, 0, s>>>(pbegin, pend, pp_ptr, pp_nchild, pp, Gsep, coef);
        else if (cones_per_block == 4 && CPBMAX >= 4)
            k_propagate_t<R, PS, PA, 4><<<nblk_a(pend - pbegin, 4), 4 * PS * PA, 0, s>>>(pbegin, pend, pp_ptr, pp_nchild, pp, Gsep, coef);
        else
            k_propagate_t<R, PS, PA, CPBMAX><<<nblk_a(pend - pbegin, CPBMAX), CPBMAX * PS * PA, 0, s>>>(pbegin, pend, pp_ptr,
                                                                                                     pp_nchild, pp, Gsep, coef);
    });
}
template <typename R>
void launch_final_t(int N, const int* point_leaf, const int* leaf_start, const int* near_src_off, const int* near_src,
                    const int* near_rowlen, const long long* near_off, const V2<R>* near, const V2<R>* rho,
                    const int* ip_ptr, const InterpE<R>* ip, const V2<R>* coef, int Ps, int Pang, const long long* sorting,
                    double2* y, cudaStream_t s, const V2<R>* part) {
    IFGF_DISPATCH_P(Ps, Pang, (k_final_t<R, PS, PA><<<nblk_a((long long)N * 32, 256), 256, 0, s>>>(
                                   N, point_leaf, leaf_start, near_src_off, near_src, near_rowlen, near_off, near, rho,
                                   ip_ptr, ip, coef, sorting, y, part)));
}
template <typename R>
void launch_interp_box(const int4* items, int nitems, int N, const int* leaf_start, const int* leaf_count, const int* ip_ptr,
                       const InterpE<R>* ipT, const V2<R>* coef, int Ps, int Pang, V2<R>* part, cudaStream_t s) {
    if (nitems <= 0) return;
    IFGF_DISPATCH_P(Ps, Pang, (k_interp_box<R, PS, PA><<<nblk_a((long long)nitems * 32, 256), 256, 0, s>>>(
                                   items, nitems, N, leaf_start, leaf_count, ip_ptr, ipT, coef, part)));
}
template <typename R>
void launch_near_box(const int2* items, int nitems, const int* leaf_start, const int* leaf_count, const int* near_src_off,
                     const int* near_src, const int* near_rowlen, const long long* near_off, const V2<R>* near, const V2<R>* rho,
                     const int* ip_ptr, const V2<R>* part, int N, const long long* sorting, double2* y, cudaStream_t s) {
    if (nitems > 0)
        k_near_box<R><<<nitems, 256, 0, s>>>(items, leaf_start, leaf_count, near_src_off, near_src, near_rowlen, near_off, near,
                                              rho, ip_ptr, part, N, sorting, y);
}
template <typename R>
void launch_interp_transpose(int N, const int* point_leaf, const int* leaf_start, const int* leaf_count, const int* ip_ptr,
                             const InterpE<double>* in, InterpE<R>* out, cudaStream_t s) {
    if (N > 0) k_interp_transpose<R><<<nblk_a(N, 256), 256, 0, s>>>(N, point_leaf, leaf_start, leaf_count, ip_ptr, in, out);
}
void launch_d2f(const double2* a, long long n, float2* b, cudaStream_t s) {
    if (n > 0) k_d2f<<<nblk_a(n, 256), 256, 0, s>>>(a, n, b);
}

#define IFGF_INSTANTIATE(R)                                                                                          \
    template void launch_intensities_t<R>(const double2*, const double*, const long long*, int, V2<R>*, cudaStream_t); \
    template void launch_leaf_apply_t<R>(const int*, int, int, const int*, const int*, const long long*, const V2<R>*,  \
                                         const V2<R>*, int, V2<R>*, cudaStream_t, int);                               \
    template void launch_propagate_t<R>(int, int, const long long*, const int*, const PropE<R>*, int, int, const R*,   \
                                        V2<R>*, cudaStream_t, int);                                                    \
    template void launch_final_t<R>(int, const int*, const int*, const int*, const int*, const int*,                   \
                                    const long long*, const V2<R>*, const V2<R>*, const int*, const InterpE<R>*,       \
                                    const V2<R>*, int, int, const long long*, double2*, cudaStream_t, const V2<R>*);      \
    template void launch_interp_box<R>(const int4*, int, int, const int*, const int*, const int*, const InterpE<R>*,     \
                                       const V2<R>*, int, int, V2<R>*, cudaStream_t);                                    \
    template void launch_interp_transpose<R>(int, const int*, const int*, const int*, const int*,                        \
                                             const InterpE<double>*, InterpE<R>*, cudaStream_t);                          \
    template void launch_near_box<R>(const int2*, int, const int*, const int*, const int*, const int*, const int*,       \
                                     const long long*, const V2<R>*, const V2<R>*, const int*, const V2<R>*, int,        \
                                     const long long*, double2*, cudaStream_t);
IFGF_INSTANTIATE(double)
IFGF_INSTANTIATE(float)

}  // namespace ifgf
