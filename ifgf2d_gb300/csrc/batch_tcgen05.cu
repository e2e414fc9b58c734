// batch_tcgen05.cu -- complex64 batched IFGF kernels on the fifth-generation tensor cores
// (tcgen05.mma kind::tf32) in 3xTF32 split precision: each FP32 operand is split x = hi + lo
// (TF32) and D += A_lo B_hi + A_hi B_lo + A_hi B_hi keeps FP32-level accuracy (Ootomo and
// Yokota, IJHPCA 2022).  Operands are split by the threads into shared memory (K-major, no
// swizzle; tcgen05.cuh), one thread issues the MMAs and commits them to an mbarrier, the FP32
// accumulators live in tensor memory.
//
// k_leaf_t5: leaf cone coefficients (BoxTree.h:685-762).  Per leaf box, one dense GEMM
//   D[2 r + part][(cone, m)] = sum_src A[2 r + part][src] B[(cone, m)][src],
//   A[2 r] = [Re rho_src,r | -Im rho_src,r], A[2 r + 1] = [Im rho | Re rho],
//   B[(cone, m)] = [Re L_cone[src][m] | Im L_cone[src][m]]
// (rows 2 r, 2 r + 1 = real and imaginary parts of right-hand side r), so that D holds
// Re / Im sum_src L rho.  A work item is a leaf box and up to five of its cones (125 columns,
// N = 128); sources in chunks of 16 (K = 32) accumulate in tensor memory.  The next chunk's
// densities and table entries are loaded into registers while the current chunk's MMAs run.
// Each table entry is used by 128 rows, so the arithmetic that binds the FP32 FMA kernel moves
// to the tensor pipe and the kernel is left with loads, splits and coefficient stores.
//
// k_prop_t5: child -> parent propagation (BoxTree.h:767-868, Interpolator.h:81-120).
// For one parent cone and 64 right-hand sides r, the parent's node values are
//   V[n][r] = sum over terms t of node n:  f_t sum_p w_t[p] C_{q(t)}[p][r]
// (w_t[p] = T_a(th_t) T_s(s_t), p = a PS + s, f_t the factorization ratio, C_q the child cone's
// coefficients).  Terms are grouped by child cone q; each group is one real GEMM with
//   rows    m = r (real part) and 64 + r (imaginary part):  A[r][k] = [Re C_q[p][r] | -Im C_q[p][r]],
//           A[64 + r][k] = [Im C_q[p][r] | Re C_q[p][r]]   (k = p, and 28 + p for the second half)
//   columns n = parent node:  B[n][k] = [Re (f_t w_t[p]) | Im (f_t w_t[p])] for the term t of node n
//           in the group, 0 for nodes without one
// so that D[r][n] = Re V[n][r] and D[64 + r][n] = Im V[n][r].  Every group of the parent accumulates
// into the same 128 x 32 FP32 tile in tensor memory (tcgen05.mma kind::tf32, M = 128, N = 32,
// K = 56 in 7 steps).  The values -> coefficients map (Chebyshev transform, real 25 x 25) is a second GEMM on the tile read back from tensor
// memory: D2[m][c] = sum_n D[m][n] Map[c][n].
//
// One CTA of 128 threads walks parent cones (grid stride).  Per group: the group's interpolation
// weights are computed while the previous group's MMAs run, then all threads split and store the
// A and B operands in shared memory (K-major, no swizzle), one thread issues the 21 MMAs and
// commits them to an mbarrier.  Waits are bounded; a wait that runs out sets *err, and the CTA
// stops, frees its tensor memory and returns.  Propagation terms are sparse per child cone (a
// group reads one child cone's 25 x 64 coefficients for ~20 terms), so splitting that block
// costs about as much as the FP32 FMA kernel's arithmetic: this kernel is the slower of the two
// and is kept as a launch-shape choice.
#include <algorithm>
#include "ifgf_device.cuh"
#include "tcgen05.cuh"

namespace ifgf {
namespace {

constexpr int kT5Threads = 128;
constexpr int kT5Half = 28;                  // K of one half (P <= 28)
constexpr int kT5K = 2 * kT5Half;            // 56
constexpr int kT5N = 32;                     // parent nodes (P <= 32), also coefficients of the map
constexpr int kT5MaxB = 64;
constexpr int kT5MaxTerms = 4 * 28;          // four children x P
// shared memory (bytes)
constexpr int T5_A = 128 * kT5K * 4;         // one of hi / lo: 28672
constexpr int T5_B = kT5N * kT5K * 4;        // 7168
constexpr int T5_B2 = kT5N * kT5N * 4;       // 4096
constexpr int OFF_AH = 0, OFF_AL = T5_A;
constexpr int OFF_BH = 2 * T5_A, OFF_BL = OFF_BH + T5_B;
constexpr int OFF_B2H = OFF_BL + T5_B, OFF_B2L = OFF_B2H + T5_B2;
constexpr int OFF_SW = OFF_B2L + T5_B2;                        // group weights [32][28] floats
constexpr int OFF_ST = OFF_SW + 32 * kT5Half * 4;              // the parent's terms
constexpr int OFF_NL = OFF_ST + kT5MaxTerms * (int)sizeof(PropB<float>);   // per node: (group, term) x 4
constexpr int OFF_NC = OFF_NL + kT5N * 4 * 8;                  // per node: count
constexpr int OFF_GS = OFF_NC + kT5N * 4;                      // group starts (<= terms + 1)
constexpr int OFF_BAR = (OFF_GS + (kT5MaxTerms + 2) * 4 + 15) / 16 * 16;
constexpr int T5_SMEM = OFF_BAR + 32;
static_assert(OFF_SW % 16 == 0 && OFF_ST % 8 == 0, "alignment");
constexpr long long kT5WaitCycles = 2000000000ll;   // about one second at 2 GHz

__device__ __forceinline__ void st4(unsigned char* sm, uint32_t off, float a, float b, float c, float d) {
    *(float4*)(sm + off) = make_float4(a, b, c, d);
}
// split four values and store hi / lo at the same offset of the two tiles
__device__ __forceinline__ void st4_split(unsigned char* sm, int off_hi, int off_lo, uint32_t off, float a, float b, float c,
                                          float d, float sign) {
    float ah, al, bh, bl, ch, cl, dh, dl;
    tc5::split3(a, ah, al); tc5::split3(b, bh, bl); tc5::split3(c, ch, cl); tc5::split3(d, dh, dl);
    st4(sm, off_hi + off, sign * ah, sign * bh, sign * ch, sign * dh);
    st4(sm, off_lo + off, sign * al, sign * bl, sign * cl, sign * dl);
}

// one thread waits for the MMAs (the others wait at the barrier that follows); true when they completed
__device__ __forceinline__ bool wait_one(int tid, uint32_t bar, uint32_t parity) {
    return tid == 0 ? tc5::mbar_wait(bar, parity, kT5WaitCycles) : true;
}

__device__ __forceinline__ void issue_3xtf32(uint32_t d, uint32_t ah, uint32_t al, uint32_t a_lbo, uint32_t bh, uint32_t bl,
                                             uint32_t b_lbo, int ksteps, uint32_t idesc, bool accumulate) {
    uint32_t acc = accumulate ? 1u : 0u;
    for (int ks = 0; ks < ksteps; ++ks) {
        const uint32_t ao = ks * 2 * a_lbo, bo = ks * 2 * b_lbo;
        tc5::mma_tf32(d, tc5::smem_desc(al + ao, a_lbo, 128), tc5::smem_desc(bh + bo, b_lbo, 128), idesc, acc);
        acc = 1u;
        tc5::mma_tf32(d, tc5::smem_desc(ah + ao, a_lbo, 128), tc5::smem_desc(bl + bo, b_lbo, 128), idesc, 1u);
    }
    for (int ks = 0; ks < ksteps; ++ks) {
        const uint32_t ao = ks * 2 * a_lbo, bo = ks * 2 * b_lbo;
        tc5::mma_tf32(d, tc5::smem_desc(ah + ao, a_lbo, 128), tc5::smem_desc(bh + bo, b_lbo, 128), idesc, 1u);
    }
}

template <int PS, int PA>
__global__ void __launch_bounds__(kT5Threads) k_prop_t5(int pbegin, int pend, const long long* __restrict__ pp_ptr,
                                                        const int* __restrict__ pp_nchild, const PropB<float>* __restrict__ pb,
                                                        const float* __restrict__ Gsep, int B, float2* __restrict__ coef,
                                                        int* __restrict__ err) {
    constexpr int P = PS * PA;
    static_assert(P <= kT5Half, "parent nodes must fit one K half");
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    PropB<float>* st = (PropB<float>*)(sm + OFF_ST);
    float* sw = (float*)(sm + OFF_SW);
    int2* nl = (int2*)(sm + OFF_NL);
    int* nc = (int*)(sm + OFF_NC);
    int* gstart = (int*)(sm + OFF_GS);
    int* ngroups = (int*)(sm + OFF_BAR + 12);
    const uint32_t bar = tc5::smem_u32(sm + OFF_BAR), tslot = tc5::smem_u32(sm + OFF_BAR + 8);
    const uint32_t sAH = tc5::smem_u32(sm + OFF_AH), sAL = tc5::smem_u32(sm + OFF_AL);
    const uint32_t sBH = tc5::smem_u32(sm + OFF_BH), sBL = tc5::smem_u32(sm + OFF_BL);
    const uint32_t sB2H = tc5::smem_u32(sm + OFF_B2H), sB2L = tc5::smem_u32(sm + OFF_B2L);

    // the values -> coefficients map, rows = coefficient n*PS + m, K = node l*PS + q:
    // Map = Ga[n][l] Gs[m][q] (Gsep holds Gs (PS x PS) then Ga (PA x PA))
    for (int i = tid; i < kT5N * kT5N; i += kT5Threads) {
        const int c = i >> 5, nd = i & 31;
        const float v = (c < P && nd < P) ? Gsep[PS * PS + (c / PS) * PA + nd / PS] * Gsep[(c % PS) * PS + nd % PS] : 0.f;
        float hi, lo;
        tc5::split3(v, hi, lo);
        *(float*)(sm + OFF_B2H + tc5::kmajor_off(kT5N, c, nd)) = hi;
        *(float*)(sm + OFF_B2L + tc5::kmajor_off(kT5N, c, nd)) = lo;
    }
    if (tid == 0) tc5::mbar_init(bar, 1);
    if (warp == 0) tc5::tmem_alloc(tslot, 64);
    tc5::fence_async_smem();
    tc5::fence_before_sync();
    __syncthreads();
    tc5::fence_after_sync();
    const uint32_t tmem = *(volatile uint32_t*)(sm + OFF_BAR + 8);
    const uint32_t tD = tmem, tD2 = tmem + 32, lane_base = (uint32_t)(32 * warp) << 16;
    const uint32_t idesc = tc5::idesc_tf32(128, kT5N);
    constexpr uint32_t kALbo = 16 * 128, kBLbo = 4 * 128;
    uint32_t phase = 0;
    bool ok = true;

    for (int pc = pbegin + blockIdx.x; pc < pend && ok; pc += gridDim.x) {
        const long long e0 = pp_ptr[pc];
        const int ne = pp_nchild[pc] * P;
        for (int e = tid; e < ne; e += kT5Threads) st[e] = pb[e0 + e];
        if (tid < kT5N) nc[tid] = 0;
        __syncthreads();
        if (warp == 0) {   // groups: a term opens one when its child cone differs from its predecessor's
            int base = 0;
            for (int c0 = 0; c0 < ne; c0 += 32) {
                const int e = c0 + lane;
                const bool open = e < ne && (e == 0 || st[e].child_cone != st[e - 1].child_cone);
                const unsigned m = __ballot_sync(0xffffffffu, open);
                if (open) gstart[base + __popc(m & ((1u << lane) - 1u))] = e;
                base += __popc(m);
            }
            if (lane == 0) { gstart[base] = ne; *ngroups = base; }
        }
        __syncthreads();
        const int G = *ngroups;
        for (int e = tid; e < ne; e += kT5Threads) {   // per node, its (group, term) pairs
            int lo = 0, hi = G - 1;
            while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (gstart[mid] <= e) lo = mid; else hi = mid - 1; }
            const int n = st[e].pt;
            const int slot = atomicAdd(&nc[n], 1);
            if (slot < 4) nl[n * 4 + slot] = make_int2(lo, e);
        }
        __syncthreads();

        for (int g = 0; g < G; ++g) {
            const int gs = gstart[g], nq = gstart[g + 1] - gs;
            const int q = st[gs].child_cone;
            if (tid < nq) {   // the group's interpolation weights (the previous group's MMAs may still run)
                const PropB<float> E = st[gs + tid];
                float Ts[PS], Tt[PA];
                cheb_row<float, PS>(E.s, Ts);
                cheb_row<float, PA>(E.th, Tt);
                float* w = sw + tid * kT5Half;
#pragma unroll
                for (int a = 0; a < PA; ++a)
#pragma unroll
                    for (int s2 = 0; s2 < PS; ++s2) w[a * PS + s2] = Tt[a] * Ts[s2];
#pragma unroll
                for (int p = P; p < kT5Half; ++p) w[p] = 0.f;
            }
            bool done = true;
            if (g > 0) { done = wait_one(tid, bar, phase & 1u); ++phase; }
            if (!__syncthreads_and(done)) { ok = false; break; }   // sw ready, operand tiles free
            // A: row r (real part) = [Re C | -Im C], row 64 + r (imaginary part) = [Im C | Re C]
            const float2* __restrict__ src = coef + (long long)q * P * B;
            for (int i = tid; i < kT5MaxB * (kT5Half / 4); i += kT5Threads) {
                const int r = i & 63, p0 = 4 * (i >> 6);
                float re[4], im[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int p = p0 + j;
                    const float2 c = (r < B && p < P) ? src[(long long)p * B + r] : make_float2(0.f, 0.f);
                    re[j] = c.x; im[j] = c.y;
                }
                st4_split(sm, OFF_AH, OFF_AL, tc5::kmajor_off(128, r, p0), re[0], re[1], re[2], re[3], 1.f);
                st4_split(sm, OFF_AH, OFF_AL, tc5::kmajor_off(128, r, kT5Half + p0), im[0], im[1], im[2], im[3], -1.f);
                st4_split(sm, OFF_AH, OFF_AL, tc5::kmajor_off(128, 64 + r, p0), im[0], im[1], im[2], im[3], 1.f);
                st4_split(sm, OFF_AH, OFF_AL, tc5::kmajor_off(128, 64 + r, kT5Half + p0), re[0], re[1], re[2], re[3], 1.f);
            }
            // B: row n = [Re (f w) | Im (f w)] of node n's term in this group, or zero
            for (int i = tid; i < kT5N * (kT5Half / 4); i += kT5Threads) {
                const int n = i & 31, p0 = 4 * (i >> 5);
                float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
                float fr = 0.f, fi = 0.f;
                if (n < P) {
                    const int cnt = min(nc[n], 4);
                    for (int j = 0; j < cnt; ++j) {
                        const int2 v = nl[n * 4 + j];
                        if (v.x == g) {
                            w = *(const float4*)(sw + (v.y - gs) * kT5Half + p0);
                            fr = st[v.y].wr; fi = st[v.y].wi;
                        }
                    }
                }
                st4_split(sm, OFF_BH, OFF_BL, tc5::kmajor_off(kT5N, n, p0), fr * w.x, fr * w.y, fr * w.z, fr * w.w, 1.f);
                st4_split(sm, OFF_BH, OFF_BL, tc5::kmajor_off(kT5N, n, kT5Half + p0), fi * w.x, fi * w.y, fi * w.z, fi * w.w, 1.f);
            }
            tc5::fence_async_smem();
            tc5::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc5::fence_after_sync();
                issue_3xtf32(tD, sAH, sAL, kALbo, sBH, sBL, kBLbo, kT5K / 8, idesc, g > 0);
                tc5::commit(bar);
            }
        }
        if (!ok) break;
        if (G > 0) {
            bool done = wait_one(tid, bar, phase & 1u);
            ++phase;
            if (!__syncthreads_and(done)) { ok = false; break; }
            tc5::fence_after_sync();
            float v[32];
            tc5::tmem_ld32(tD + lane_base, v);   // row tid: node values (real or imaginary part)
            // A2 = the node values (rows as A, K = node) in the A tiles
#pragma unroll
            for (int k = 0; k < kT5N; k += 4) st4_split(sm, OFF_AH, OFF_AL, tc5::kmajor_off(128, tid, k), v[k], v[k + 1], v[k + 2], v[k + 3], 1.f);
            tc5::fence_async_smem();
            tc5::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc5::fence_after_sync();
                issue_3xtf32(tD2, sAH, sAL, kALbo, sB2H, sB2L, kBLbo, kT5N / 8, idesc, false);
                tc5::commit(bar);
            }
            done = wait_one(tid, bar, phase & 1u);
            ++phase;
            if (!__syncthreads_and(done)) { ok = false; break; }
            tc5::fence_after_sync();
            tc5::tmem_ld32(tD2 + lane_base, v);
            const int part = tid >> 6, r = tid & 63;
            if (r < B) {
                float* out = (float*)(coef + (long long)pc * P * B + r) + part;
#pragma unroll
                for (int c = 0; c < P; ++c) out[(long long)c * B * 2] = v[c];
            }
            tc5::fence_before_sync();
        } else {
            for (int i = tid; i < P * B; i += kT5Threads) coef[(long long)pc * P * B + i] = make_float2(0.f, 0.f);
        }
        __syncthreads();   // the terms, groups and tensor memory are reused by the next parent cone
    }
    if (!ok && tid == 0) {   // a wait on commit (phase - 1) ran out: record it and give those MMAs one more bounded wait
        atomicExch(err, 1);
        tc5::mbar_wait(bar, (phase - 1u) & 1u, kT5WaitCycles);
    }
    tc5::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc5::tmem_dealloc(tmem, 64);
}


// ------------------------------------------------------------------ leaf cones
constexpr int kL5Threads = 256;
constexpr int kL5Src = 16;                   // sources per chunk: K = 32
constexpr int kL5K = 2 * kL5Src;
constexpr int kL5Cones = 5;                  // cones per work item (125 columns of N = 128)
constexpr int kL5N = 128;
constexpr int L5_T = 128 * kL5K * 4;         // 16384: one 128-row tile of one split term
// NS split terms per operand: A tiles at t L5_T, B tiles at (NS + t) L5_T, the mbarrier after them
__host__ __device__ constexpr int l5_off_bar(int NS) { return 2 * NS * L5_T; }
__host__ __device__ constexpr int l5_smem(int NS) { return l5_off_bar(NS) + 16; }
// per thread and source chunk: one density item (right-hand side, 4 sources) and two table items
// (row = (cone, m), 4 sources); the 125 x 4 table items of a chunk take 500 of the 512 slots
constexpr int kL5BItems = 2;

template <int P>
struct LeafChunk {
    float2 a[4], b[kL5BItems][4];
};

template <int P>
__device__ __forceinline__ void leaf_load(LeafChunk<P>& t, int tid, int sb, int n, int s0, int c0, int c1, const long long* __restrict__ leaf_off,
                                          const float2* __restrict__ L, const float2* __restrict__ rho, int B) {
    {
        const int rr = tid & 63, k0 = 4 * (tid >> 6);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int src = sb + k0 + j;
            t.a[j] = (rr < B && src < n) ? rho[(long long)(s0 + src) * B + rr] : make_float2(0.f, 0.f);
        }
    }
#pragma unroll
    for (int q = 0; q < kL5BItems; ++q) {
        const int i = tid + q * kL5Threads;
        const int row = i % (kL5Cones * P), k0 = 4 * (i / (kL5Cones * P));
        const int c = c0 + row / P, m = row % P;
        const bool live = i < kL5Cones * P * 4 && c < c1;
        const float2* Lc = L + (live ? leaf_off[c] : 0);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int src = sb + k0 + j;
            t.b[q][j] = (live && src < n) ? Lc[(long long)src * P + m] : make_float2(0.f, 0.f);
        }
    }
}
// x = sum of NS TF32 terms, each the rounding of what the previous ones left
template <int NS>
__device__ __forceinline__ void split_n(float x, float* t) {
#pragma unroll
    for (int i = 0; i < NS - 1; ++i) { t[i] = tc5::tf32_hi(x); x -= t[i]; }
    t[NS - 1] = tc5::tf32_hi(x);
}
// four values (each split in NS terms, term i of value j at v[j][i]) to tile `base + i L5_T`
template <int NS>
__device__ __forceinline__ void st4_terms(unsigned char* sm, int base, uint32_t off, const float (*v)[NS], float sign) {
#pragma unroll
    for (int i = 0; i < NS; ++i) st4(sm, base + i * L5_T + off, sign * v[0][i], sign * v[1][i], sign * v[2][i], sign * v[3][i]);
}
template <int P, int NS>
__device__ __forceinline__ void leaf_store(const LeafChunk<P>& t, int tid, unsigned char* sm) {
    constexpr int offA = 0, offB = NS * L5_T;
    {
        const int rr = tid & 63, k0 = 4 * (tid >> 6);
        float re[4][NS], im[4][NS];
#pragma unroll
        for (int j = 0; j < 4; ++j) { split_n<NS>(t.a[j].x, re[j]); split_n<NS>(t.a[j].y, im[j]); }
        // rows 2 r = [Re rho | -Im rho], 2 r + 1 = [Im rho | Re rho]
        st4_terms<NS>(sm, offA, tc5::kmajor_off(128, 2 * rr, k0), re, 1.f);
        st4_terms<NS>(sm, offA, tc5::kmajor_off(128, 2 * rr, kL5Src + k0), im, -1.f);
        st4_terms<NS>(sm, offA, tc5::kmajor_off(128, 2 * rr + 1, k0), im, 1.f);
        st4_terms<NS>(sm, offA, tc5::kmajor_off(128, 2 * rr + 1, kL5Src + k0), re, 1.f);
    }
#pragma unroll
    for (int q = 0; q < kL5BItems; ++q) {
        const int i = tid + q * kL5Threads;
        if (i >= kL5Cones * P * 4) continue;
        const int row = i % (kL5Cones * P), k0 = 4 * (i / (kL5Cones * P));
        float re[4][NS], im[4][NS];
#pragma unroll
        for (int j = 0; j < 4; ++j) { split_n<NS>(t.b[q][j].x, re[j]); split_n<NS>(t.b[q][j].y, im[j]); }
        // row (cone, m) = [Re L[src][m] | Im L[src][m]]
        st4_terms<NS>(sm, offB, tc5::kmajor_off(kL5N, row, k0), re, 1.f);
        st4_terms<NS>(sm, offB, tc5::kmajor_off(kL5N, row, kL5Src + k0), im, 1.f);
    }
}
// D_big (+)= A_0 B_0 and D_small (+)= the other term pairs (i, j) with i + j <= NS - 1, the
// smallest first: 2 + 1 MMAs per K step for two terms (3xTF32), 5 + 1 for three.  The tensor
// core's FP32 accumulator rounds each addition toward zero, so its error grows with the number
// of additions into a large value; keeping the large products in their own tile (one addition
// per K step) and the small ones apart, and adding the two tiles in FP32 at read-back, holds the
// result to FP32 accuracy (one tile for all products over 65 sources: about 4x the FP32 error).
template <int NS>
__device__ __forceinline__ void issue_split(uint32_t d_big, uint32_t d_small, uint32_t a0, uint32_t b0, uint32_t tile, uint32_t lbo,
                                            int ksteps, uint32_t idesc, bool accumulate) {
    uint32_t acc = accumulate ? 1u : 0u;
#pragma unroll
    for (int sum = NS - 1; sum >= 1; --sum)
#pragma unroll
        for (int i = 0; i <= sum; ++i) {
            const int j = sum - i;
            for (int ks = 0; ks < ksteps; ++ks) {
                const uint32_t o = ks * 2 * lbo;
                tc5::mma_tf32(d_small, tc5::smem_desc(a0 + i * tile + o, lbo, 128), tc5::smem_desc(b0 + j * tile + o, lbo, 128), idesc,
                              acc);
                acc = 1u;
            }
        }
    acc = accumulate ? 1u : 0u;
    for (int ks = 0; ks < ksteps; ++ks) {
        const uint32_t o = ks * 2 * lbo;
        tc5::mma_tf32(d_big, tc5::smem_desc(a0 + o, lbo, 128), tc5::smem_desc(b0 + o, lbo, 128), idesc, acc);
        acc = 1u;
    }
}

template <int P, int NS>
__global__ void __launch_bounds__(kL5Threads, 2) k_leaf_t5(const int4* __restrict__ items, int nitems, const int* __restrict__ leaf_start,
                                                        const int* __restrict__ leaf_count, const long long* __restrict__ leaf_off,
                                                        const float2* __restrict__ L, const float2* __restrict__ rho, int B,
                                                        float2* __restrict__ coef, int* __restrict__ err) {
    static_assert(kL5Cones * P <= kL5N && kL5Cones * P * 4 <= kL5BItems * kL5Threads, "a work item's table must fit");
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr int OFF_BAR5 = l5_off_bar(NS);
    const uint32_t bar = tc5::smem_u32(sm + OFF_BAR5), tslot = tc5::smem_u32(sm + OFF_BAR5 + 8);
    const uint32_t sA = tc5::smem_u32(sm), sB = tc5::smem_u32(sm + NS * L5_T);
    if (tid == 0) tc5::mbar_init(bar, 1);
    if (warp == 0) tc5::tmem_alloc(tslot, 2 * kL5N);   // large-product tile, then small-product tile
    tc5::fence_before_sync();
    __syncthreads();
    tc5::fence_after_sync();
    const uint32_t tmem = *(volatile uint32_t*)(sm + OFF_BAR5 + 8);
    // read-back: warp w holds accumulator rows 32 (w % 4) .. + 31, columns 64 (w / 4) .. + 63
    const uint32_t tread = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 64 * (warp >> 2);
    const int row = 32 * (warp & 3) + (tid & 31), r = row >> 1, part = row & 1, col0 = 64 * (warp >> 2);
    const uint32_t idesc = tc5::idesc_tf32(128, kL5N);
    constexpr uint32_t kLbo = 16 * 128;
    uint32_t phase = 0;
    bool ok = true;
    for (int it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
        const int4 item = items[it];         // leaf box, first cone, end cone (level-local, at most kL5Cones)
        const int n = leaf_count[item.x], s0 = leaf_start[item.x];
        const int nch = max(1, (n + kL5Src - 1) / kL5Src);
        LeafChunk<P> t;
        leaf_load<P>(t, tid, 0, n, s0, item.y, item.z, leaf_off, L, rho, B);
        for (int ch = 0; ch < nch; ++ch) {
            bool done = true;
            if (ch > 0) { done = wait_one(tid, bar, phase & 1u); ++phase; }
            if (!__syncthreads_and(done)) { ok = false; break; }   // the previous chunk's MMAs have read the tiles
            leaf_store<P, NS>(t, tid, sm);
            tc5::fence_async_smem();
            tc5::fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                tc5::fence_after_sync();
                issue_split<NS>(tmem, tmem + kL5N, sA, sB, L5_T, kLbo, kL5K / 8, idesc, ch > 0);
                tc5::commit(bar);
            }
            if (ch + 1 < nch) leaf_load<P>(t, tid, (ch + 1) * kL5Src, n, s0, item.y, item.z, leaf_off, L, rho, B);
        }
        if (!ok) break;
        const bool done = wait_one(tid, bar, phase & 1u);
        ++phase;
        if (!__syncthreads_and(done)) { ok = false; break; }
        tc5::fence_after_sync();
        // column col = (cone - first cone) * P + m sits at coefficient row first cone * P + col
        const int ncol = (item.z - item.y) * P;
        float* out = (float*)(coef + (long long)item.y * P * B + r) + part;
        const long long cstride = 2ll * B;
#pragma unroll 1
        for (int q = 0; q < 4; ++q) {
            float v[16], v2[16];
            tc5::tmem_ld16(tread + 16 * q, v);
            tc5::tmem_ld16(tread + kL5N + 16 * q, v2);
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] += v2[j];
            const int cb = col0 + 16 * q;
            if (r < B) {
                float* o = out + cb * cstride;
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (cb + j < ncol) o[j * cstride] = v[j];
            }
        }
        tc5::fence_before_sync();
        __syncthreads();   // the accumulators are overwritten by the next item
    }
    if (!ok && tid == 0) {
        atomicExch(err, 1);
        tc5::mbar_wait(bar, (phase - 1u) & 1u, kT5WaitCycles);
    }
    tc5::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc5::tmem_dealloc(tmem, 2 * kL5N);
}

}  // namespace

cudaError_t prop_t5_init_attributes() {
    cudaError_t e = cudaFuncSetAttribute(k_prop_t5<5, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize, T5_SMEM);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_leaf_t5<25, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, l5_smem(2));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_leaf_t5<25, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, l5_smem(3));
    return e;
}

bool launch_leaf_t5(const int4* items, int nitems, const int* leaf_start, const int* leaf_count, const long long* leaf_off,
                    const float2* L, const float2* rho, int Ps, int Pang, int B, float2* coef, int* err, int nsm, int terms,
                    cudaStream_t s) {
    if (Ps != 5 || Pang != 5 || B > kT5MaxB || B <= 0 || (terms != 2 && terms != 3)) return false;
    if (nitems <= 0) return true;
    const int grid = std::min(nitems, 2 * std::max(nsm, 1));
    if (terms == 3)
        k_leaf_t5<25, 3><<<grid, kL5Threads, l5_smem(3), s>>>(items, nitems, leaf_start, leaf_count, leaf_off, L, rho, B, coef, err);
    else
        k_leaf_t5<25, 2><<<grid, kL5Threads, l5_smem(2), s>>>(items, nitems, leaf_start, leaf_count, leaf_off, L, rho, B, coef, err);
    return true;
}

bool launch_prop_t5(int pbegin, int pend, const long long* pp_ptr, const int* pp_nchild, const PropB<float>* pb, int Ps, int Pang,
                    const float* Gsep, int B, float2* coef, int* err, int nsm, cudaStream_t s) {
    if (Ps != 5 || Pang != 5 || B > kT5MaxB || B <= 0) return false;
    if (pend <= pbegin) return true;
    const int grid = std::min(pend - pbegin, 2 * std::max(nsm, 1));
    k_prop_t5<5, 5><<<grid, kT5Threads, T5_SMEM, s>>>(pbegin, pend, pp_ptr, pp_nchild, pb, Gsep, B, coef, err);
    return true;
}

}  // namespace ifgf
