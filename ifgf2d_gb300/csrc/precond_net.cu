// precond_net.cu -- kernels of the learned right preconditioner (see precond_net.cuh).
//
// The convolutions are implicit GEMMs on the fifth-generation tensor cores (tcgen05.mma
// kind::f16, BF16 operands, FP32 accumulation in tensor memory): per CTA M = 128 rows, N = the
// output channels, K = 7 taps x input channels.  The CTA stages its input rows (with the 3-row
// reach on either side) and the packed weight matrix in shared memory in the K-major
// no-swizzle core-matrix layout; because each 8-channel slab of the input tile stores its rows
// contiguously (16 bytes per row), the operand of tap t is the same tile with its descriptor's
// start moved by t rows, so no im2col copy is made.  One thread issues the 7 x CIN/16 MMAs and
// commits them to an mbarrier (bounded wait); the four warps read the accumulator rows back
// from tensor memory for the epilogue (bias, ReLU, residual).  The backward data pass is the same
// kernel on the packed transposed weights (taps flipped, channels swapped).  Weight gradients
// are FP32 sums over rows: per-block partials of a 4 x 4 (co, ci) tile per tap, then a
// reduction.
#include "precond_net.cuh"
#include "tcgen05.cuh"
#include <cstdint>

namespace ifgf {

static inline unsigned nblk_n(long long n, int b) { return (unsigned)((n + b - 1) / b); }

constexpr int kConvRows = 128;                        // rows per CTA: the MMA's M
constexpr int kConvIRows = kConvRows + 2 * kHalo;     // staged input rows
constexpr long long kConvWaitCycles = 2000000000ll;   // about one second at 2 GHz

template <int CIN> __host__ __device__ constexpr int conv_in_bytes() { return kConvIRows * CIN * 2; }
template <int CIN, int COUT> __host__ __device__ constexpr int conv_w_bytes() { return COUT * kNetTaps * CIN * 2; }
// dynamic shared memory per CTA: the tiles, the mbarrier and the TMEM address, and at least 29 KB,
// so that at most 7 CTAs share an SM and their tensor memory (at most 64 columns each) never
// exceeds the SM's 512 columns: tcgen05.alloc never has to wait
template <int CIN, int COUT> __host__ __device__ constexpr int conv_smem() {
    return conv_in_bytes<CIN>() + conv_w_bytes<CIN, COUT>() + 16 > 29 * 1024 ? conv_in_bytes<CIN>() + conv_w_bytes<CIN, COUT>() + 16
                                                                              : 29 * 1024;
}

// instruction descriptor of kind::f16 with BF16 operands: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 in bits 17-22, M / 16 in bits 24-28
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// D (+)= A B^T, K = 16, issued by one thread
__device__ __forceinline__ void mma_bf16_tc(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// out[r][co] = act(bias[co] + sum_{tap, ci} Wt[co][tap * CIN + ci] in[r + tap - 3][ci]) (+ in[r][co])
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv_tc(const __nv_bfloat16* __restrict__ in, int rows,
                                                 const __nv_bfloat16* __restrict__ Wt, const float* __restrict__ bias,
                                                 int relu, int residual, __nv_bfloat16* __restrict__ out_bf,
                                                 float* __restrict__ out_f32, int* __restrict__ err) {
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 256, "K steps of 16, N a multiple of 16");
    constexpr int K = kNetTaps * CIN;
    constexpr uint32_t LBO_A = kConvIRows * 16;          // between the input tile's 8-channel slabs
    constexpr uint32_t LBO_B = (COUT / 8) * 128;         // between the weights' 8-wide K slabs
    constexpr uint32_t TCOLS = COUT < 32 ? 32 : COUT;    // tensor-memory columns (a power of 2, >= 32)
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* s_in = sm;                                          // [CIN/8][IROWS][8] BF16
    unsigned char* s_w = sm + conv_in_bytes<CIN>();                    // [K/8][COUT/8][8][8] BF16
    unsigned char* s_bar = s_w + conv_w_bytes<CIN, COUT>();            // mbarrier, then the TMEM address
    const uint32_t bar = tc5::smem_u32(s_bar), tslot = tc5::smem_u32(s_bar + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long n0 = (long long)blockIdx.x * kConvRows;
    if (tid == 0) tc5::mbar_init(bar, 1);
    if (warp == 0) tc5::tmem_alloc(tslot, TCOLS);
    // input rows n0 - 3 .. n0 + 130 in 16-byte chunks; rows outside [0, rows) are zero
    for (int q = tid; q < kConvIRows * (CIN / 8); q += blockDim.x) {
        const int r = q / (CIN / 8), c8 = q % (CIN / 8);
        const long long gr = n0 - kHalo + r;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gr >= 0 && gr < rows) v = *reinterpret_cast<const uint4*>(in + gr * CIN + c8 * 8);
        *reinterpret_cast<uint4*>(s_in + c8 * LBO_A + r * 16) = v;
    }
    for (int q = tid; q < COUT * (K / 8); q += blockDim.x) {
        const int co = q / (K / 8), k8 = q % (K / 8);
        *reinterpret_cast<uint4*>(s_w + k8 * LBO_B + (co >> 3) * 128 + (co & 7) * 16) =
            *reinterpret_cast<const uint4*>(Wt + (long long)co * K + k8 * 8);
    }
    tc5::fence_async_smem();
    tc5::fence_before_sync();
    __syncthreads();
    tc5::fence_after_sync();
    const uint32_t tmem = *(volatile uint32_t*)(s_bar + 8);
    bool ok = true;
    if (tid == 0) {
        const uint32_t idesc = idesc_bf16(kConvRows, COUT);
        const uint32_t a0 = tc5::smem_u32(s_in), b0 = tc5::smem_u32(s_w);
        uint32_t acc = 0;
#pragma unroll 1
        for (int tap = 0; tap < kNetTaps; ++tap)
#pragma unroll
            for (int c = 0; c < CIN / 16; ++c) {
                const uint32_t a = a0 + 2 * c * LBO_A + tap * 16;                 // rows shifted by the tap
                const uint32_t b = b0 + ((tap * CIN + 16 * c) / 8) * LBO_B;
                mma_bf16_tc(tmem, tc5::smem_desc(a, LBO_A, 128), tc5::smem_desc(b, LBO_B, 128), idesc, acc);
                acc = 1u;
            }
        tc5::commit(bar);
        ok = tc5::mbar_wait(bar, 0, kConvWaitCycles);
    }
    if (!__syncthreads_and(ok)) {
        if (tid == 0) {
            atomicExch(err, 1);
            tc5::mbar_wait(bar, 0, kConvWaitCycles);   // the MMAs in flight, before the memory goes
        }
        tc5::fence_before_sync();
        __syncthreads();
        if (warp == 0) tc5::tmem_dealloc(tmem, TCOLS);
        return;
    }
    tc5::fence_after_sync();
    // warp w reads accumulator rows 32 w .. 32 w + 31 (its tensor-memory lanes): one row per thread
    const int row = 32 * warp + (tid & 31);
    const long long gr = n0 + row;
    const uint32_t tread = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < COUT; c0 += 16) {
        float v[16];
        tc5::tmem_ld16(tread + c0, v);   // warp-collective: every lane loads, then rows past the end skip the stores
        if (gr < rows) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int col = c0 + j;
                float x = v[j] + bias[col];
                if (relu) x = fmaxf(x, 0.f);
                if (residual)   // CIN == COUT
                    x += __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(s_in + (col >> 3) * LBO_A + (row + kHalo) * 16 +
                                                                                   (col & 7) * 2));
                v[j] = x;
            }
            if (out_f32) {
#pragma unroll
                for (int j = 0; j < 16; j += 4)
                    *reinterpret_cast<float4*>(out_f32 + gr * COUT + c0 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            }
            if (out_bf) {
#pragma unroll
                for (int j = 0; j < 16; j += 2)
                    *reinterpret_cast<__nv_bfloat162*>(out_bf + gr * COUT + c0 + j) = __floats2bfloat162_rn(v[j], v[j + 1]);
            }
        }
    }
    tc5::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc5::tmem_dealloc(tmem, TCOLS);
}

__global__ void k_halo(__nv_bfloat16* __restrict__ buf, int C, const int* __restrict__ seg_start, const int* __restrict__ seg_len,
                       int nseg) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = 2LL * kHalo * C;
    if (t >= per * nseg) return;
    const int s = (int)(t / per);
    const int rem = (int)(t % per), hr = rem / C, c = rem % C;
    const long long st = seg_start[s], len = seg_len[s];
    long long dst, src;
    if (hr < kHalo) { dst = st - kHalo + hr; src = st + len - kHalo + hr; }   // left halo <- the segment's tail
    else { dst = st + len + (hr - kHalo); src = st + (hr - kHalo); }          // right halo <- its head
    buf[dst * C + c] = buf[src * C + c];
}

// per block: rows [r0, r0 + kWgRows); thread tile = 4 output channels x 4 input channels of one tap
constexpr int kWgRows = 64;
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv_wgrad(const __nv_bfloat16* __restrict__ x, const float* __restrict__ gpre, int rows,
                                                    float* __restrict__ part) {
    constexpr int XROWS = kWgRows + 2 * kHalo;
    __shared__ float sg[kWgRows][COUT + 1];
    __shared__ float sx[XROWS][CIN + 1];
    const int tid = threadIdx.x;
    const long long r0 = (long long)blockIdx.x * kWgRows;
    for (int q = tid; q < kWgRows * COUT; q += blockDim.x) {
        const int r = q / COUT, c = q % COUT;
        const long long gr = r0 + r;
        sg[r][c] = gr < rows ? gpre[gr * COUT + c] : 0.f;
    }
    for (int q = tid; q < XROWS * CIN; q += blockDim.x) {
        const int r = q / CIN, c = q % CIN;
        const long long gr = r0 - kHalo + r;
        sx[r][c] = (gr >= 0 && gr < rows) ? __bfloat162float(x[gr * CIN + c]) : 0.f;
    }
    __syncthreads();
    constexpr int TCO = COUT / 4, TCI = CIN / 4, NTILE = TCO * TCI * kNetTaps;
    constexpr int NOUT = COUT * kNetTaps * CIN + COUT;
    float* out = part + (long long)blockIdx.x * NOUT;
    for (int tile = tid; tile < NTILE; tile += blockDim.x) {
        const int tap = tile / (TCO * TCI), rem = tile % (TCO * TCI);
        const int co0 = (rem / TCI) * 4, ci0 = (rem % TCI) * 4;
        float a[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) a[i][j] = 0.f;
        for (int r = 0; r < kWgRows; ++r) {
            float gv[4], xv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) gv[i] = sg[r][co0 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) xv[j] = sx[r + tap][ci0 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) a[i][j] = fmaf(gv[i], xv[j], a[i][j]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) out[((long long)(co0 + i) * kNetTaps + tap) * CIN + ci0 + j] = a[i][j];
    }
    for (int c = tid; c < COUT; c += blockDim.x) {
        float s = 0.f;
        for (int r = 0; r < kWgRows; ++r) s += sg[r][c];
        out[COUT * kNetTaps * CIN + c] = s;
    }
}

__global__ void k_reduce_parts(const float* __restrict__ part, int nchunk, int nout, float* __restrict__ dW, float* __restrict__ db,
                               int nw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nout) return;
    float s = 0.f;
    for (int c = 0; c < nchunk; ++c) s += part[(long long)c * nout + i];
    if (i < nw) dW[i] = s;
    else db[i - nw] = s;
}

__global__ void k_net_pack(const float* __restrict__ W, int cin, int cout, __nv_bfloat16* __restrict__ Wt,
                           __nv_bfloat16* __restrict__ Wb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = cout * kNetTaps * cin;
    if (i >= n) return;
    const int co = i / (kNetTaps * cin), rem = i % (kNetTaps * cin), tap = rem / cin, ci = rem % cin;
    const __nv_bfloat16 v = __float2bfloat16_rn(W[i]);
    Wt[i] = v;   // Wt[co][tap * cin + ci]
    if (Wb) Wb[((long long)ci * kNetTaps + (kNetTaps - 1 - tap)) * cout + co] = v;   // Wb[ci][tap' * cout + co]
}

__global__ void k_adamw(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v, long long n,
                        float lr, float b1, float b2, float eps, float wd, float c1, float c2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi; v[i] = vi;
    p[i] -= lr * ((mi * c1) / (sqrtf(vi * c2) + eps) + wd * p[i]);
}

// ------------------------------------------------------------------ features, targets, loss, elementwise
// per sample: sigma = RMS |r| and the canonical phase phi = arg(sum r^2) / 2, stored as
// (sigma, cos phi, sin phi) (block per sample)
__global__ void k_seg_rms(const double2* __restrict__ r, const int* __restrict__ seg_pt, const int* __restrict__ seg_len,
                          float* __restrict__ sigma) {
    const int sg = blockIdx.x;
    const int p0 = seg_pt[sg], n = seg_len[sg];
    double a = 0.0, sr = 0.0, si = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 v = r[p0 + i];
        a += v.x * v.x + v.y * v.y;
        sr += v.x * v.x - v.y * v.y;
        si += 2.0 * v.x * v.y;
    }
    __shared__ double red[3][256];
    red[0][threadIdx.x] = a; red[1][threadIdx.x] = sr; red[2][threadIdx.x] = si;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double rms = sqrt(red[0][0] / (double)(n > 0 ? n : 1));
        const double phi = 0.5 * atan2(red[2][0], red[1][0]);
        sigma[3 * sg] = (float)(rms > 0 ? rms : 1.0);
        sigma[3 * sg + 1] = (float)cos(phi);
        sigma[3 * sg + 2] = (float)sin(phi);
    }
}
// feature rows of every point: [Re, Im of r e^{-i phi} / sigma, kappa / k, tx, ty, k h, 0 ...]
__global__ void k_features(const double2* __restrict__ r, const double4* __restrict__ geom, const double* __restrict__ kseg,
                           const float* __restrict__ sigma, const int* __restrict__ pt_row, const int* __restrict__ pt_seg, int npts,
                           __nv_bfloat16* __restrict__ X) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const int sg = pt_seg[p];
    const float is = 1.f / sigma[3 * sg], c = sigma[3 * sg + 1], sn = sigma[3 * sg + 2];
    const double2 v = r[p];
    const double4 gm = geom[p];   // kappa, tx, ty, h
    const double k = kseg[sg];
    __nv_bfloat16* row = X + (long long)pt_row[p] * kNetInPad;
    float f[kNetInPad];
#pragma unroll
    for (int q = 0; q < kNetInPad; ++q) f[q] = 0.f;
    const float vr = (float)v.x, vi = (float)v.y;
    f[0] = (vr * c + vi * sn) * is; f[1] = (vi * c - vr * sn) * is;
    f[2] = (float)(gm.x / k); f[3] = (float)gm.y; f[4] = (float)gm.z; f[5] = (float)(k * gm.w);
#pragma unroll
    for (int q = 0; q < kNetInPad; q += 2) *reinterpret_cast<__nv_bfloat162*>(row + q) = __floats2bfloat162_rn(f[q], f[q + 1]);
}
// training targets (e - base r) e^{-i phi} / sigma of every point, FP32 [row][2]
__global__ void k_targets(const double2* __restrict__ r, const double2* __restrict__ e, const float* __restrict__ sigma,
                          const int* __restrict__ pt_row, const int* __restrict__ pt_seg, int npts, float* __restrict__ T) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const int sg = pt_seg[p];
    const double is = 1.0 / sigma[3 * sg], c = sigma[3 * sg + 1], sn = sigma[3 * sg + 2];
    const double2 a = r[p], b = e[p];
    const double dr = b.x - kNetBase * a.x, di = b.y - kNetBase * a.y;
    T[(long long)pt_row[p] * 2] = (float)((dr * c + di * sn) * is);
    T[(long long)pt_row[p] * 2 + 1] = (float)((di * c - dr * sn) * is);
}
// z = base r + sigma e^{i phi} (o_0 + i o_1) at every point
__global__ void k_combine(const double2* __restrict__ r, const float* __restrict__ O, const float* __restrict__ sigma,
                          const int* __restrict__ pt_row, const int* __restrict__ pt_seg, int npts, double2* __restrict__ z) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const int sg = pt_seg[p];
    const double s = sigma[3 * sg], c = sigma[3 * sg + 1], sn = sigma[3 * sg + 2];
    const float* o = O + (long long)pt_row[p] * kNetOutPad;
    const double2 v = r[p];
    z[p] = make_double2(kNetBase * v.x + s * (o[0] * c - o[1] * sn), kNetBase * v.y + s * (o[0] * sn + o[1] * c));
}
// mean squared error over the points' two output channels; gO = dL/dO (zero elsewhere)
__global__ void k_mse(const float* __restrict__ O, const float* __restrict__ T, const int* __restrict__ pt_row, int npts,
                      float* __restrict__ gO, float* __restrict__ gO_bf_src, double* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (p < npts) {
        const long long r = pt_row[p];
        const float scale = 2.f / (2.f * (float)npts);
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const float d = O[r * kNetOutPad + c] - T[r * 2 + c];
            l += (double)d * d;
            gO[r * kNetOutPad + c] = scale * d;
        }
    }
    (void)gO_bf_src;
    __shared__ double red[256];
    red[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] / (2.0 * (double)npts));
}
__global__ void k_add_bf(const __nv_bfloat16* __restrict__ y, const __nv_bfloat16* __restrict__ x, long long n,
                         __nv_bfloat16* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16_rn(__bfloat162float(y[i]) + __bfloat162float(x[i]));
}
// dpre = G * (Y > 0) (FP32 and BF16 copies)
__global__ void k_relu_grad(const float* __restrict__ G, const __nv_bfloat16* __restrict__ Y, long long n, float* __restrict__ dpre,
                            __nv_bfloat16* __restrict__ dpre_bf) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = __bfloat162float(Y[i]) > 0.f ? G[i] : 0.f;
    dpre[i] = v;
    dpre_bf[i] = __float2bfloat16_rn(v);
}
__global__ void k_f2bf(const float* __restrict__ a, long long n, __nv_bfloat16* __restrict__ b) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16_rn(a[i]);
}
__global__ void k_axpy_f(const float* __restrict__ a, long long n, float* __restrict__ b) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] += a[i];
}
// gradients that reached halo rows belong to the interior rows they copy: add them there
__global__ void k_halo_fold(float* __restrict__ G, int C, const int* __restrict__ seg_start, const int* __restrict__ seg_len,
                            int nseg) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = 2LL * kHalo * C;
    if (t >= per * nseg) return;
    const int s = (int)(t / per);
    const int rem = (int)(t % per), hr = rem / C, c = rem % C;
    const long long st = seg_start[s], len = seg_len[s];
    long long dst, src;
    if (hr < kHalo) { dst = st - kHalo + hr; src = st + len - kHalo + hr; }
    else { dst = st + len + (hr - kHalo); src = st + (hr - kHalo); }
    G[src * C + c] += G[dst * C + c];
    G[dst * C + c] = 0.f;
}

// ------------------------------------------------------------------ launchers
void launch_conv_fwd(const __nv_bfloat16* in, int rows, int cin, const __nv_bfloat16* Wt, const float* bias, int cout,
                     bool relu, bool residual, __nv_bfloat16* out_bf, float* out_f32, int* err, cudaStream_t s) {
    if (rows <= 0) return;
    const unsigned grid = nblk_n(rows, kConvRows);
    if (cin == 16 && cout == 64) {
        k_conv_tc<16, 64><<<grid, 128, conv_smem<16, 64>(), s>>>(in, rows, Wt, bias, relu, residual, out_bf, out_f32, err);
    } else if (cin == 64 && cout == 64) {
        k_conv_tc<64, 64><<<grid, 128, conv_smem<64, 64>(), s>>>(in, rows, Wt, bias, relu, residual, out_bf, out_f32, err);
    } else if (cin == 64 && cout == 16) {
        k_conv_tc<64, 16><<<grid, 128, conv_smem<64, 16>(), s>>>(in, rows, Wt, bias, relu, residual, out_bf, out_f32, err);
    }
}
void launch_halo(__nv_bfloat16* buf, int C, const int* seg_start, const int* seg_len, int nseg, cudaStream_t s) {
    const long long n = 2LL * kHalo * C * nseg;
    if (n > 0) k_halo<<<nblk_n(n, 256), 256, 0, s>>>(buf, C, seg_start, seg_len, nseg);
}
cudaError_t conv_init_attributes() {
    // dynamic shared memory above 48 KB needs the opt-in (a per-device function attribute)
    cudaError_t e = cudaFuncSetAttribute(k_conv_tc<64, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, conv_smem<64, 64>());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_conv_tc<64, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, conv_smem<64, 16>());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_conv_tc<16, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, conv_smem<16, 64>());
    return e;
}
int conv_wgrad_chunks(int rows) { return (int)nblk_n(rows, kWgRows); }
void launch_conv_wgrad(const __nv_bfloat16* x, const float* g, const unsigned char* /*row_mask*/, int rows, int cin, int cout,
                       float* part, float* dW, float* db, cudaStream_t s) {
    if (rows <= 0) return;
    const int nchunk = conv_wgrad_chunks(rows);
    if (cin == 16 && cout == 64) k_conv_wgrad<16, 64><<<nchunk, 256, 0, s>>>(x, g, rows, part);
    else if (cin == 64 && cout == 64) k_conv_wgrad<64, 64><<<nchunk, 256, 0, s>>>(x, g, rows, part);
    else if (cin == 64 && cout == 16) k_conv_wgrad<64, 16><<<nchunk, 256, 0, s>>>(x, g, rows, part);
    const int nw = cout * kNetTaps * cin, nout = nw + cout;
    k_reduce_parts<<<nblk_n(nout, 256), 256, 0, s>>>(part, nchunk, nout, dW, db, nw);
}
void launch_net_pack(const float* W, int cin, int cout, __nv_bfloat16* Wt, __nv_bfloat16* Wb, cudaStream_t s) {
    const int n = cout * kNetTaps * cin;
    k_net_pack<<<nblk_n(n, 256), 256, 0, s>>>(W, cin, cout, Wt, Wb);
}
void launch_adamw(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps, float wd,
                  int step, cudaStream_t s) {
    const float c1 = 1.f / (1.f - powf(b1, (float)step)), c2 = 1.f / (1.f - powf(b2, (float)step));
    k_adamw<<<nblk_n(n, 256), 256, 0, s>>>(p, g, m, v, n, lr, b1, b2, eps, wd, c1, c2);
}

void launch_seg_rms(const double2* r, const int* seg_pt, const int* seg_len, int nseg, float* sigma, cudaStream_t s) {
    if (nseg > 0) k_seg_rms<<<nseg, 256, 0, s>>>(r, seg_pt, seg_len, sigma);
}
void launch_features(const double2* r, const double4* geom, const double* kseg, const float* sigma, const int* pt_row,
                     const int* pt_seg, int npts, __nv_bfloat16* X, cudaStream_t s) {
    if (npts > 0) k_features<<<nblk_n(npts, 256), 256, 0, s>>>(r, geom, kseg, sigma, pt_row, pt_seg, npts, X);
}
void launch_targets(const double2* r, const double2* e, const float* sigma, const int* pt_row, const int* pt_seg, int npts, float* T,
                    cudaStream_t s) {
    if (npts > 0) k_targets<<<nblk_n(npts, 256), 256, 0, s>>>(r, e, sigma, pt_row, pt_seg, npts, T);
}
void launch_combine(const double2* r, const float* O, const float* sigma, const int* pt_row, const int* pt_seg, int npts, double2* z,
                    cudaStream_t s) {
    if (npts > 0) k_combine<<<nblk_n(npts, 256), 256, 0, s>>>(r, O, sigma, pt_row, pt_seg, npts, z);
}
void launch_mse(const float* O, const float* T, const int* pt_row, int npts, float* gO, double* loss, cudaStream_t s) {
    if (npts > 0) k_mse<<<nblk_n(npts, 256), 256, 0, s>>>(O, T, pt_row, npts, gO, nullptr, loss);
}
void launch_add_bf(const __nv_bfloat16* y, const __nv_bfloat16* x, long long n, __nv_bfloat16* out, cudaStream_t s) {
    if (n > 0) k_add_bf<<<nblk_n(n, 256), 256, 0, s>>>(y, x, n, out);
}
void launch_relu_grad(const float* G, const __nv_bfloat16* Y, long long n, float* dpre, __nv_bfloat16* dpre_bf, cudaStream_t s) {
    if (n > 0) k_relu_grad<<<nblk_n(n, 256), 256, 0, s>>>(G, Y, n, dpre, dpre_bf);
}
void launch_f2bf(const float* a, long long n, __nv_bfloat16* b, cudaStream_t s) {
    if (n > 0) k_f2bf<<<nblk_n(n, 256), 256, 0, s>>>(a, n, b);
}
void launch_axpy_f(const float* a, long long n, float* b, cudaStream_t s) {
    if (n > 0) k_axpy_f<<<nblk_n(n, 256), 256, 0, s>>>(a, n, b);
}
void launch_halo_fold(float* G, int C, const int* seg_start, const int* seg_len, int nseg, cudaStream_t s) {
    const long long n = 2LL * kHalo * C * nseg;
    if (n > 0) k_halo_fold<<<nblk_n(n, 256), 256, 0, s>>>(G, C, seg_start, seg_len, nseg);
}

}  // namespace ifgf
