// precond_net.cuh -- the learned right preconditioner: a 1D convolutional network along the
// boundary parameter (device side).
//
// Network (fixed shape): 6 layers of kernel 7 with circular padding along each closed curve.
//   layer 0: 6 features -> 64, ReLU;  layers 1..4: 64 -> 64, ReLU, plus the layer's input
//   (residual connection);  layer 5: 64 -> 2 (no activation).
// Features per point: Re and Im of the residual turned to its canonical phase and over its
// RMS (r e^{-i phi} / sigma, sigma = RMS(r), phi = arg(sum r^2) / 2, so that the map commutes
// with a global phase as A^{-1} does), curvature / k, unit tangent (2), k h (h = the point's
// quadrature weight, the local arc length).  Output o (2 channels): the preconditioner is
// M(r) = 2 r + sigma e^{i phi} (o_0 + i o_1), 2 r being the inverse of the combined field's
// jump term 1/2 I; an untrained (zero) output layer gives M = 2 I and flexible GMRES
// reduces to GMRES.
//
// Layouts.  Activations: [row][C] BF16, where every sample (curve) occupies len + 2 * kHalo
// rows with kHalo = 3 copies of its wrapped neighbours on either side, so the circular
// convolution is a plain one over the padded buffer (halo rows are refilled after every
// layer; outputs at halo rows are discarded).  C is padded to a multiple of 16: 16 for the
// input features, 64 hidden, 16 for the 2-channel output.  Weights for the tensor cores:
// Wt[co][tap * CIN + ci] BF16 (the K index of the implicit GEMM runs over taps then input
// channels), FP32 master copies W[co][tap][ci] for the optimiser.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>

namespace ifgf {

constexpr int kNetLayers = 6;
constexpr int kNetTaps = 7;
constexpr int kHalo = 3;
constexpr int kNetHidden = 64;
constexpr int kNetInPad = 16;     // 6 features padded
constexpr int kNetOutPad = 16;    // 2 outputs padded
constexpr int kNetFeatures = 6;
constexpr int kNetOutputs = 2;
constexpr double kNetBase = 2.0;  // M(r) = kNetBase r + ...: the inverse of the jump term 1/2 I

inline int net_cin(int l) { return l == 0 ? kNetInPad : kNetHidden; }
inline int net_cout(int l) { return l == kNetLayers - 1 ? kNetOutPad : kNetHidden; }

// one convolution over padded rows [0, rows): out[r][co] = act(b[co] + sum_{tap, ci}
// Wt[co][tap * CIN + ci] in[r + tap - 3][ci]) (+ in[r][co] when residual); rows outside
// [0, rows) read as zero.  out_f32 (optional) receives the FP32 values, out_bf (optional) BF16.
// On tcgen05 tensor cores; *err is set when a CTA's bounded wait for its MMAs ran out.
void launch_conv_fwd(const __nv_bfloat16* in, int rows, int cin, const __nv_bfloat16* Wt, const float* bias, int cout,
                     bool relu, bool residual, __nv_bfloat16* out_bf, float* out_f32, int* err, cudaStream_t s);
// the per-device kernel attributes the convolutions need (call on the device before use,
// outside stream capture)
cudaError_t conv_init_attributes();
// refill the halo rows of every sample: seg_start[s] is the first interior row, seg_len[s] its length
void launch_halo(__nv_bfloat16* buf, int C, const int* seg_start, const int* seg_len, int nseg, cudaStream_t s);
// dW[co][tap][ci] and db[co] of one layer from the pre-activation gradient g[row][cout] and the
// layer input x[row][cin], over interior rows only (row_mask[row] = 1); FP32
void launch_conv_wgrad(const __nv_bfloat16* x, const float* g, const unsigned char* row_mask, int rows, int cin, int cout,
                       float* part, float* dW, float* db, cudaStream_t s);
int conv_wgrad_chunks(int rows);
// Wt (forward) and Wb (backward data, taps flipped, in/out swapped) BF16 packs of FP32 W
void launch_net_pack(const float* W, int cin, int cout, __nv_bfloat16* Wt, __nv_bfloat16* Wb, cudaStream_t s);
// AdamW on n parameters (FP32): p -= lr (mhat / (sqrt(vhat) + eps) + wd p)
void launch_adamw(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2, float eps, float wd,
                  int step, cudaStream_t s);

// per-sample RMS of the residual; feature rows; training targets; preconditioner output
void launch_seg_rms(const double2* r, const int* seg_pt, const int* seg_len, int nseg, float* sigma, cudaStream_t s);
void launch_features(const double2* r, const double4* geom, const double* kseg, const float* sigma, const int* pt_row,
                     const int* pt_seg, int npts, __nv_bfloat16* X, cudaStream_t s);
void launch_targets(const double2* r, const double2* e, const float* sigma, const int* pt_row, const int* pt_seg, int npts, float* T,
                    cudaStream_t s);
void launch_combine(const double2* r, const float* O, const float* sigma, const int* pt_row, const int* pt_seg, int npts, double2* z,
                    cudaStream_t s);
// mean squared error of the two output channels over the points (added into *loss), gO = dL/dO
void launch_mse(const float* O, const float* T, const int* pt_row, int npts, float* gO, double* loss, cudaStream_t s);
void launch_add_bf(const __nv_bfloat16* y, const __nv_bfloat16* x, long long n, __nv_bfloat16* out, cudaStream_t s);
void launch_relu_grad(const float* G, const __nv_bfloat16* Y, long long n, float* dpre, __nv_bfloat16* dpre_bf, cudaStream_t s);
void launch_f2bf(const float* a, long long n, __nv_bfloat16* b, cudaStream_t s);
void launch_axpy_f(const float* a, long long n, float* b, cudaStream_t s);
void launch_halo_fold(float* G, int C, const int* seg_start, const int* seg_len, int nseg, cudaStream_t s);

}  // namespace ifgf
