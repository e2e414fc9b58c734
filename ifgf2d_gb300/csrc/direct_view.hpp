// direct_view.hpp -- read-only view of the context state the direct forward map uses.
#pragma once
#include <cuda_runtime.h>
#include "ifgf2d_kernels.cuh"

struct ifgf2d_ctx;

namespace ifgf {

// Device pointers and sizes of compute_Ax_unacc's operands (ForwardMap.tpp:517-540).
struct DirectView {
    int N = 0, Np = 0, device = 0;
    double k = 0.0;
    cudaStream_t stream = nullptr;
    const double2* W = nullptr;          // folded rectangular-polar weights
    const int* srow_ptr = nullptr;       // per output row: its weight columns
    const int* srow_col = nullptr;
    const RPColumn* cols = nullptr;
    const double* wq = nullptr;          // per-point quadrature factor
    const double* x = nullptr;           // points (original order)
    const double* y = nullptr;
    const int* patch_of = nullptr;
    const int* nsp_ptr = nullptr;        // per point: patches it is near-singular to
    const int* nsp = nullptr;
    const double* nx = nullptr;          // unit normals (original order)
    const double* ny = nullptr;
    int form = 0;                        // IFGF2D_SINGLE_LAYER or IFGF2D_COMBINED
    double eta = 0.0, half = 0.0;        // coupling and jump-term factor
};

// Fills `v` once the rectangular-polar weights are on the device; returns an IFGF2D status
// (IFGF2D_ERR_STATE, with the context's error message set, before that).
int direct_view(ifgf2d_ctx* ctx, DirectView* v);
// Sets the context's error message (ifgf2d_last_error).
void set_error(ifgf2d_ctx* ctx, const char* msg);
// Set-up work of ifgf2d_apply_direct_noalloc on `device` (the current device): resolves its
// scratch array's address and loads its kernels, so that the call allocates nothing.
int noalloc_prepare(int device);

}  // namespace ifgf
