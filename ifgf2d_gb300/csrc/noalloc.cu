// noalloc.cu -- the direct forward map without any device allocation in the call.
//
// ifgf2d_apply_direct_noalloc computes the same y = A x as ifgf2d_apply_device(...,
// IFGF2D_APPLY_DIRECT) on caller-owned device vectors.  The one scratch buffer of that path
// (the quadrature-weighted density, N complex values) lives in a fixed, file-scope device
// array instead of the context's allocation, so the call itself performs no cudaMalloc,
// cudaFree or allocating library call.  It serves callers that cannot allocate device memory
// at the point of the call: a host application or plugin framework that owns the device
// memory budget and forbids driver allocations, or a latency-critical loop that cannot
// afford the implicit synchronisation of cudaMalloc / cudaFree.
//
// Under CUDA's lazy module loading, the module holding the array is loaded (and the array
// allocated) by the first lookup of its address, and each kernel by its first launch or
// attribute query.  Both happen in the context's set-up (noalloc_prepare, called by
// ifgf2d_precompute and so by ifgf2d_setup), never in the call itself.
#include "../../include/ifgf2d.h"
#include "direct_view.hpp"

#include <mutex>

namespace {

// Scratch of ifgf2d_apply_direct_noalloc: IFGF2D_NOALLOC_MAX_N complex values (1 MiB).  Each
// GPU holds it from the set-up of the first context on it until the process exits.  All calls
// share it.
static __device__ __align__(256) double2 g_noalloc_scratch[IFGF2D_NOALLOC_MAX_N];

constexpr int kMaxDevices = 64;
double2* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_lock;

}  // namespace

namespace ifgf {

// Resolves the scratch array's device address on `device` (the current device) with
// cudaGetSymbolAddress, and loads the kernels the entry point launches.  The host-side symbol
// is only a stand-in for the array, so the address is looked up here and cached per device.
// It is looked up again at every set-up, so a set-up after cudaDeviceReset (which frees the
// array and invalidates the cached address) refreshes it.
int noalloc_prepare(int device) {
    if (device < 0 || device >= kMaxDevices) return IFGF2D_OK;   // such a device cannot use the entry point
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return IFGF2D_ERR_CUDA;
    if (preload_direct_kernels() != cudaSuccess || preload_intensities_kernel() != cudaSuccess) return IFGF2D_ERR_CUDA;
    std::lock_guard<std::mutex> guard(g_scratch_lock);
    g_scratch_addr[device] = static_cast<double2*>(p);
    return IFGF2D_OK;
}

}  // namespace ifgf

extern "C" int ifgf2d_apply_direct_noalloc(ifgf2d_ctx* ctx, const void* d_x, void* d_y) {
    if (!ctx || !d_x || !d_y) return IFGF2D_ERR_ARG;
    ifgf::DirectView v;
    int rc = ifgf::direct_view(ctx, &v);
    if (rc != IFGF2D_OK) return rc;
    if (v.N > IFGF2D_NOALLOC_MAX_N) {
        ifgf::set_error(ctx, "ifgf2d_apply_direct_noalloc: N exceeds IFGF2D_NOALLOC_MAX_N (65536 unknowns)");
        return IFGF2D_ERR_ARG;
    }
    int current = -1;
    if (cudaGetDevice(&current) != cudaSuccess) { ifgf::set_error(ctx, "cudaGetDevice failed"); return IFGF2D_ERR_CUDA; }
    if (current != v.device) {
        ifgf::set_error(ctx, "ifgf2d_apply_direct_noalloc: make the context's device current before the call");
        return IFGF2D_ERR_ARG;
    }
    if (v.device < 0 || v.device >= kMaxDevices) {
        ifgf::set_error(ctx, "ifgf2d_apply_direct_noalloc: supports device ordinals 0 to 63");
        return IFGF2D_ERR_ARG;
    }
    double2* rho = nullptr;
    {
        std::lock_guard<std::mutex> guard(g_scratch_lock);
        rho = g_scratch_addr[v.device];
    }
    if (!rho) {
        ifgf::set_error(ctx, "ifgf2d_apply_direct_noalloc: no set-up on this device resolved the scratch array");
        return IFGF2D_ERR_STATE;
    }
    const double2* x = static_cast<const double2*>(d_x);
    double2* y = static_cast<double2*>(d_y);
    // every entry of the scratch is rewritten by the intensities kernel before it is read
    ifgf::launch_sing_apply(x, v.W, v.srow_ptr, v.srow_col, v.cols, v.N, v.Np, v.half, y, v.stream);
    ifgf::launch_intensities(x, v.wq, nullptr, v.N, rho, v.stream);
    ifgf::launch_direct_far(v.x, v.y, v.N, v.patch_of, v.nsp_ptr, v.nsp, v.x, v.y, v.nx, v.ny, v.patch_of, rho, v.N, v.k,
                            v.form, v.eta, y, 1, v.stream);
    if (cudaGetLastError() != cudaSuccess) { ifgf::set_error(ctx, "kernel launch failed"); return IFGF2D_ERR_CUDA; }
    return IFGF2D_OK;
}
