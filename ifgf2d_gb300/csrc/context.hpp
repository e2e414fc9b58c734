// context.hpp -- the context behind the C ABI handle, shared by the translation units that
// implement include/ifgf2d.h (ifgf2d_capi.cu: set-up, single apply, GMRES; batch.cu: batched
// apply and solve).  Internal: nothing outside the library sees these types.
#pragma once
#include "../../include/ifgf2d.h"
#include "geometry.hpp"
#include "tree.hpp"
#include "ifgf2d_kernels.cuh"

#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <complex>
#include <functional>
#include <memory>
#include <string>
#include <vector>

struct BatchWork;
struct EvalWork;
struct SpectralWork;
constexpr int kTuneLevels = 24;   // levels covered by the launch-shape table
constexpr int kBatchTcLeaf = 1;   // leaf-cone sums (k_leaf_t5)
constexpr int kBatchTcProp = 2;   // propagation (k_prop_t5)
constexpr int kBatchTcLeaf6 = 4;  // leaf-cone sums with three TF32 terms per operand (6 products)
constexpr int kBatchBulkProp = 8; // FP32 FMA propagation with TMA-staged child coefficients (k_prop_bk)
constexpr int kBatchGroupedInterp = 16;   // interpolation grouped by cone per leaf box (k_interp_grp)
constexpr int kSingleInterpBox64 = 32;    // single vector, FP64: interpolation by leaf box (k_interp_box)
constexpr int kSingleInterpBox32 = 64;    // single vector, complex64: interpolation by leaf box
constexpr int kKernelBits = kBatchTcLeaf | kBatchTcProp | kBatchTcLeaf6 | kBatchBulkProp | kBatchGroupedInterp |
                            kSingleInterpBox64 | kSingleInterpBox32;

namespace ifgf {

// The allocation stream of the calling thread.  While an AllocStream guard names a stream,
// DBuf allocates and frees stream-ordered on it (cudaMallocAsync / cudaFreeAsync from the
// device's memory pool, no device-wide synchronisation) and uploads with cudaMemcpyAsync, so
// threads that set up or tear down contexts do not stall one another's streams; otherwise it uses
// cudaMalloc / cudaFree / cudaMemcpy.  A buffer remembers how and on which stream it was
// allocated and is freed the same way, on that stream (which must outlive it).
inline cudaStream_t& alloc_stream() {
    static thread_local cudaStream_t s = nullptr;
    return s;
}
struct AllocStream {
    cudaStream_t prev;
    explicit AllocStream(cudaStream_t s) : prev(alloc_stream()) { alloc_stream() = s; }
    ~AllocStream() { alloc_stream() = prev; }
    AllocStream(const AllocStream&) = delete;
    AllocStream& operator=(const AllocStream&) = delete;
};
// keep freed stream-ordered memory in the device's pool for reuse (once per process and device)
void keep_pool_memory(int device);
// pinned host scratch of the calling thread (at least n elements; grown, never shrunk, kept for
// the thread's life): the Hessenberg columns a solve reads back.  A thread runs one solve at a
// time, so its contexts share it, and no context pays for pinning and unpinning memory (which
// synchronises the device) at set-up and tear-down.
double2* pinned_scratch(size_t n);

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t owner = nullptr;   // non-null: allocated stream-ordered on this stream
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void release() {
        if (p) {
            if (owner) cudaFreeAsync(p, owner);
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
        owner = nullptr;
    }
    cudaError_t alloc(size_t cnt) {
        release();
        n = cnt;
        if (cnt == 0) return cudaSuccess;
        if (cudaStream_t s = alloc_stream()) {
            owner = s;
            return cudaMallocAsync((void**)&p, cnt * sizeof(T), s);
        }
        return cudaMalloc((void**)&p, cnt * sizeof(T));
    }
    cudaError_t upload(const T* src, size_t cnt) {
        cudaError_t e = alloc(cnt);
        if (e != cudaSuccess || cnt == 0) return e;
        if (owner) return cudaMemcpyAsync(p, src, cnt * sizeof(T), cudaMemcpyHostToDevice, owner);
        return cudaMemcpy(p, src, cnt * sizeof(T), cudaMemcpyHostToDevice);
    }
    cudaError_t upload(const std::vector<T>& v) { return upload(v.data(), v.size()); }
};

}  // namespace ifgf

using namespace ifgf;

// GMRES workspace of a context: Krylov basis, Arnoldi state and one captured iteration graph
// per apply mode.  Kept across solves; rebuilt when the restart length or the tables change.
struct GmresWork {
    DBuf<double2> V, w, h, t, H, y, vin, part;
    // the solve's own vectors (right-hand side, solution, refinement residual, correction,
    // product, one scalar), kept so that a solve after the first allocates and frees nothing:
    // cudaFree synchronises the device, which would serialise contexts solving concurrently
    DBuf<double2> sb, sx, sr, sd, st, shb;
    long long sn = 0;
    // flexible GMRES with the learned preconditioner: z_j = M(v_j) for every column, and the
    // preconditioner's output buffer the captured iteration writes before copying it into Z
    DBuf<double2> Z, zt, zt2, zt3;   // zt2, zt3: the network's output and its weighting, when it corrects the spectral preconditioner
    DBuf<double> nrm2;
    DBuf<int> jdev;
    // least squares on the device (LsqDev): rotated columns, rotated right-hand side, rotations,
    // cycle state
    DBuf<double2> lsR, lsg, lsgs;
    DBuf<double> lsgc, lssc;
    DBuf<int> lsst;
    long long n = 0;
    int m = 0;
    // mode x preconditioner (none, network, spectral, spectral corrected by the network)
    cudaGraphExec_t exec[12] = {};
    cudaGraphExec_t apply_exec[3] = {nullptr, nullptr, nullptr};   // per mode: one apply, vin -> vout
    void drop_graphs() {
        for (auto& e : exec) if (e) { cudaGraphExecDestroy(e); e = nullptr; }
        for (auto& e : apply_exec) if (e) { cudaGraphExecDestroy(e); e = nullptr; }
    }
    ~GmresWork() { drop_graphs(); }
};


struct ifgf2d_ctx {
    Discretisation D;
    ifgf2d_options opt{};
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    double k = 0.0;
    bool device_ready = false, precomputed = false, ifgf_ready = false;
    std::vector<int> h_nsp_ptr, h_nsp, h_srow_ptr, h_srow_col;
    int nlevels = 0;
    // launch shapes per precision (0 FP64, 1 complex64): leaf-kernel source chunks, and cones
    // per block of each level's propagation (0 = the most that fit 256 threads); set by
    // ifgf2d_autotune / ifgf2d_set_tuning
    int tune_leaf[2] = {5, 5};      // complex64 also 0: the table streamed by TMA bulk copies (k_leaf_tma)
    int tune_prop[2][kTuneLevels] = {};
    // kernel choices (bit mask): batched complex64 kernels on the tcgen05 tensor cores in 3xTF32
    // (else FP32 FMA), the batched grouped interpolation, the single-vector interpolation by box
    int tune_batch_tc = kBatchTcLeaf | kBatchGroupedInterp | kSingleInterpBox32;
    // a host-side tree from ifgf2d_prepare waiting for ifgf2d_setup (same k and request)
    bool prep_ready = false;
    double prep_k = 0.0;
    int prep_request = 0, prep_nlevels = 0;
    int form = IFGF2D_SINGLE_LAYER;
    double eta = 0.0;               // coupling of the combined formulation, resolved at precompute
    // geometry (original order)
    DBuf<double> x, y, nx, ny, wq, edge;
    DBuf<int> patch_of;
    DBuf<DevCurve> curves;
    DBuf<DevPatch> patches;
    DBuf<double> nsn, nsw;
    DBuf<int> nsp_ptr, nsp;        // per point: patches it is near-singular to
    // rectangular-polar correction
    std::vector<RPColumn> hcols;
    std::vector<int> col_ptr;      // per patch: first column
    DBuf<RPColumn> cols;
    DBuf<double2> M, W;
    DBuf<int> srow_ptr, srow_col;
    // IFGF tree
    Tree T;
    DBuf<long long> sorting, inverse;
    DBuf<double> xs_s, ys_s, nxs_s, nys_s;
    DBuf<int> patch_s, nsp_ptr_s, nsp_s;
    DBuf<int> leaf_start, leaf_count, point_leaf, nbr_ptr, nbr_box;
    DBuf<long long> near_off;
    DBuf<double2> near;
    DBuf<int> leaf_cone_box;
    DBuf<long long> leaf_off;
    DBuf<LeafNode> leaf_nodes_d;
    DBuf<double2> leafL;
    DBuf<long long> pp_ptr;
    DBuf<int> pp_nchild;
    DBuf<PropEntryD> pp;
    DBuf<int> ip_ptr;
    DBuf<InterpEntryD> ip;
    DBuf<double2> coef;
    DBuf<double> Gm, Gsep;          // full and separable values->coefficients maps
    DBuf<int> near_rowlen;          // per leaf box: sources in its 3x3 neighbourhood
    DBuf<int> near_src_off, near_src;   // per leaf box: the Morton indices of those sources, in row order
    // complex64 copies of the IFGF tables (mixed form)
    DBuf<float2> near32, leafL32, coef32, rho32;
    DBuf<PropE<float>> pp32;
    DBuf<InterpE<float>> ip32;
    DBuf<float> Gsep32;
    // interpolation by leaf box (k_interp_box): work items, the plan box-transposed in both
    // precisions, and the pieces' sums per target
    DBuf<int4> ib_items;
    DBuf<int2> nb_items;            // near field by leaf box (k_near_box): (box, first of up to 32 targets)
    DBuf<InterpE<double>> ipT;
    DBuf<InterpE<float>> ip32T;
    DBuf<double2> ib_part;
    DBuf<float2> ib_part32;
    // work vectors
    DBuf<double2> rho, vin, vout;
    std::unique_ptr<GmresWork> gw;
    BatchWork* bw = nullptr;        // batched apply / solve workspace (batch.cu), freed by destroy
    EvalWork* ew = nullptr;         // off-surface evaluation plan (offsurface.cu), freed by destroy
    SpectralWork* sw = nullptr;     // spectral right preconditioner (spectral_precond.cu), freed by destroy and precompute
    long long counts[8] = {0};
    int last_passes = 0;            // FP64 refinement passes of the last mixed solve (batched: of the batch)
    int nsm = 0;                    // SMs of the context's device
    DBuf<int> kerr;                 // set by a kernel whose bounded wait ran out (checked after synchronisations)
};

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                \
            return IFGF2D_ERR_CUDA;                                                       \
        }                                                                                 \
    } while (0)

static inline int fail(ifgf2d_ctx* ctx, int code, const std::string& msg) { ctx->err = msg; return code; }

// true when all n doubles are finite (host buffers at the C ABI: a NaN or Inf density or
// right-hand side is reported as IFGF2D_ERR_NONFINITE instead of spreading through the solve)
// NaN or Inf anywhere in v[0..n): a double is non-finite exactly when its 11 exponent bits are
// all ones.  The flags are OR-reduced without branches in blocks of 4096, which the compiler
// vectorises; the scan stops after the first block that holds one.
static inline bool all_finite(const double* v, long long n) {
    constexpr uint64_t kExp = 0x7FF0000000000000ull;
    for (long long i0 = 0; i0 < n; i0 += 4096) {
        const long long i1 = n - i0 < 4096 ? n : i0 + 4096;
        uint64_t bad = 0;
        for (long long i = i0; i < i1; ++i) {
            uint64_t b;
            std::memcpy(&b, v + i, sizeof b);
            bad |= (uint64_t)((b & kExp) == kExp);
        }
        if (bad) return false;
    }
    return true;
}

namespace ifgf {
// What a group of obstacles (group.cu) changes in the device part of the IFGF set-up: (k, eta)
// per leaf box and per leaf cone (device arrays), and the leaf-cone nodes and the propagation
// plan, both built member by member.
struct SetupExtra {
    const double2* keta_leafbox = nullptr;
    const double2* keta_leafcone = nullptr;
    std::function<cudaError_t(LeafNode*, cudaStream_t)> build_nodes;
    std::function<cudaError_t(PropE<double>*, PropE<float>*, int*, cudaStream_t)> build_plan;
};
// the host tables of a context built from ctx->D: near-singular patches per point, the
// rectangular-polar columns and rows (ifgf2d_capi.cu)
int init_host_tables(ifgf2d_ctx* ctx);
// the device copies of the discretisation, made on first use (ifgf2d_capi.cu)
int ensure_device_ctx(ifgf2d_ctx* ctx);
// the device tables of an IFGF set-up from ctx->T and ctx->D (ifgf2d_capi.cu); ex for a group
int setup_tables(ifgf2d_ctx* ctx, double k, int nlevels, const SetupExtra* ex);
// single-vector apply on device vectors in original order: y = A x (ifgf2d_capi.cu)
int apply_single(ifgf2d_ctx* ctx, const double2* x, double2* y, int mode);
// batched workspace release (batch.cu)
void free_batch(ifgf2d_ctx* ctx);
// off-surface evaluation plan release (offsurface.cu)
void free_eval(ifgf2d_ctx* ctx);
// the spectral right preconditioner (spectral_precond.cu): set-up of its tables for the context's
// k and coupling (or per curve, for a group of obstacles), with glancing damping
// eps = scale k^(1/3); release; z = M r queued on s (capturable: the tables stay fixed until
// the next set-up)
int spectral_setup(ifgf2d_ctx* ctx, double scale, const double* curve_k = nullptr, const double* curve_eta = nullptr);
void free_spectral(ifgf2d_ctx* ctx);
// which: 0 the preconditioner z = M r, 1 the flat symbol's magnitude |sigma|, 2 its inverse
void spectral_launch(SpectralWork* sw, const double2* r, double2* z, int Np, cudaStream_t s, int which = 0);
// the same for B interleaved vectors (point i of vector b at i * B + b), through a grid buffer
// of B * spectral_grid_size(sw) complex64 values
void spectral_launch_batch(SpectralWork* sw, const double2* r, double2* z, int B, float2* u, int Np, cudaStream_t s, int which = 0);
long long spectral_grid_size(const SpectralWork* sw);
// z += zn - 2 r (the learned network's output zn correcting the spectral preconditioner's z)
void launch_precond_sum(double2* z, const double2* zn, const double2* r, long long n, cudaStream_t s);
// the learned preconditioner on one curve of N points (precond_capi.cu): prepare lays the
// network out for N points with the curve's geometry (host call, synchronous, not capturable);
// launch queues z = M(r) on stream s (capturable; the buffers stay fixed until the next prepare)
int net_prepare_single(ifgf2d_net* net, long long N, const double* geom_host, double k, std::string& err);
// the propagation plan's entries from the tree's slot form, on the device (plan_device.cu):
// FP64 into pp64 and, when pp32 is not null, the complex64 copy; *err is set when a node's child
// cone does not exist (an inconsistent tree).  Under an AllocStream guard on `s` the work stays
// queued on `s`; otherwise the stream is synchronised before returning.  For a member of a group
// of obstacles, level_cone_base[l] replaces level l's first global cone id and
// level_entry_base[l] the first entry of the slots with children at level l.
cudaError_t build_prop_plan(const Tree& T, PropE<double>* pp64, PropE<float>* pp32, int* err, cudaStream_t s,
                            const int* level_cone_base = nullptr, const long long* level_entry_base = nullptr);
// The propagation plan computed level by level while the host builds the tree's cones: after
// each level's cones and slots exist, add() uploads them and launches that level's entries into
// buffers of their own on a stream of its own; gather() copies every level into pp64 / pp32 at
// its entry offset once the plan is allocated, ordered after the work queued so far on `s` and
// before the work queued on `s` next, and copies the error flag (as build_prop_plan's) to *err.
// Errors of add() are kept and returned by gather().
class PropPlanByLevel {
public:
    PropPlanByLevel();
    ~PropPlanByLevel();
    PropPlanByLevel(const PropPlanByLevel&) = delete;
    PropPlanByLevel& operator=(const PropPlanByLevel&) = delete;
    void add(const Tree& T, int level);
    cudaError_t gather(PropE<double>* pp64, PropE<float>* pp32, int* err, cudaStream_t s);
private:
    struct Impl;
    Impl* d;
};
// the leaf-cone interpolation nodes of T (position, 1 / factorization; BoxTree.h:714-745) on the
// device, P per leaf cone in cone order (plan_device.cu); stream handling as build_prop_plan
cudaError_t build_leaf_nodes(const Tree& T, LeafNode* out, cudaStream_t s);
// a parent's propagation terms sorted by child cone (stable), with the parent node recorded, for
// the batched propagation
template <typename R>
void launch_sort_plan(const long long* pp_ptr, int ncones, const PropE<double>* pp, int P, PropB<R>* out, cudaStream_t s);
// the complex64 copy of the interpolation plan
void launch_interp_to_c64(const InterpE<double>* in, long long n, InterpE<float>* out, cudaStream_t s);
void net_precondition_launch(ifgf2d_net* net, const double2* r, double2* z, cudaStream_t s);
// after a synchronisation: IFGF2D_ERR_CUDA (and the flag cleared) when one of the network's
// tensor-core convolutions gave up waiting for its MMAs, else IFGF2D_OK
int net_kernel_error(ifgf2d_net* net);
// the network's output is |sigma|-weighted (ifgf2d_net_set_output_weighting)
bool net_weighted(const ifgf2d_net* net);
// z = a x + b y (z may be x or y)
void launch_axpby(double2* z, double a, const double2* x, double b, const double2* y, long long n, cudaStream_t s);
}  // namespace ifgf
