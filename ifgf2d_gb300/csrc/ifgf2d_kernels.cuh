// ifgf2d_kernels.cuh -- device data layouts and kernel launchers of the forward map.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace ifgf {

// Curve on the device (twin of HostCurve, Geometry/Curve.hpp:106-161)
struct DevCurve {
    int type;
    int pad;
    double p[16];
};

// One rectangular-polar column: a target point (singular or near-singular) on a patch
struct RPColumn {
    int patch;
    int pad;
    double tsing, xs, ys;
};

struct DevPatch {
    double t1, t2;
    int curve, ist1, ist2, pad;
};

// Leaf cone interpolation node: position and 1/(e^{ikr}/sqrt r) at the node radius
struct LeafNode {
    double x, y;
    double ir, ii;
};

// complex vector type of a real type
template <typename R> struct Cx;
template <> struct Cx<double> { using V = double2; };
template <> struct Cx<float> { using V = float2; };
template <typename R> using V2 = typename Cx<R>::V;

// one (target, level, cousin) interpolation term: cone id, Chebyshev (s, theta), e^{ikr}/sqrt r
template <typename R> struct InterpE;
template <> struct InterpE<double> { int cone; int pad; double s, th, fr, fi; };
template <> struct InterpE<float> { int cone; float s, th, fr, fi; };
// batched complex64 interpolation term, grouped by leaf box and cone: cone id, Morton target,
// (s, theta), factor
struct InterpG { int cone; int t; float s, th, fr, fi; };
// one (parent cone, child, node) propagation term: child cone id, (s, theta), factor ratio
template <typename R> struct PropE;
template <> struct PropE<double> { int child_cone; int pad; double s, th, wr, wi; };
template <> struct PropE<float> { int child_cone; float s, th, wr, wi; };
// batched propagation term: the parent node pt it feeds, then as PropE.  A parent's terms are
// sorted by child cone, so a warp loads each child cone's coefficients once per parent.
template <typename R> struct PropB;
template <> struct PropB<double> { int child_cone; int pt; double s, th, wr, wi; };
template <> struct PropB<float> { int child_cone; int pt; float s, th, wr, wi; };
using InterpEntryD = InterpE<double>;
using PropEntryD = PropE<double>;

constexpr int kMaxP = 64;          // Ps * Pang limit of the device interpolator

// ---------------- setup kernels ----------------
// keta, when given, holds (k, eta) per item (per column, leaf box or leaf cone) and overrides the
// scalar k and eta: a group of obstacles with their own wavenumbers sets up in one launch.
void launch_rp_precompute(const RPColumn* cols, int ncols, const DevPatch* patches, const DevCurve* curves,
                          const double* ns_nodes, const double* ns_weights, int Np, double p, double k,
                          int form, double eta, double2* M, cudaStream_t s, const double2* keta = nullptr);
void launch_rp_fold(const double2* M, const RPColumn* cols, int ncols, const double* edge_jac, const DevPatch* patches,
                    int Np, double2* W, cudaStream_t s);
void launch_near_setup(const int* leaf_start, const int* leaf_count, const int* nbr_ptr, const int* nbr_box,
                       const long long* near_off, int nleaf, const double* xs, const double* ys,
                       const double* nxs, const double* nys, const int* patch_s, const int* nsp_ptr,
                       const int* nsp, double k, int form, double eta, double2* near, cudaStream_t s,
                       const double2* keta = nullptr);
// leaf-cone tables: Green values at the cone nodes times 1/factorization, mapped to Chebyshev
// coefficients with the separable map Gsep (Ps x Ps radial, then Pang x Pang angular);
// Ps * Pang <= 64
void launch_leaf_setup(const int* cone_box, int ncones, const int* leaf_start, const int* leaf_count,
                       const long long* leaf_off, const LeafNode* nodes, const double* xs, const double* ys,
                       const double* nxs, const double* nys, int Ps, int Pang, double k, int form, double eta,
                       const double* Gsep, double2* L, cudaStream_t s, const double2* keta = nullptr);

// ---------------- per-apply kernels ----------------
// y = singular correction (+ half * x: the jump term of the combined formulation)
void launch_sing_apply(const double2* x, const double2* W, const int* row_ptr, const int* row_col,
                       const RPColumn* cols, int N, int Np, double half, double2* y, cudaStream_t s);
// the same, also writing the quadrature-weighted density to rho64 or rho32 at inv[o] (or o)
void launch_sing_intens(const double2* x, const double2* W, const int* row_ptr, const int* row_col,
                        const RPColumn* cols, int N, int Np, double half, double2* y, const double* wq,
                        const long long* inv, double2* rho64, float2* rho32, cudaStream_t s);
// sources with unit normals snx, sny (NULL for the single layer); form 0 single layer, 2 combined
void launch_direct_far(const double* tx, const double* ty, int ntarget, const int* t_patch, const int* t_nsp_ptr,
                       const int* t_nsp, const double* sx, const double* sy, const double* snx, const double* sny,
                       const int* s_patch, const double2* rho, int nsource, double k, int form, double eta, double2* y,
                       int accumulate, cudaStream_t s);

// precision-templated IFGF apply (ifgf_apply.cu); R = double (plain) or float (mixed)
template <typename R>
void launch_intensities_t(const double2* x, const double* wq, const long long* perm, int N, V2<R>* rho, cudaStream_t s);
template <typename R>
void launch_leaf_apply_t(const int* cone_box, int ncones, int cone_base, const int* leaf_start, const int* leaf_count,
                         const long long* leaf_off, const V2<R>* L, const V2<R>* rho, int P, V2<R>* coef, cudaStream_t s,
                         int chunks = 5);
// complex64 leaf cones with the table streamed through shared memory by TMA bulk copies
// (P = 25); false when not launched (other P, or leaf_tma_init not run).  *err is set when a
// completion wait runs out.  leaf_tma_init sets the kernel's shared-memory attribute (outside
// stream capture).  The table array must carry 16 bytes of padding after its end.
bool launch_leaf_tma(const int* cone_box, int ncones, int cone_base, const int* leaf_start, const int* leaf_count,
                     const long long* leaf_off, const float2* L, const float2* rho, int P, float2* coef, int* err, int nsm,
                     cudaStream_t s);
cudaError_t leaf_tma_init();
// the propagation variant that stages child coefficient blocks in shared memory (k_propagate_st);
// other values of cones_per_block: 2, 4, or 0 for the most that fit 256 threads
constexpr int kPropStaged = 1;
template <typename R>
void launch_propagate_t(int pbegin, int pend, const long long* pp_ptr, const int* pp_nchild, const PropE<R>* pp, int Ps,
                        int Pang, const R* Gsep, V2<R>* coef, cudaStream_t s, int cones_per_block = 0);
// with `part`, the interpolation terms were summed by launch_interp_box: the near field plus each
// target's pieces in order
template <typename R>
void launch_final_t(int N, const int* point_leaf, const int* leaf_start, const int* near_src_off, const int* near_src,
                    const int* near_rowlen, const long long* near_off, const V2<R>* near,
                    const V2<R>* rho, const int* ip_ptr, const InterpE<R>* ip, const V2<R>* coef, int Ps, int Pang,
                    const long long* sorting, double2* y, cudaStream_t s, const V2<R>* part = nullptr);
// interpolation by leaf box (k_interp_box): items[w] = (leaf box, first target, first term, end
// term), pieces of kIbPiece terms; part[piece * N + target] receives each piece's sum
constexpr int kIbPiece = 8;
template <typename R>
void launch_interp_box(const int4* items, int nitems, int N, const int* leaf_start, const int* leaf_count, const int* ip_ptr,
                       const InterpE<R>* ipT, const V2<R>* coef, int Ps, int Pang, V2<R>* part, cudaStream_t s);
// near field by leaf box (k_near_box): items[w] = (leaf box, first of up to 32 targets); adds the
// near field, then the target's interpolation pieces (when part is not null), into y
constexpr int kNearChunk = 1024, kNearTargets = 32;
template <typename R>
void launch_near_box(const int2* items, int nitems, const int* leaf_start, const int* leaf_count, const int* near_src_off,
                     const int* near_src, const int* near_rowlen, const long long* near_off, const V2<R>* near, const V2<R>* rho,
                     const int* ip_ptr, const V2<R>* part, int N, const long long* sorting, double2* y, cudaStream_t s);
// the interpolation plan box-transposed (term j of box target t at the box's first entry + j n + t)
template <typename R>
void launch_interp_transpose(int N, const int* point_leaf, const int* leaf_start, const int* leaf_count, const int* ip_ptr,
                             const InterpE<double>* in, InterpE<R>* out, cudaStream_t s);
void launch_d2f(const double2* a, long long n, float2* b, cudaStream_t s);
// Load the direct map's kernels (singular correction, FP64 intensities, both far-sum shapes) into
// the current device's context now.  Under lazy module loading a kernel is otherwise loaded,
// with a device allocation for its code, on its first launch.
cudaError_t preload_direct_kernels();
cudaError_t preload_intensities_kernel();
// direct path intensities (patch order), as in ForwardMap::compute_intensities
inline void launch_intensities(const double2* x, const double* wq, const long long* perm, int N, double2* rho, cudaStream_t s) {
    launch_intensities_t<double>(x, wq, perm, N, rho, s);
}

// ---------------- batched apply (ifgf_batch.cu) ----------------
// A batch of B right-hand sides is held interleaved, [N][B] (RHS index fastest); cone
// coefficients likewise [cone][P][B].  One warp serves 32 right-hand sides of one row, cone or
// target, so every table entry is read once per 32 right-hand sides.
constexpr int kMaxBatch = 64;      // right-hand sides per batched apply (larger batches are chunked)
void launch_interleave(const double2* x, long long N, int B, double2* xt, cudaStream_t s);     // [B][N] -> [N][B]
void launch_deinterleave(const double2* xt, long long N, int B, double2* x, cudaStream_t s);   // [N][B] -> [B][N]
// rho32 given: the mixed form (complex64 densities xt32 and weights W32, FP32 sums); else FP64
// with xt and W.  The jump term and the intensities use xt.
void launch_sing_b(const double2* xt, const float2* xt32, const double2* W, const float2* W32, const int* row_ptr,
                   const int* row_col, const RPColumn* cols, int N, int Np, int B, double half, double2* yt,
                   const double* wq, const long long* inv, double2* rho64, float2* rho32, cudaStream_t s);
template <typename R>
void launch_leaf_b(const int* cone_box, int ncones, int cone_base, const int* leaf_start, const int* leaf_count,
                   const long long* leaf_off, const V2<R>* L, const V2<R>* rho, int Ps, int Pang, int B, V2<R>* coef,
                   cudaStream_t s);
// rows (optional): the terms' Chebyshev rows from launch_plan_rows, read instead of computed
template <typename R>
void launch_prop_b(int pbegin, int pend, const long long* pp_ptr, const int* pp_nchild, const PropB<R>* pb, int Ps, int Pang,
                   const R* Gsep, int B, V2<R>* coef, cudaStream_t s, const R* rows = nullptr);
// the Chebyshev rows T_0..T_{Ps-1}(s), T_0..T_{Pang-1}(th) of n batched plan terms, [term][Ps + Pang]
template <typename R>
void launch_plan_rows(const PropB<R>* pb, long long n, int Ps, int Pang, R* rows, cudaStream_t s);
// the complex64 propagation on the tcgen05 tensor cores in 3xTF32 (batch_tcgen05.cu); false when
// the shape is not supported (Ps x Pang other than 5 x 5, more than 64 right-hand sides) and
// nothing was launched.  *err is set when a completion wait runs out.  The kernel's shared-memory
// attribute must be set once per device (prop_t5_init_attributes), outside stream capture.
bool launch_prop_t5(int pbegin, int pend, const long long* pp_ptr, const int* pp_nchild, const PropB<float>* pb, int Ps, int Pang,
                    const float* Gsep, int B, float2* coef, int* err, int nsm, cudaStream_t s);
// the complex64 leaf-cone sums on the tcgen05 tensor cores in 3xTF32: items[i] = (leaf box, first
// cone, end cone, 0), at most kLeafT5Cones cones, indices local to the leaf level; coef offset to
// the level's first cone
constexpr int kLeafT5Cones = 5;
// terms = 2: 3xTF32 (each operand hi + lo, 3 products); terms = 3: three TF32 terms per operand
// and 6 products, FP32-level operands
bool launch_leaf_t5(const int4* items, int nitems, const int* leaf_start, const int* leaf_count, const long long* leaf_off,
                    const float2* L, const float2* rho, int Ps, int Pang, int B, float2* coef, int* err, int nsm, int terms,
                    cudaStream_t s);
cudaError_t prop_t5_init_attributes();
// the complex64 FMA propagation with each child cone's coefficient block staged in shared memory
// by a TMA bulk copy one group ahead; false when the shape is not supported (Ps x Pang other
// than 5 x 5, B odd or above 64) and nothing was launched
// yt[sorting[t]] += the cousin-cone interpolation of the targets of each work item
// items[i] = (first term, end term, first Morton target, targets <= kInterpGrpTargets), terms
// sorted by cone within an item; complex64 coefficients [cone][P][B], B <= 64
constexpr int kInterpGrpTargets = 8;
bool launch_interp_grp(const int4* items, int nitems, const InterpG* terms, const float2* coef, int Ps, int Pang,
                       const long long* sorting, int B, double2* yt, cudaStream_t s);
bool launch_prop_bk(int pbegin, int pend, const long long* pp_ptr, const int* pp_nchild, const PropB<float>* pb, int Ps, int Pang,
                    const float* Gsep, int B, float2* coef, int* err, cudaStream_t s);
template <typename R>
void launch_final_b(int N, const int* point_leaf, const int* leaf_start, const int* leaf_count, const int* nbr_ptr,
                    const int* nbr_box, const int* near_rowlen, const long long* near_off, const V2<R>* near,
                    const V2<R>* rho, const int* ip_ptr, const InterpE<R>* ip, const V2<R>* coef, int Ps, int Pang,
                    const long long* sorting, int B, double2* yt, cudaStream_t s);
// batched GMRES helpers on interleaved [N][B] vectors; column c of a basis starts at V + c * ldc
int bdot_chunks(long long N);
// h[c][r] = sum_i conj(V_c[i][r]) w[i][r] for c < ncols; Hcol[c][r] = h (add: +=).  With
// sqrt_row >= 0 (ncols = 1, V = w): Hcol[sqrt_row][r] = sqrt(sum_i |w[i][r]|^2) instead.
void launch_bdot(const double2* V, long long ldc, int ncols, const double2* w, long long N, int B, double2* part,
                 double2* h, double2* Hcol, int add, int sqrt_row, cudaStream_t s);
// w[i][r] += sign * sum_{c < ncols} V_c[i][r] h[c][r]
void launch_bupdate(const double2* V, long long ldc, int ncols, const double2* h, double sign, long long N, int B, double2* w,
                    cudaStream_t s);
// out[i][r] = w[i][r] / hn[r].x, 0 where hn[r] = 0
void launch_bscale(const double2* w, const double2* hn, long long N, int B, double2* out, cudaStream_t s);

// ---------------- tests / GMRES helpers ----------------
void launch_hankel(int order, const double* x, int n, double2* out, cudaStream_t s);
void launch_multidot(const double2* V, long long ldv, int ncols, const double2* w, long long n, double2* h, cudaStream_t s);
void launch_multi_axpy(const double2* V, long long ldv, int ncols, const double2* h, double sign, long long n, double2* w, cudaStream_t s);
void launch_scale(const double2* w, double2 a, long long n, double2* out, cudaStream_t s);
void launch_sub(const double2* a, const double2* b, long long n, double2* out, cudaStream_t s);
// out[i][j] = in[i][act[j]] for an interleaved in [N][B] and a compact out [N][Bc], and back
// (out[i][act[j]] (+)= in[i][j])
void launch_gather_cols(const double2* in, int B, const int* act, int Bc, long long N, double2* out, cudaStream_t s);
void launch_scatter_cols(const double2* in, int Bc, const int* act, int B, long long N, bool add, double2* out, cudaStream_t s);
void launch_nonfinite_check(const double2* v, long long n, int* flag, cudaStream_t s);
// ---------------- GMRES least squares on the device (gmres_device.cu) ----------------
// One right-hand side: R (ldh x m, column-major) the Hessenberg columns rotated to upper
// triangular form, g (m + 1) the rotated right-hand side, gc / gs (m) the rotations, st the
// cycle state [stopped, columns, iteration limit, iterations], sc [estimate, ||r0||, tol].
struct LsqDev {
    double2* R; double2* g; double* gc; double2* gs; int* st; double* sc; int m;
};
// B right-hand sides, each with the arrays of LsqDev at offsets r * ldh * m (R), r * (m + 1) (g),
// r * m (gc, gs), 4 r (st), 3 r (sc)
struct LsqBatchDev {
    double2* R; double2* g; double* gc; double2* gs; int* st; double* sc; int m; int B;
};
// a restart cycle starts: g = beta e_1, j = 0, limit iterations allowed
void launch_lsq_init(LsqDev L, int* jp, double beta, double r0n, double tol, int limit, cudaStream_t s);
// after the Arnoldi step of column j = *jp: rotate it into R, update g and the estimate
// |g_{j+1}| / ||r0||, stop on convergence, the limit or a breakdown, j += 1; with use_cond, set
// the condition of the graph while-loop around the iteration (0 ends the cycle)
void launch_lsq_givens(const double2* H, int ldh, int* jp, LsqDev L, cudaGraphConditionalHandle cond, bool use_cond,
                       cudaStream_t s);
// y = R^{-1} g over the cycle's columns (st[1])
void launch_lsq_solve(LsqDev L, int ldh, double2* y, cudaStream_t s);
// w += sum_{c < *ncols} V[:, c] y[c]
void launch_multi_axpy_dyn(const double2* V, long long ldv, const int* ncols, const double2* y, long long n, double2* w,
                           cudaStream_t s);
// batched: init from per-RHS norms beta[r].x and par[3 r ..] = (||r0||, tol, iteration limit; <= 0 frozen)
void launch_lsq_init_batch(LsqBatchDev L, const double2* beta, const double* par, cudaStream_t s);
// column j (host index) of every running right-hand side, Hcol[i * B + r]; active[j] = how many still run
void launch_lsq_givens_batch(const double2* Hcol, int j, LsqBatchDev L, int* active, cudaStream_t s);
// Y[i * B + r] = (R_r^{-1} g_r)_i, zero from the right-hand side's own column count up to ncols
void launch_lsq_solve_batch(LsqBatchDev L, int ncols, double2* Y, cudaStream_t s);
// the same Givens step with j = *jp read on the device (H: columns of (m + 1) * B entries), for a
// captured iteration: active[j] = the right-hand sides still running, j += 1, and the while-loop
// condition set to 0 once none runs or the cycle is full
void launch_lsq_givens_batch_dev(const double2* H, int* jp, LsqBatchDev L, int* active, cudaGraphConditionalHandle cond,
                                 cudaStream_t s);
// Segmented vectors: B segments side by side in vectors of n entries (one per obstacle of a
// group).  Chunk c covers [chunk_lo[c], chunk_lo[c + 1]) inside one segment; segment s owns
// chunks [seg_chunk[s], seg_chunk[s + 1]); seg_of[i] is the segment of entry i; part holds
// (m + 1) * nchunk partial sums.
struct SegDesc {
    long long n; int B; int nchunk;
    const long long* chunk_lo; const int* seg_chunk; const int* seg_of; double2* part;
};
// one Arnoldi step per segment after w = A v_j (j = *jp): classical Gram-Schmidt `passes`
// times with per-segment coefficients into H column j (layout [row][segment]), the per-segment
// norms into nrm and H's subdiagonal, V[:, j + 1] = w / norm
void launch_seg_arnoldi(const SegDesc& S, double2* V, int m, int* jp, double2* w, double2* hh, double2* H, double2* nrm,
                        int passes, cudaStream_t s);
// nrm[s] = (||v_s||, 0)
void launch_seg_norms(const SegDesc& S, const double2* v, double2* nrm, cudaStream_t s);
// V[:, 0] = w / nrm per segment
void launch_seg_scale0(const SegDesc& S, const double2* w, const double2* nrm, double2* V, cudaStream_t s);
// x += V[:, 0..ncols) Y per segment (Y[c * B + s])
void launch_seg_axpy(const SegDesc& S, const double2* V, int ncols, const double2* Y, double2* x, cudaStream_t s);

// one Arnoldi step after w = A v_j, with j read from *jp (for a captured iteration graph):
// classical Gram-Schmidt against V[:, 0..j], `passes` times (2: CGS2), into the Hessenberg
// column j, ||w||^2 into *nrm2 (zeroed by launch_copy_col), h_{j+1,j} and
// V[:, j+1] = w / h_{j+1,j}; then, with lsq, the Givens step of launch_lsq_givens (which
// advances j), else j += 1
void launch_arnoldi_step(double2* V, long long n, int m, int* jp, double2* w, double2* h, double2* H, double* nrm2,
                         double2* part, cudaStream_t s, int passes = 2, const LsqDev* lsq = nullptr,
                         cudaGraphConditionalHandle cond = 0, bool use_cond = false);
// size (double2 entries) of the partial-sum buffer launch_arnoldi_step needs
int arnoldi_part_size(long long n, int m);
// Z[:, *jp] = z
void launch_store_col(const double2* z, long long n, const int* jp, double2* Z, cudaStream_t s);
// out = V[:, *jp]; zeroes *nrm2 when given
void launch_copy_col(const double2* V, long long n, const int* jp, double2* out, double* nrm2, cudaStream_t s);
// FP64 FMA throughput (TFLOP/s) of the current device; false on a CUDA error
bool launch_fp64_peak(double* tflops);

}  // namespace ifgf
