/* ifgf2d.h -- C ABI of the GB300 IFGF2D forward map (libifgf2d.so).
 *
 * Drop-in boundary for the matvec that GMRES calls in IFGF2D: the reference's
 * ForwardMap<Np, SingleLayer, Ps, Pang> / LinearOperator / opGMRES path.  Plain pointers
 * and sizes only; complex vectors are interleaved (re, im) doubles, i.e. the memory layout
 * of std::complex<double> / Eigen::VectorXcd.  Every call returns an int status (IFGF2D_OK
 * or an IFGF2D_ERR_* code) and never throws; ifgf2d_last_error() gives the message.
 * Calls on one context are serialised on the context's own CUDA stream; distinct contexts
 * are independent.  Reference citations are paths inside the IFGF2D repository.
 */
#ifndef IFGF2D_H
#define IFGF2D_H

#ifdef __cplusplus
extern "C" {
#endif

/* curve types (Geometry/Curve.hpp:106-161; STAR is an extension) */
#define IFGF2D_CURVE_CIRCLE 0 /* params: cx, cy, r */
#define IFGF2D_CURVE_KITE 1   /* params: A, B, C, D: x = A cos t + B cos 2t + C, y = D sin t */
#define IFGF2D_CURVE_LINE 2   /* params: x1, y1, x2, y2 on t in [-1, 1] (open) */
#define IFGF2D_CURVE_STAR 3   /* params: cx, cy, M, a_1..a_M, b_1..b_M (M <= 6) */

/* status codes */
#define IFGF2D_OK 0
#define IFGF2D_ERR_ARG 1          /* bad argument (size, pointer, option) */
#define IFGF2D_ERR_GEOMETRY 2     /* point outside the tree box, empty curve, ... */
#define IFGF2D_ERR_NEIGHBORHOOD 3 /* singular/near-singular point outside the leaf neighbourhood */
#define IFGF2D_ERR_NLEVELS 4      /* nlevels < 3 or too deep */
#define IFGF2D_ERR_CUDA 5         /* CUDA runtime error (message in ifgf2d_last_error) */
#define IFGF2D_ERR_STATE 6        /* call out of order (apply before setup, ...) */
#define IFGF2D_ERR_NONFINITE 7    /* non-finite value in an output */
#define IFGF2D_ERR_NOCONV 8       /* GMRES did not reach the tolerance */

/* formulations (FormulationType, ForwardMap/GreenFunctions.hpp:15-20) */
#define IFGF2D_SINGLE_LAYER 0 /* S phi, kernel (i/4) H0(k r) (the reference's working formulation) */
#define IFGF2D_COMBINED 2     /* (1/2 I + K - i eta S) phi: sound-soft combined field equation, with
                               * K the double layer (normal derivative at the source).  The
                               * reference's Combined is commented out (GreenFunctions.hpp:68-75);
                               * this one is written from the Colton-Kress formulation. */

/* apply modes */
#define IFGF2D_APPLY_DIRECT 0 /* ForwardMap::compute_Ax_unacc  (ForwardMap/ForwardMap.tpp:517-540) */
#define IFGF2D_APPLY_IFGF 1   /* ForwardMap::compute_Ax_acc    (ForwardMap/ForwardMap.tpp:609-655) */
#define IFGF2D_APPLY_IFGF_MIXED 2 /* compute_Ax_acc with the IFGF far field in complex64 (FP32
                                   * arithmetic on tables computed in FP64); the rectangular-polar
                                   * correction stays FP64.  No counterpart in the reference. */

typedef struct ifgf2d_curve {
    int type;        /* IFGF2D_CURVE_* */
    int closed;      /* Curve::is_closed */
    double tlim1;    /* Curve::tlim1 */
    double tlim2;    /* Curve::tlim2 */
    double params[16];
} ifgf2d_curve;

/* Junction (Geometry/Curve.hpp:10-17): curve `curve` touches `touching_curve` */
typedef struct ifgf2d_junction {
    int curve;
    int touching_curve;
    int t1_touches_t1;
} ifgf2d_junction;

/* ForwardMap template and constructor parameters (ForwardMap/ForwardMap.hpp:49, 94-97) */
typedef struct ifgf2d_options {
    int Np;                        /* points per patch (template Np) */
    double delta;                  /* rectangular-polar near-singularity distance */
    double wavelengths_per_patch;  /* patch size rule (Curve.cpp:37-68) */
    double patch_split_wavenumber; /* wavenumber of the patch size rule */
    double p;                      /* change-of-variables order (default 4) */
    int patches_per_curve;         /* > 0: equal-parameter split instead (extension) */
    int Ps;                        /* IFGF radial Chebyshev nodes (template Ps, default 5) */
    int Pang;                      /* IFGF angular Chebyshev nodes (template Pang, default 5) */
    int formulation;               /* IFGF2D_SINGLE_LAYER (template Formulation) or IFGF2D_COMBINED */
    double coupling;               /* eta of IFGF2D_COMBINED; <= 0 means eta = wavenumber */
    int device_geometry;           /* 1: ifgf2d_create computes the points, patch bounding boxes and
                                    * near-singular points on the current GPU (the patch limits stay on
                                    * the host); 0: all on the host, bit for bit as the reference's
                                    * constructor (ForwardMap.tpp:37-285).  Extension. */
} ifgf2d_options;

typedef struct ifgf2d_ctx ifgf2d_ctx;

/* ForwardMap::ForwardMap (ForwardMap/ForwardMap.tpp:15-35): discretise the curves. */
int ifgf2d_create(const ifgf2d_curve* curves, int ncurves, const ifgf2d_junction* junctions,
                  int njunctions, const ifgf2d_options* opts, ifgf2d_ctx** out);
int ifgf2d_destroy(ifgf2d_ctx* ctx);
const char* ifgf2d_last_error(const ifgf2d_ctx* ctx);

/* Host threads one set-up call may use (tree, plans, discretisation; process-wide): 0 = all
 * cores (the default), 1 = serial.  A caller that sets up many contexts concurrently from its
 * own threads (independent obstacles) sets 1 and keeps its own threads busy instead. */
int ifgf2d_set_host_threads(int n);

/* ForwardMap::total_num_unknowns_, num_patches_ (ForwardMap/ForwardMap.hpp:52-53) */
long long ifgf2d_num_unknowns(const ifgf2d_ctx* ctx);
long long ifgf2d_num_patches(const ifgf2d_ctx* ctx);
/* ForwardMap::xs_, ys_, nxs_, nys_ (ForwardMap/ForwardMap.hpp:72-75); any pointer may be NULL */
int ifgf2d_get_points(const ifgf2d_ctx* ctx, double* xs, double* ys, double* nxs, double* nys);
/* per patch: t1, t2 and near-singular point count (Geometry/Patch.hpp:40, 69-74) */
int ifgf2d_get_patches(const ifgf2d_ctx* ctx, double* t1t2, long long* ns_count);
/* concatenated near-singular lists, patch by patch: point index and Brent t value */
int ifgf2d_get_near_singular(const ifgf2d_ctx* ctx, long long* idx, double* t);

/* ForwardMap::compute_precomputations (ForwardMap/ForwardMap.tpp:391-423), on the GPU. */
int ifgf2d_precompute(ifgf2d_ctx* ctx, double wavenumber);
/* patch p's rectangular-polar matrix, Np x (Np + n_ns), column-major, interleaved complex */
int ifgf2d_get_precomputations(ifgf2d_ctx* ctx, long long patch, double* out);

/* ForwardMap::precomps_and_setup (ForwardMap/ForwardMap.tpp:542-565): precomputations,
 * BoxTree::Reinitialize (IFGF_Source/BoxTree.h:995-1008), the neighbourhood check
 * (BoxTree.h:1079-1161) and the exclusion sets (ForwardMap.tpp:567-607), all flattened into
 * device tables.  nlevels <= 0 picks the deepest tree that passes the neighbourhood check.
 * The host builds the tree in stages while the GPU computes the tables whose inputs exist; the
 * call returns when all of it is done.  When the tree fails (IFGF2D_ERR_NEIGHBORHOOD, ...) the
 * precomputations of the new wavenumber are still made, as the reference makes them first. */
int ifgf2d_setup(ifgf2d_ctx* ctx, double wavenumber, int nlevels);
/* The host part of ifgf2d_setup alone: tree depth, neighbourhood check, tree and plans.  It
 * makes no CUDA call, so it may run on any host thread while the GPU works on other contexts;
 * a following ifgf2d_setup with the same wavenumber and nlevels does only the device part.
 * Until that setup the context's IFGF applies return IFGF2D_ERR_STATE. */
int ifgf2d_prepare(ifgf2d_ctx* ctx, double wavenumber, int nlevels);
int ifgf2d_get_nlevels(const ifgf2d_ctx* ctx);
/* BoxTree::getSorting (IFGF_Source/BoxTree.h:1163-1165) */
int ifgf2d_get_sorting(const ifgf2d_ctx* ctx, long long* sorting);

/* y = A x, host vectors of N complex values (LinearOperator::operator*,
 * ForwardMap/LinearOperator.cpp:14-22 -> compute_Ax_unacc / compute_Ax_acc).  The first call
 * per mode after a set-up, precomputation or tuning change captures the device part as a CUDA
 * graph; later calls launch that graph between the two copies. */
int ifgf2d_apply(ifgf2d_ctx* ctx, const double* x, double* y, int mode);
/* the same on device-resident vectors (cudaMalloc'ed, N complex each) */
int ifgf2d_apply_device(ifgf2d_ctx* ctx, const void* d_x, void* d_y, int mode);
/* BoxTree::Solve alone (IFGF_Source/BoxTree.h:1020-1071) on given intensities, host vectors:
 * the far-field sum that excludes self, same-patch and near-singular pairs. */
int ifgf2d_ifgf_far(ifgf2d_ctx* ctx, const double* intensities, double* y);

/* ForwardMap::solve (ForwardMap/ForwardMap.tpp:658-697): GMRES on the device, initial guess 0,
 * stop when the residual estimate |w_k|/||r0|| < tol, restart after `restart` steps.
 * mode IFGF2D_APPLY_IFGF_MIXED: FP64 iterative refinement -- the residual b - A x is formed with
 * the FP64 IFGF operator, corrections come from GMRES on the complex64 operator, and the stop
 * test is the FP64 relative residual; *iters counts inner GMRES iterations.
 * Returns IFGF2D_ERR_NOCONV (with x filled) when max_iters is reached first. */
int ifgf2d_solve(ifgf2d_ctx* ctx, const double* rhs, double* x, int mode, double tol, int restart,
                 int max_iters, int* iters, double* est_error);

/* Batched forms for nrhs right-hand sides with one geometry and wavenumber (the reference
 * calls LinearOperator::operator* / ForwardMap::solve once per right-hand side,
 * ForwardMap.tpp:658-697).  x, y, rhs are column-major N x nrhs complex matrices (right-hand
 * side r at offset 2*N*r doubles, interleaved re/im), as an Eigen::MatrixXcd stores them.  The
 * IFGF modes process up to IFGF2D_MAX_BATCH right-hand sides per pass over the tables (larger
 * batches run in chunks); IFGF2D_APPLY_DIRECT runs one right-hand side at a time. */
#define IFGF2D_MAX_BATCH 64
int ifgf2d_apply_batch(ifgf2d_ctx* ctx, const double* x, double* y, int nrhs, int mode);
/* the same on device-resident matrices (cudaMalloc'ed, N * nrhs complex each); asynchronous on
 * the context's stream */
int ifgf2d_apply_batch_device(ifgf2d_ctx* ctx, const void* d_x, void* d_y, int nrhs, int mode);
/* ifgf2d_solve for every column of rhs: GMRES runs for all right-hand sides in lock step with
 * the batched operator, each with its own Krylov basis, Hessenberg matrix, rotations and stop
 * test (a converged right-hand side is frozen).  iters[r] and est_error[r] as in ifgf2d_solve
 * (either may be NULL).  Returns IFGF2D_ERR_NOCONV when some right-hand side reached max_iters
 * first. */
int ifgf2d_solve_batch(ifgf2d_ctx* ctx, const double* rhs, double* x, int nrhs, int mode, double tol, int restart,
                       int max_iters, int* iters, double* est_error);

/* ForwardMap::propagate_unacc (ForwardMap/ForwardMap.tpp:701-727): direct off-surface field */
int ifgf2d_propagate(ifgf2d_ctx* ctx, long long m, const double* xp, const double* yp,
                     const double* density, double* out);

/* The off-surface field with the IFGF (no counterpart in the reference, which sums directly:
 * ForwardMap::propagate_unacc, ForwardMap.tpp:701-727).  setup builds the evaluation plan for
 * m targets (anywhere, also outside the tree's box) on a context that ifgf2d_setup prepared;
 * it stays valid until the next setup or precompute.  eval then takes a density (N complex,
 * patch order) and writes the field at the m targets (m complex): direct sums over the
 * sources of each target's adjacent leaf boxes plus cone interpolation for the rest, within
 * the IFGF tolerance of ifgf2d_propagate. */
int ifgf2d_eval_offsurface_setup(ifgf2d_ctx* ctx, long long m, const double* xp, const double* yp);
int ifgf2d_eval_offsurface(ifgf2d_ctx* ctx, const double* density, double* out);
/* work of one evaluation: near pairs, leaf evaluations, propagation evaluations, interpolation
 * evaluations */
int ifgf2d_eval_offsurface_counts(const ifgf2d_ctx* ctx, long long out[4]);

/* The learned right preconditioner (no counterpart in the reference, which runs GMRES
 * unpreconditioned).  A 1D convolutional network along the boundary parameter: 6 layers of
 * kernel 7 with circular padding, 64 channels, BF16 weights and activations with FP32
 * accumulation on the tensor cores.  Per point it reads the residual turned to its canonical
 * phase and over its RMS (r e^{-i phi} / sigma, sigma = RMS(r), phi = arg(sum r^2) / 2),
 * curvature / k, the unit tangent and k h (h the quadrature weight), and returns two channels
 * o; the preconditioner is M(r) = 2 r + sigma e^{i phi} (o_0 + i o_1), and the training target
 * is o = (e - 2 r) e^{-i phi} / sigma.  A new network's output layer is zero (M = 2 I).  Samples (one residual each, in a curve's patch order) are passed
 * concatenated: len[s] points each, complex interleaved r / e, geom = 4 doubles per point
 * (curvature, tangent x, tangent y, h, as ifgf2d_get_geometry_features gives them), k per
 * sample.  Parameters: per layer the FP32 weights [cout][7][cin] then the bias [cout], with
 * cin / cout padded to 16, 64, 64, 64, 64, 64 / 64, 64, 64, 64, 64, 16. */
typedef struct ifgf2d_net ifgf2d_net;
long long ifgf2d_net_num_params(void);
int ifgf2d_net_create(unsigned long long seed, ifgf2d_net** out);
int ifgf2d_net_destroy(ifgf2d_net* net);
const char* ifgf2d_net_last_error(const ifgf2d_net* net);
int ifgf2d_net_get_params(ifgf2d_net* net, float* params);
int ifgf2d_net_set_params(ifgf2d_net* net, const float* params);
/* mean squared error of o against its target and the gradient w.r.t. the parameters */
int ifgf2d_net_gradient(ifgf2d_net* net, int nseg, const int* len, const double* r, const double* e, const double* geom,
                        const double* k, double* loss, float* grad);
/* one AdamW step (beta 0.9 / 0.999) on that loss */
int ifgf2d_net_train_step(ifgf2d_net* net, int nseg, const int* len, const double* r, const double* e, const double* geom,
                          const double* k, float lr, float weight_decay, double* loss);
/* z = M(r) per sample (complex interleaved), and / or the raw outputs o (2 floats per point) */
int ifgf2d_net_apply(ifgf2d_net* net, int nseg, const int* len, const double* r, const double* geom, const double* k, double* z,
                     float* out2);
/* 1: the network's output is a correction weighted by the flat symbol's magnitude (trained on
 * targets Op(|sigma|) e, see ifgf2d_spectral_symbol); together with the spectral preconditioner
 * the correction applied is then Op(1/|sigma|) of it.  0 (default): unweighted. */
int ifgf2d_net_set_output_weighting(ifgf2d_net* net, int weighted);
int ifgf2d_net_output_weighting(const ifgf2d_net* net);
/* ifgf2d_solve with the network as right preconditioner: flexible GMRES (z_j = M(v_j)) on the
 * operator of `mode` inside FP64 iterative refinement (the stop test is the FP64 relative
 * residual, formed with the FP64 IFGF operator, or the direct one in IFGF2D_APPLY_DIRECT).  A
 * preconditioned correction that misses its tolerance switches the rest of the solve to plain
 * GMRES.  *iters counts inner iterations. */
int ifgf2d_solve_precond(ifgf2d_ctx* ctx, ifgf2d_net* net, const double* rhs, double* x, int mode, double tol, int restart,
                         int max_iters, int* iters, double* est_error);

/* Spectral right preconditioner of the combined-field operator on closed curves (no
 * counterpart in the reference, whose GMRES, ForwardMap/opGMRES.hpp:68-269, is
 * unpreconditioned).  M r = 2 r + B F^-1 [(1/sigma - 2) F (W r)]: W resamples each curve's node
 * values onto a uniform arc-length grid, F is the FFT along the curve, sigma(xi) =
 * 1/2 + eta / (2 sqrt((k + i eps)^2 - xi^2)) the flat-boundary symbol of 1/2 I + K - i eta S with
 * the glancing damping eps = scale k^(1/3), and B interpolates back to the nodes.  FP32 on the
 * device.  Set-up (after precompute; host tables, uploaded; a new precompute drops them):
 * scale <= 0 takes IFGF2D_SPECTRAL_DEFAULT_SCALE.  Needs the combined formulation and closed
 * curves of at most 2^20 points each. */
#define IFGF2D_SPECTRAL_DEFAULT_SCALE 0.25
int ifgf2d_spectral_setup(ifgf2d_ctx* ctx, double scale);
/* z = M r on host vectors (complex interleaved, N entries), for tests */
int ifgf2d_spectral_apply(ifgf2d_ctx* ctx, const double* r, double* z);
/* z = Op(m) r for one of the tables' symbols (host vectors): IFGF2D_SYMBOL_PRECONDITIONER is
 * ifgf2d_spectral_apply; IFGF2D_SYMBOL_MAGNITUDE applies |sigma|, the operator's flat-boundary
 * magnitude, and IFGF2D_SYMBOL_INVERSE_MAGNITUDE 1/|sigma|.  The last two weight the learned
 * network's training targets and output (residual-space error). */
#define IFGF2D_SYMBOL_PRECONDITIONER 0
#define IFGF2D_SYMBOL_MAGNITUDE 1
#define IFGF2D_SYMBOL_INVERSE_MAGNITUDE 2
int ifgf2d_spectral_symbol(ifgf2d_ctx* ctx, int which, const double* r, double* z);
/* ifgf2d_solve_precond with the preconditioner chosen by `precond`: IFGF2D_PRECOND_NET (net
 * required), IFGF2D_PRECOND_SPECTRAL (set up with the default scale on first use when
 * ifgf2d_spectral_setup was not called), or both: the spectral preconditioner plus the
 * network's correction, z = M_s r + (N(r) - 2 r), for a network trained on the spectral
 * preconditioner's errors. */
#define IFGF2D_PRECOND_NET 1
#define IFGF2D_PRECOND_SPECTRAL 2
int ifgf2d_solve_flexible(ifgf2d_ctx* ctx, ifgf2d_net* net, int precond, const double* rhs, double* x, int mode, double tol,
                          int restart, int max_iters, int* iters, double* est_error);
/* ifgf2d_solve_batch with flexible GMRES and the spectral preconditioner (precond must be
 * IFGF2D_PRECOND_SPECTRAL; mode IFGF2D_APPLY_IFGF or IFGF2D_APPLY_IFGF_MIXED): every right-hand
 * side's Krylov vector is preconditioned in the same launches. */
int ifgf2d_solve_batch_flexible(ifgf2d_ctx* ctx, int precond, const double* rhs, double* x, int nrhs, int mode, double tol,
                                int restart, int max_iters, int* iters, double* est_error);
/* per point of the context (patch order): curvature, unit tangent x, y, quadrature weight */
int ifgf2d_get_geometry_features(const ifgf2d_ctx* ctx, double* geom);

/* Device Hankel evaluator (replaces sp_bessel::hankelH1, complex_bessel
 * besselFunctions.h:313-341, for real arguments): out[i] = H_order^(1)(x[i]), order 0 or 1.
 * Orders 2 and 3 give H0 and H1 from the fused evaluator of the combined-field kernel (both
 * orders of one argument at once); they equal orders 0 and 1 bit for bit. */
int ifgf2d_hankel(int order, long long n, const double* x, double* out);

/* The context's CUDA stream (cudaStream_t) for callers that time or order work on it. */
void* ifgf2d_stream(ifgf2d_ctx* ctx);
/* Algorithmic work of one IFGF apply: near pairs, leaf evaluations, propagation evaluations,
 * interpolation evaluations, cones, levels, singular-correction entries, bytes resident. */
int ifgf2d_work_counts(const ifgf2d_ctx* ctx, long long out[8]);
/* FP64 refinement passes of the context's last mixed solve (ifgf2d_solve or
 * ifgf2d_solve_batch in IFGF2D_APPLY_IFGF_MIXED): each pass is one inner complex64 GMRES and one
 * FP64 residual.  -1 for a NULL context. */
int ifgf2d_last_refinements(const ifgf2d_ctx* ctx);

/* Timed apply on device vectors: CUDA events on the context's stream between the phases
 * (no counterpart in the reference, whose timers are std::chrono prints, ForwardMap.tpp:545-563).
 * ms[0..4] = singular correction, intensities (+ Morton permutation), leaf cones,
 * propagation (all levels), near field + interpolation; the direct mode reports its far sum
 * in ms[4]. */
int ifgf2d_apply_timed(ifgf2d_ctx* ctx, const void* d_x, void* d_y, int mode, double ms[5]);

/* Launch-shape autotuner (no counterpart in the reference): times every launch shape of the
 * leaf-cone kernel (source chunks per coefficient 1, 2, 5, 10; complex64 also 0, the table
 * streamed through shared memory by TMA bulk copies), of each level's propagation (2, 4 or the
 * most cones per block, or 1: child blocks staged in shared memory) and of the single-vector
 * interpolation (by target or by leaf box) on this context's own tables, in both precisions, and
 * keeps the fastest.  The table has ifgf2d_tuning_size() ints: leaf FP64, leaf complex64, then
 * per precision one propagation entry per level (0 = the most cones per block), then a bit
 * mask of kernel choices: the batched complex64 kernels that run in 3xTF32 on the tcgen05
 * tensor cores (IFGF2D_BATCH_TC_*; FP32 FMA otherwise), the other batched choices and the
 * single-vector interpolation by leaf box (IFGF2D_SINGLE_INTERP_BY_BOX_*); the default is
 * IFGF2D_BATCH_TC_LEAF | IFGF2D_BATCH_GROUPED_INTERP | IFGF2D_SINGLE_INTERP_BY_BOX_C64.
 * get / set read and restore it (e.g. from an on-disk cache); applies use the context's
 * current table. */
#define IFGF2D_BATCH_TC_LEAF 1          /* leaf-cone sums, 3xTF32 (two TF32 terms per operand) */
#define IFGF2D_BATCH_TC_PROPAGATION 2   /* propagation, 3xTF32 */
#define IFGF2D_BATCH_TC_LEAF_FP32 4     /* leaf-cone sums, three TF32 terms per operand (6 products) */
#define IFGF2D_BATCH_BULK_PROPAGATION 8 /* FP32 FMA propagation, child coefficients staged by TMA bulk copies */
#define IFGF2D_BATCH_GROUPED_INTERP 16  /* complex64 interpolation grouped by cone per leaf box */
#define IFGF2D_SINGLE_INTERP_BY_BOX_FP64 32  /* single vector, FP64: interpolation by leaf box, a lane per target */
#define IFGF2D_SINGLE_INTERP_BY_BOX_C64 64   /* single vector, complex64: the same */
int ifgf2d_tuning_size(void);
int ifgf2d_autotune(ifgf2d_ctx* ctx, int reps, int* choices);
int ifgf2d_get_tuning(const ifgf2d_ctx* ctx, int* choices);
int ifgf2d_set_tuning(ifgf2d_ctx* ctx, const int* choices);

/* FP64 FMA throughput of the current GPU in TFLOP/s (a dependent-FMA microbenchmark); the
 * roofline denominator of the FP64 kernels (no counterpart in the reference). */
int ifgf2d_measure_fp64_peak(double* tflops);

/* Many obstacles as one block-diagonal operator (no counterpart in the reference, which solves one
 * obstacle per ForwardMap::solve, ForwardMap.tpp:658-697).  group_create merges n <= 1024 contexts, each
 * created and prepared (ifgf2d_prepare: its wavenumber, tree and plans) with the same Np, Ps,
 * Pang, p and formulation, into one operator whose tables hold every member side by side, with
 * the tree levels aligned from the leaves: each phase of its set-up and of an apply is one launch
 * over all members.  The members may be destroyed afterwards.  Vectors hold every member's
 * unknowns in member order (member o at ifgf2d_group_offsets()[o]).  group_solve runs GMRES for
 * all members in lock step, each with its own Krylov basis, Gram-Schmidt sums, rotations and stop
 * test (IFGF2D_APPLY_IFGF_MIXED: FP64 refinement around complex64 inner solves, each member
 * stopping on its own FP64 relative residual); iters[o] and est[o] per member. */
typedef struct ifgf2d_group ifgf2d_group;
int ifgf2d_group_create(ifgf2d_ctx* const* members, int n, ifgf2d_group** out);
int ifgf2d_group_destroy(ifgf2d_group* group);
const char* ifgf2d_group_last_error(const ifgf2d_group* group);
long long ifgf2d_group_num_unknowns(const ifgf2d_group* group);
/* n + 1 entries: the first unknown of each member, then the total */
int ifgf2d_group_offsets(const ifgf2d_group* group, long long* offsets);
int ifgf2d_group_apply(ifgf2d_group* group, const double* x, double* y, int mode);
int ifgf2d_group_solve(ifgf2d_group* group, const double* rhs, double* x, int mode, double tol, int restart, int max_iters,
                       int* iters, double* est);
/* ifgf2d_group_solve with flexible GMRES and the spectral preconditioner (precond must be
 * IFGF2D_PRECOND_SPECTRAL), each member's curve with its own wavenumber and coupling; the tables
 * are built on the first call. */
int ifgf2d_group_solve_flexible(ifgf2d_group* group, int precond, const double* rhs, double* x, int mode, double tol,
                                int restart, int max_iters, int* iters, double* est);

/* Largest N accepted by ifgf2d_apply_direct_noalloc. */
#define IFGF2D_NOALLOC_MAX_N 65536

/* The direct forward map (as ifgf2d_apply_device with IFGF2D_APPLY_DIRECT) on caller-owned
 * device vectors, with no device allocation inside the call.  No counterpart in the reference.
 * For callers that cannot allocate at the call site: a host application or plugin framework
 * that owns the device memory budget, or a latency-critical loop that cannot take the implicit
 * synchronisation of cudaMalloc / cudaFree.  Its scratch (the weighted density) is a fixed
 * 1 MiB device array inside the library, so N must not exceed IFGF2D_NOALLOC_MAX_N
 * (IFGF2D_ERR_ARG otherwise).  The context must have been precomputed (ifgf2d_precompute or
 * ifgf2d_setup) and its device must be current.  That set-up looks up the array's device
 * address (cudaGetSymbolAddress, which under lazy module loading loads the array) and loads
 * the kernels the call launches, so the call itself loads and allocates nothing.
 * cudaDeviceReset frees the array: run a set-up again on that device before the next call.
 * Work is queued on the context's stream; synchronise before reading d_y.  All calls share
 * the one array, so calls that overlap on the GPU (several contexts or streams at once) race:
 * order them on one stream or synchronise between them. */
int ifgf2d_apply_direct_noalloc(ifgf2d_ctx* ctx, const void* d_x, void* d_y);

#ifdef __cplusplus
}
#endif
#endif /* IFGF2D_H */
