// batch.cu -- batched apply and solve of the C ABI (include/ifgf2d.h): many right-hand sides
// (incidence angles) with one geometry and wavenumber.
//
// The reference solves one right-hand side per ForwardMap::solve call (ForwardMap.tpp:658-697);
// every call re-reads the same operator.  Here up to kMaxBatch right-hand sides share one pass
// over the tables (ifgf_batch.cu), and GMRES runs for all of them in lock step: one batched
// apply per iteration, per-RHS Gram-Schmidt coefficients from batched reductions, and each
// right-hand side's own Givens rotations, residual estimate and stop test on the device.
#include "context.hpp"
#include "host_threads.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

struct BatchWork {
    int cap = 0;                               // right-hand sides the apply buffers hold
    DBuf<double2> xt, yt;                      // interleaved [N][cap]
    DBuf<double2> rho64, coef64;
    DBuf<float2> rho32, coef32;
    DBuf<PropB<double>> pb64;
    DBuf<double> rows64;                       // the FP64 plan terms' Chebyshev rows (FP64-pipe work the lanes share)
    DBuf<PropB<float>> pb32;
    DBuf<float2> W32;                          // complex64 copy of the singular-correction weights
    DBuf<float2> xt32;                         // complex64 copy of the interleaved input (mixed form)
    DBuf<double2> xcm, ycm;                    // column-major staging of the host entry points
    // the tensor-core propagation: its error flag (an mbarrier wait that ran out) and the SM count
    DBuf<int> t5err;
    int nsm = 0;
    DBuf<int4> leaf_items;                     // (leaf box, first cone, end cone, 0) of the tensor-core leaf kernel
    // the complex64 interpolation grouped by cone: work items (terms, targets) and their terms
    DBuf<int4> ig_items;
    DBuf<InterpG> ig_terms;
    // GMRES
    int m = 0, scap = 0;
    DBuf<double2> V, w, t, h, H, part, Y, hn, b, x, r, d, ones;
    // refinement passes after the first work on the columns still short of the tolerance,
    // gathered into compact [N][Bc] arrays (right-hand side, solution, residual, correction, A x)
    DBuf<double2> cb, cx, cr, cd, ct;
    DBuf<int> act;
    // least squares on the device (LsqBatchDev), per-RHS cycle parameters and the per-iteration
    // count of the right-hand sides still running
    DBuf<double2> lsR, lsg, lsgs;
    DBuf<double> lsgc, lssc, lspar;
    DBuf<int> lsst, lsact;
    // flexible GMRES with the spectral preconditioner: z_j = M v_j for every column (right-hand
    // sides interleaved as V), and the preconditioner's grid values of every right-hand side
    DBuf<double2> Z;
    DBuf<float2> ug;
    int zcap = 0, zm = 0;
};

void ifgf::free_batch(ifgf2d_ctx* ctx) {
    delete ctx->bw;
    ctx->bw = nullptr;
}

namespace {

// The interpolation terms of each leaf box's targets, kInterpGrpTargets targets per work item,
// sorted by cone (stable) within an item: items (first term, end term, first target, targets).
void grouped_interp_plan(const Tree& T, std::vector<int4>& items, std::vector<InterpG>& terms) {
    const int nleaf = (int)T.leaf_start.size();
    std::vector<long long> item_ptr(nleaf + 1, 0), term_ptr(nleaf + 1, 0);
    for (int b = 0; b < nleaf; ++b) {
        const int t0 = T.leaf_start[b], n = T.leaf_count[b];
        item_ptr[b + 1] = item_ptr[b] + (n + kInterpGrpTargets - 1) / kInterpGrpTargets;
        term_ptr[b + 1] = term_ptr[b] + (n > 0 ? T.ip_ptr[t0 + n] - T.ip_ptr[t0] : 0);
    }
    items.resize(item_ptr[nleaf]);
    terms.resize(term_ptr[nleaf]);
    parallel_for(nleaf, [&](long long b0, long long b1) {
        std::vector<int> idx;
        for (long long b = b0; b < b1; ++b) {
            const int t0 = T.leaf_start[b], n = T.leaf_count[b];
            long long it = item_ptr[b], e = term_ptr[b];
            for (int c0 = 0; c0 < n; c0 += kInterpGrpTargets, ++it) {
                const int nt = std::min(kInterpGrpTargets, n - c0);
                const int e0 = T.ip_ptr[t0 + c0], e1 = T.ip_ptr[t0 + c0 + nt];
                idx.resize(e1 - e0);
                for (int i = 0; i < e1 - e0; ++i) idx[i] = e0 + i;
                std::stable_sort(idx.begin(), idx.end(), [&](int a, int c) { return T.ip[a].cone < T.ip[c].cone; });
                const long long first = e;
                for (int i : idx) {
                    int t = t0 + c0;
                    while (T.ip_ptr[t + 1] <= i) ++t;   // the target owning term i
                    const InterpEntry& q = T.ip[i];
                    terms[e++] = InterpG{q.cone, t, (float)q.s, (float)q.th, (float)q.fr, (float)q.fi};
                }
                items[it] = make_int4((int)first, (int)e, t0 + c0, nt);
            }
        }
    }, 64);
}

int ensure_apply(ifgf2d_ctx* ctx, int B, bool mixed) {
    if (!ctx->bw) ctx->bw = new BatchWork;
    BatchWork& W = *ctx->bw;
    const long long N = ctx->D.N;
    const size_t ncoef = (size_t)ctx->T.total_cones * ctx->T.P;
    if (W.cap < B) {
        W.xt.release(); W.yt.release(); W.rho64.release(); W.coef64.release(); W.rho32.release(); W.coef32.release();
        W.xt32.release();
        CK(W.xt.alloc((size_t)N * B)); CK(W.yt.alloc((size_t)N * B));
        W.cap = B;
    }
    if (mixed) {
        if (!W.rho32.p) {
            CK(W.rho32.alloc((size_t)N * W.cap)); CK(W.coef32.alloc(ncoef * W.cap)); CK(W.xt32.alloc((size_t)N * W.cap));
        }
        if (!W.pb32.p) {
            CK(W.pb32.alloc(ctx->pp.n));
            launch_sort_plan<float>(ctx->pp_ptr.p, ctx->T.total_cones, ctx->pp.p, ctx->T.P, W.pb32.p, ctx->stream);
            CK(cudaGetLastError());
        }
        if (!W.t5err.p) {
            CK(prop_t5_init_attributes());
            CK(W.t5err.alloc(1));
            CK(cudaMemsetAsync(W.t5err.p, 0, sizeof(int), ctx->stream));
            int dev = 0;
            CK(cudaGetDevice(&dev));
            CK(cudaDeviceGetAttribute(&W.nsm, cudaDevAttrMultiProcessorCount, dev));
            const TreeLevel& LD = ctx->T.L[ctx->nlevels - 1];
            std::vector<int4> items;
            for (size_t b = 0; b + 1 < LD.cone_ptr.size(); ++b)   // at most kLeafT5Cones cones per item
                for (int c = LD.cone_ptr[b]; c < LD.cone_ptr[b + 1]; c += kLeafT5Cones)
                    items.push_back(make_int4((int)b, c, std::min(c + kLeafT5Cones, LD.cone_ptr[b + 1]), 0));
            CK(W.leaf_items.upload(items));
            std::vector<int4> gi;
            std::vector<InterpG> gt;
            grouped_interp_plan(ctx->T, gi, gt);
            CK(W.ig_items.upload(gi));
            CK(W.ig_terms.upload(gt));
        }
        if (!W.W32.p) {
            CK(W.W32.alloc(ctx->W.n));
            launch_d2f(ctx->W.p, (long long)ctx->W.n, W.W32.p, ctx->stream);
        }
    } else {
        if (!W.rho64.p) { CK(W.rho64.alloc((size_t)N * W.cap)); CK(W.coef64.alloc(ncoef * W.cap)); }
        if (!W.pb64.p) {
            CK(W.pb64.alloc(ctx->pp.n));
            launch_sort_plan<double>(ctx->pp_ptr.p, ctx->T.total_cones, ctx->pp.p, ctx->T.P, W.pb64.p, ctx->stream);
            CK(cudaGetLastError());
            CK(W.rows64.alloc(ctx->pp.n * (size_t)(ctx->T.Ps + ctx->T.Pang)));
            launch_plan_rows<double>(W.pb64.p, (long long)ctx->pp.n, ctx->T.Ps, ctx->T.Pang, W.rows64.p, ctx->stream);
            CK(cudaGetLastError());
        }
    }
    return IFGF2D_OK;
}

template <typename R>
void far_b(ifgf2d_ctx* ctx, const V2<R>* rho, const V2<R>* near, const V2<R>* leafL, const PropB<R>* pb,
           const InterpE<R>* ip, const R* Gsep, V2<R>* coef, int B, double2* yt) {
    const Tree& T = ctx->T;
    const int Dl = ctx->nlevels - 1;
    const TreeLevel& LD = T.L[Dl];
    cudaStream_t s = ctx->stream;
    bool leaf_done = false;
    if constexpr (sizeof(R) == 4) {
        BatchWork& W = *ctx->bw;
        if (ctx->tune_batch_tc & (kBatchTcLeaf | kBatchTcLeaf6))
            leaf_done = launch_leaf_t5(W.leaf_items.p, (int)W.leaf_items.n, ctx->leaf_start.p, ctx->leaf_count.p, ctx->leaf_off.p,
                                       leafL, rho, T.Ps, T.Pang, B, coef + (long long)LD.cone_base * T.P * B, W.t5err.p, W.nsm,
                                       (ctx->tune_batch_tc & kBatchTcLeaf6) ? 3 : 2, s);
    }
    if (!leaf_done)
        launch_leaf_b<R>(ctx->leaf_cone_box.p, (int)LD.cone_nonrel.size(), LD.cone_base, ctx->leaf_start.p, ctx->leaf_count.p,
                         ctx->leaf_off.p, leafL, rho, T.Ps, T.Pang, B, coef, s);
    for (int l = Dl; l >= 3; --l) {
        const TreeLevel& Lp = T.L[l - 1];
        const int p0 = Lp.cone_base, p1 = Lp.cone_base + (int)Lp.cone_nonrel.size();
        if constexpr (sizeof(R) == 4) {
            BatchWork& W = *ctx->bw;
            if ((ctx->tune_batch_tc & kBatchTcProp) && launch_prop_t5(p0, p1, ctx->pp_ptr.p, ctx->pp_nchild.p, pb, T.Ps, T.Pang, Gsep, B, coef,
                                                     W.t5err.p, W.nsm, s))
                continue;
            if ((ctx->tune_batch_tc & kBatchBulkProp) &&
                launch_prop_bk(p0, p1, ctx->pp_ptr.p, ctx->pp_nchild.p, pb, T.Ps, T.Pang, Gsep, B, coef, W.t5err.p, s))
                continue;
        }
        const R* rows = nullptr;
        if constexpr (sizeof(R) == 8) rows = ctx->bw->rows64.p;
        launch_prop_b<R>(p0, p1, ctx->pp_ptr.p, ctx->pp_nchild.p, pb, T.Ps, T.Pang, Gsep, B, coef, s, rows);
    }
    bool grouped = false;
    if constexpr (sizeof(R) == 4) grouped = (ctx->tune_batch_tc & kBatchGroupedInterp) && B <= 64 && T.Ps == 5 && T.Pang == 5;
    launch_final_b<R>((int)ctx->D.N, ctx->point_leaf.p, ctx->leaf_start.p, ctx->leaf_count.p, ctx->nbr_ptr.p, ctx->nbr_box.p,
                      ctx->near_rowlen.p, ctx->near_off.p, near, rho, ctx->ip_ptr.p, grouped ? nullptr : ip, coef, T.Ps, T.Pang,
                      ctx->sorting.p, B, yt, s);
    if constexpr (sizeof(R) == 4) {
        if (grouped) {
            BatchWork& W = *ctx->bw;
            launch_interp_grp(W.ig_items.p, (int)W.ig_items.n, W.ig_terms.p, coef, T.Ps, T.Pang, ctx->sorting.p, B, yt, s);
        }
    }
}

// yt = A xt for B <= kMaxBatch interleaved right-hand sides (IFGF modes)
int apply_il(ifgf2d_ctx* ctx, const double2* xt, double2* yt, int B, int mode) {
    const bool mixed = mode == IFGF2D_APPLY_IFGF_MIXED;
    int rc = ensure_apply(ctx, B, mixed);
    if (rc != IFGF2D_OK) return rc;
    BatchWork& W = *ctx->bw;
    const Discretisation& D = ctx->D;
    const double half = ctx->form == IFGF2D_COMBINED ? 0.5 : 0.0;
    if (mixed) launch_d2f(xt, (long long)D.N * B, W.xt32.p, ctx->stream);
    launch_sing_b(xt, W.xt32.p, ctx->W.p, W.W32.p, ctx->srow_ptr.p, ctx->srow_col.p, ctx->cols.p, (int)D.N, D.Np, B, half, yt, ctx->wq.p,
                  ctx->inverse.p, mixed ? nullptr : W.rho64.p, mixed ? W.rho32.p : nullptr, ctx->stream);
    if (mixed)
        far_b<float>(ctx, W.rho32.p, ctx->near32.p, ctx->leafL32.p, W.pb32.p, ctx->ip32.p, ctx->Gsep32.p, W.coef32.p, B, yt);
    else
        far_b<double>(ctx, W.rho64.p, ctx->near.p, ctx->leafL.p, W.pb64.p, ctx->ip.p, ctx->Gsep.p, W.coef64.p, B, yt);
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

// after a synchronisation: did a tensor-core propagation give up on a wait?
int check_t5(ifgf2d_ctx* ctx) {
    if (!ctx->bw || !ctx->bw->t5err.p) return IFGF2D_OK;
    int v = 0;
    CK(cudaMemcpy(&v, ctx->bw->t5err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (!v) return IFGF2D_OK;
    CK(cudaMemsetAsync(ctx->bw->t5err.p, 0, sizeof(int), ctx->stream));
    return fail(ctx, IFGF2D_ERR_CUDA, "tensor-core propagation: a tensor-memory completion wait ran out");
}

int check_mode(ifgf2d_ctx* ctx, int mode) {
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) before apply");
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_DIRECT && mode != IFGF2D_APPLY_IFGF_MIXED)
        return fail(ctx, IFGF2D_ERR_ARG, "unknown apply mode");
    if (mode != IFGF2D_APPLY_DIRECT && !ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup before an IFGF apply");
    return IFGF2D_OK;
}

// column-major device matrices, any nrhs
int apply_cm(ifgf2d_ctx* ctx, const double2* x, double2* y, int nrhs, int mode) {
    const long long N = ctx->D.N;
    if (mode == IFGF2D_APPLY_DIRECT) {
        for (int r = 0; r < nrhs; ++r) {
            int rc = apply_single(ctx, x + (long long)r * N, y + (long long)r * N, mode);
            if (rc != IFGF2D_OK) return rc;
        }
        return IFGF2D_OK;
    }
    for (int r0 = 0; r0 < nrhs; r0 += kMaxBatch) {
        const int B = std::min(kMaxBatch, nrhs - r0);
        int rc = ensure_apply(ctx, B, mode == IFGF2D_APPLY_IFGF_MIXED);
        if (rc != IFGF2D_OK) return rc;
        BatchWork& W = *ctx->bw;
        launch_interleave(x + (long long)r0 * N, N, B, W.xt.p, ctx->stream);
        if ((rc = apply_il(ctx, W.xt.p, W.yt.p, B, mode))) return rc;
        launch_deinterleave(W.yt.p, N, B, y + (long long)r0 * N, ctx->stream);
    }
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

// ---------------------------------------------------------------- batched GMRES
int ensure_solve(ifgf2d_ctx* ctx, int B, int m) {
    if (!ctx->bw) ctx->bw = new BatchWork;
    BatchWork& W = *ctx->bw;
    const long long N = ctx->D.N;
    if (W.scap < B || W.m != m) {
        const size_t nb = (size_t)N * B;
        CK(W.V.alloc(nb * (m + 1))); CK(W.w.alloc(nb)); CK(W.t.alloc(nb));
        CK(W.b.alloc(nb)); CK(W.x.alloc(nb)); CK(W.r.alloc(nb)); CK(W.d.alloc(nb));
        CK(W.h.alloc((size_t)(m + 1) * B)); CK(W.H.alloc((size_t)m * (m + 1) * B));
        CK(W.part.alloc((size_t)bdot_chunks(N) * (m + 1) * B)); CK(W.Y.alloc((size_t)m * B)); CK(W.hn.alloc(B));
        CK(W.lsR.alloc((size_t)B * (m + 1) * m)); CK(W.lsg.alloc((size_t)B * (m + 1))); CK(W.lsgc.alloc((size_t)B * m));
        CK(W.lsgs.alloc((size_t)B * m)); CK(W.lssc.alloc((size_t)3 * B)); CK(W.lspar.alloc((size_t)3 * B));
        CK(W.lsst.alloc((size_t)4 * B)); CK(W.lsact.alloc(m));
        std::vector<double2> one(B, make_double2(1.0, 0.0));
        CK(W.ones.upload(one));
        W.scap = B; W.m = m;
    }
    return IFGF2D_OK;
}

// per-RHS 2-norms of interleaved vectors into W.hn, copied to host
int bnorms(ifgf2d_ctx* ctx, const double2* v, int B, std::vector<double>& out) {
    BatchWork& W = *ctx->bw;
    const long long N = ctx->D.N;
    launch_bdot(v, 0, 1, v, N, B, W.part.p, nullptr, W.hn.p, 0, 0, ctx->stream);
    std::vector<double2> hv(B);
    CK(cudaMemcpyAsync(hv.data(), W.hn.p, sizeof(double2) * B, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    out.resize(B);
    for (int r = 0; r < B; ++r) out[r] = hv[r].x;
    return IFGF2D_OK;
}

// x = A^{-1} b for B interleaved right-hand sides, initial guess 0 (opGMRES.hpp:383-392).
// Right-hand side r stops when |g_{j+1}| / ||r0|| < tol[r] (opGMRES.hpp:207), after max_iters
// iterations, or at the start when skip[r]; a stopped right-hand side keeps its x.  Each
// right-hand side's Givens rotations, estimate and stop test run on the device
// (launch_lsq_givens_batch).  The host reads back only how many still run, 4 bytes per
// iteration; a batched iteration is long (milliseconds at k = 2000), so that wait costs less
// than running one iteration past the last stop would.
int gmres_batch(ifgf2d_ctx* ctx, const double2* b, double2* x, int B, int mode, const std::vector<double>& tol, int restart,
                int max_iters, const std::vector<char>& skip, std::vector<int>& iters, std::vector<double>& est,
                int gs_passes = 2, SpectralWork* spec = nullptr) {
    const long long N = ctx->D.N;
    const int m = (int)std::min<long long>(restart, N);
    int rc = ensure_solve(ctx, B, m);
    if (rc != IFGF2D_OK) return rc;
    BatchWork& W = *ctx->bw;
    if (spec && (W.zcap < W.scap || W.zm != m)) {   // flexible: the preconditioned columns Z
        CK(W.Z.alloc((size_t)N * W.scap * m));
        CK(W.ug.alloc((size_t)spectral_grid_size(spec) * W.scap));
        W.zcap = W.scap; W.zm = m;
    }
    cudaStream_t s = ctx->stream;
    const long long nb = N * B;
    const int ldh = m + 1;
    CK(cudaMemsetAsync(x, 0, sizeof(double2) * nb, s));
    iters.assign(B, 0);
    est.assign(B, 0.0);
    std::vector<double> beta, r0n;
    if ((rc = bnorms(ctx, b, B, beta))) return rc;
    r0n = beta;
    std::vector<char> done(B, 0);
    for (int r = 0; r < B; ++r) {
        done[r] = skip[r] || beta[r] == 0.0;
        est[r] = done[r] ? 0.0 : 1.0;
    }
    CK(cudaMemcpyAsync(W.w.p, b, sizeof(double2) * nb, cudaMemcpyDeviceToDevice, s));
    const LsqBatchDev L{W.lsR.p, W.lsg.p, W.lsgc.p, W.lsgs.p, W.lsst.p, W.lssc.p, m, B};
    // pinned host mirror: per-RHS parameters (3 B doubles), estimates (3 B doubles), states
    // (4 B ints), running counts (m ints)
    const size_t pin_bytes = sizeof(double) * 6 * B + sizeof(int) * (4 * B + m);
    char* pin = reinterpret_cast<char*>(pinned_scratch((pin_bytes + 15) / 16));
    if (!pin) return fail(ctx, IFGF2D_ERR_CUDA, "cudaMallocHost of the GMRES read-back buffer failed");
    double* h_par = reinterpret_cast<double*>(pin);
    double* h_sc = h_par + 3 * B;
    int* h_st = reinterpret_cast<int*>(h_sc + 3 * B);
    int* h_act = h_st + 4 * B;
    auto all_done = [&]() { for (int r = 0; r < B; ++r) if (!done[r]) return false; return true; };
    const long long cap = std::min<long long>(max_iters, N);
    while (!all_done()) {
        // v_0 = r / ||r|| (W.hn holds ||r|| per RHS; 0 gives a zero vector)
        launch_bscale(W.w.p, W.hn.p, N, B, W.V.p, s);
        CK(cudaMemsetAsync(W.H.p, 0, sizeof(double2) * (size_t)m * ldh * B, s));
        for (int r = 0; r < B; ++r) {
            h_par[3 * r] = r0n[r];
            h_par[3 * r + 1] = tol[r];
            h_par[3 * r + 2] = done[r] ? 0.0 : (double)std::max<long long>(0, cap - iters[r]);
        }
        CK(cudaMemcpyAsync(W.lspar.p, h_par, sizeof(double) * 3 * B, cudaMemcpyHostToDevice, s));
        launch_lsq_init_batch(L, W.hn.p, W.lspar.p, s);
        int ncols = 0;
        for (int j = 0; j < m; ++j) {
            double2* vj = W.V.p + (long long)j * nb;
            double2* Hcol = W.H.p + (long long)j * ldh * B;
            const double2* src = vj;
            if (spec) {   // flexible GMRES: z_j = M v_j, w = A z_j
                double2* zj = W.Z.p + (long long)j * nb;
                spectral_launch_batch(spec, vj, zj, B, W.ug.p, ctx->D.Np, s);
                src = zj;
            }
            if ((rc = apply_il(ctx, src, W.w.p, B, mode))) return rc;
            for (int pass = 0; pass < gs_passes; ++pass) {   // classical Gram-Schmidt, once or twice
                launch_bdot(W.V.p, nb, j + 1, W.w.p, N, B, W.part.p, W.h.p, Hcol, pass, -1, s);
                launch_bupdate(W.V.p, nb, j + 1, W.h.p, -1.0, N, B, W.w.p, s);
            }
            launch_bdot(W.w.p, 0, 1, W.w.p, N, B, W.part.p, nullptr, Hcol, 0, j + 1, s);
            launch_bscale(W.w.p, Hcol + (long long)(j + 1) * B, N, B, W.V.p + (long long)(j + 1) * nb, s);
            launch_lsq_givens_batch(Hcol, j, L, W.lsact.p, s);
            CK(cudaMemcpyAsync(h_act + j, W.lsact.p + j, sizeof(int), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            ncols = j + 1;
            if (h_act[j] == 0) break;
        }
        // y_r = R_r^{-1} g_r over its own column count, x += V Y
        launch_lsq_solve_batch(L, ncols, W.Y.p, s);
        launch_bupdate(spec ? W.Z.p : W.V.p, nb, ncols, W.Y.p, 1.0, N, B, x, s);   // x += V Y, or Z Y (flexible)
        CK(cudaMemcpyAsync(h_sc, W.lssc.p, sizeof(double) * 3 * B, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(h_st, W.lsst.p, sizeof(int) * 4 * B, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        CK(cudaGetLastError());
        for (int r = 0; r < B; ++r) {
            if (done[r]) continue;
            iters[r] += h_st[4 * r + 3];
            est[r] = h_sc[3 * r];
            if (h_st[4 * r] || h_st[4 * r + 3] <= 0) done[r] = 1;
        }
        if (all_done()) break;
        // restart: r = b - A x; the estimate keeps the first ||r0|| (opGMRES.hpp:207)
        if ((rc = apply_il(ctx, x, W.t.p, B, mode))) return rc;
        launch_sub(b, W.t.p, nb, W.w.p, s);
        if ((rc = bnorms(ctx, W.w.p, B, beta))) return rc;
        for (int r = 0; r < B; ++r) if (!done[r] && beta[r] == 0.0) { done[r] = 1; est[r] = 0.0; }
    }
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

// Gram-Schmidt passes of the complex64 inner solves.  They stop at a relative residual of 2e-7
// or more, and every correction is checked by the FP64 residual of the refinement; one
// classical pass (half the basis traffic of two) keeps them at their iteration counts, and a
// correction that came out short costs one more refinement pass, not a wrong answer.  The FP64
// solves keep the second pass.
constexpr int kInnerGsPasses = 1;

// solve B <= kMaxBatch interleaved right-hand sides W.b into W.x
int solve_il(ifgf2d_ctx* ctx, int B, int mode, double tol, int restart, int max_iters, std::vector<int>& iters,
             std::vector<double>& est, SpectralWork* spec = nullptr) {
    BatchWork& W = *ctx->bw;
    const long long N = ctx->D.N;
    const long long nb = N * B;
    cudaStream_t s = ctx->stream;
    int rc;
    if (mode != IFGF2D_APPLY_IFGF_MIXED) {
        std::vector<double> tv(B, tol);
        std::vector<char> skip(B, 0);
        return gmres_batch(ctx, W.b.p, W.x.p, B, mode, tv, restart, max_iters, skip, iters, est, 2, spec);
    }
    // FP64 iterative refinement per right-hand side, as ifgf2d_solve: residual with the FP64
    // operator, correction from GMRES on the complex64 operator
    std::vector<double> bn, rn;
    if ((rc = bnorms(ctx, W.b.p, B, bn))) return rc;
    rn = bn;
    iters.assign(B, 0);
    est.assign(B, 0.0);
    std::vector<char> done(B, 0);
    for (int r = 0; r < B; ++r) { est[r] = bn[r] > 0 ? 1.0 : 0.0; done[r] = est[r] < tol; }
    CK(cudaMemsetAsync(W.x.p, 0, sizeof(double2) * nb, s));
    CK(cudaMemcpyAsync(W.r.p, W.b.p, sizeof(double2) * nb, cudaMemcpyDeviceToDevice, s));
    std::vector<double> itol(B);
    std::vector<int> it;
    std::vector<double> e;
    int passes = 0;
    for (int outer = 0; outer < 30; ++outer) {
        std::vector<int> act;
        int most = 0;
        for (int r = 0; r < B; ++r) {
            if (!done[r] && iters[r] < max_iters) act.push_back(r);
            most = std::max(most, iters[r]);
            itol[r] = std::max(2e-7, 0.3 * tol * bn[r] / std::max(rn[r], 1e-300));
        }
        if (act.empty()) break;
        ++passes;
        const int Bc = (int)act.size();
        if (Bc == B) {
            std::vector<char> skip(B, 0);
            if ((rc = gmres_batch(ctx, W.r.p, W.d.p, B, IFGF2D_APPLY_IFGF_MIXED, itol, restart, std::max(1, max_iters - most),
                                  skip, it, e, kInnerGsPasses, spec)))
                return rc;
            for (int r = 0; r < B; ++r) iters[r] += it[r];
            launch_bupdate(W.d.p, 0, 1, W.ones.p, 1.0, N, B, W.x.p, s);   // x += d
            if ((rc = apply_il(ctx, W.x.p, W.t.p, B, IFGF2D_APPLY_IFGF))) return rc;
            launch_sub(W.b.p, W.t.p, nb, W.r.p, s);
            if ((rc = bnorms(ctx, W.r.p, B, rn))) return rc;
        } else {
            // only the columns still short of the tolerance: the batched applies cost in
            // proportion to their columns, frozen ones included
            const size_t nc = (size_t)N * Bc;
            if (W.cb.n < nc) {
                CK(W.cb.alloc((size_t)N * B)); CK(W.cx.alloc((size_t)N * B)); CK(W.cr.alloc((size_t)N * B));
                CK(W.cd.alloc((size_t)N * B)); CK(W.ct.alloc((size_t)N * B));
            }
            CK(W.act.upload(act));
            std::vector<double> itc(Bc), rnc;
            for (int j = 0; j < Bc; ++j) itc[j] = itol[act[j]];
            std::vector<char> skip(Bc, 0);
            launch_gather_cols(W.r.p, B, W.act.p, Bc, N, W.cr.p, s);
            if ((rc = gmres_batch(ctx, W.cr.p, W.cd.p, Bc, IFGF2D_APPLY_IFGF_MIXED, itc, restart, std::max(1, max_iters - most),
                                  skip, it, e, kInnerGsPasses, spec)))
                return rc;
            for (int j = 0; j < Bc; ++j) iters[act[j]] += it[j];
            launch_scatter_cols(W.cd.p, Bc, W.act.p, B, N, true, W.x.p, s);   // x += d on the active columns
            launch_gather_cols(W.x.p, B, W.act.p, Bc, N, W.cx.p, s);
            launch_gather_cols(W.b.p, B, W.act.p, Bc, N, W.cb.p, s);
            if ((rc = apply_il(ctx, W.cx.p, W.ct.p, Bc, IFGF2D_APPLY_IFGF))) return rc;
            launch_sub(W.cb.p, W.ct.p, (long long)nc, W.cr.p, s);
            launch_scatter_cols(W.cr.p, Bc, W.act.p, B, N, false, W.r.p, s);
            if ((rc = bnorms(ctx, W.cr.p, Bc, rnc))) return rc;
            for (int j = 0; j < Bc; ++j) rn[act[j]] = rnc[j];
        }
        for (int r : act) {
            est[r] = bn[r] > 0 ? rn[r] / bn[r] : 0.0;
            if (est[r] < tol) done[r] = 1;
        }
    }
    ctx->last_passes = passes;
    return IFGF2D_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" int ifgf2d_apply_batch_device(ifgf2d_ctx* ctx, const void* d_x, void* d_y, int nrhs, int mode) {
    if (!ctx || nrhs < 0 || (nrhs > 0 && (!d_x || !d_y))) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    int rc = check_mode(ctx, mode);
    if (rc != IFGF2D_OK || nrhs == 0) return rc;
    return apply_cm(ctx, (const double2*)d_x, (double2*)d_y, nrhs, mode);
}

extern "C" int ifgf2d_apply_batch(ifgf2d_ctx* ctx, const double* x, double* y, int nrhs, int mode) {
    if (!ctx || nrhs < 0 || (nrhs > 0 && (!x || !y))) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    int rc = check_mode(ctx, mode);
    if (rc != IFGF2D_OK || nrhs == 0) return rc;
    const long long N = ctx->D.N;
    if (!all_finite(x, 2 * N * nrhs)) return fail(ctx, IFGF2D_ERR_NONFINITE, "non-finite value in the densities");
    const int chunk = std::min(nrhs, kMaxBatch);
    if (!ctx->bw) ctx->bw = new BatchWork;
    BatchWork& W = *ctx->bw;
    if (W.xcm.n < (size_t)N * chunk) { CK(W.xcm.alloc((size_t)N * chunk)); CK(W.ycm.alloc((size_t)N * chunk)); }
    for (int r0 = 0; r0 < nrhs; r0 += chunk) {
        const int B = std::min(chunk, nrhs - r0);
        const size_t bytes = sizeof(double2) * (size_t)N * B;
        CK(cudaMemcpyAsync(W.xcm.p, x + 2 * (size_t)N * r0, bytes, cudaMemcpyHostToDevice, ctx->stream));
        if ((rc = apply_cm(ctx, W.xcm.p, W.ycm.p, B, mode))) return rc;
        CK(cudaMemcpyAsync(y + 2 * (size_t)N * r0, W.ycm.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return check_t5(ctx);
}

namespace {
int solve_batch(ifgf2d_ctx* ctx, const double* rhs, double* x, int nrhs, int mode, double tol, int restart, int max_iters,
                int* iters, double* est_error, SpectralWork* spec) {
    int rc = check_mode(ctx, mode);
    if (rc != IFGF2D_OK || nrhs == 0) return rc;
    const long long N = ctx->D.N;
    if (!all_finite(rhs, 2 * N * nrhs)) return fail(ctx, IFGF2D_ERR_NONFINITE, "non-finite value in the right-hand sides");
    bool all_ok = true;
    if (mode == IFGF2D_APPLY_DIRECT) {   // one right-hand side at a time
        for (int r = 0; r < nrhs; ++r) {
            int it = 0; double e = 0.0;
            rc = ifgf2d_solve(ctx, rhs + 2 * (size_t)N * r, x + 2 * (size_t)N * r, mode, tol, restart, max_iters, &it, &e);
            if (rc != IFGF2D_OK && rc != IFGF2D_ERR_NOCONV) return rc;
            all_ok = all_ok && rc == IFGF2D_OK;
            if (iters) iters[r] = it;
            if (est_error) est_error[r] = e;
        }
        return all_ok ? IFGF2D_OK : IFGF2D_ERR_NOCONV;
    }
    const int chunk = std::min(nrhs, kMaxBatch);
    if ((rc = ensure_apply(ctx, chunk, mode == IFGF2D_APPLY_IFGF_MIXED))) return rc;
    if (mode == IFGF2D_APPLY_IFGF_MIXED && (rc = ensure_apply(ctx, chunk, false))) return rc;
    if ((rc = ensure_solve(ctx, chunk, (int)std::min<long long>(restart, N)))) return rc;
    BatchWork& W = *ctx->bw;
    if (W.xcm.n < (size_t)N * chunk) { CK(W.xcm.alloc((size_t)N * chunk)); CK(W.ycm.alloc((size_t)N * chunk)); }
    cudaStream_t s = ctx->stream;
    for (int r0 = 0; r0 < nrhs; r0 += chunk) {
        const int B = std::min(chunk, nrhs - r0);
        const size_t bytes = sizeof(double2) * (size_t)N * B;
        CK(cudaMemcpyAsync(W.xcm.p, rhs + 2 * (size_t)N * r0, bytes, cudaMemcpyHostToDevice, s));
        launch_interleave(W.xcm.p, N, B, W.b.p, s);
        std::vector<int> it;
        std::vector<double> e;
        if ((rc = solve_il(ctx, B, mode, tol, restart, max_iters, it, e, spec))) return rc;
        launch_deinterleave(W.x.p, N, B, W.ycm.p, s);
        CK(cudaMemcpyAsync(x + 2 * (size_t)N * r0, W.ycm.p, bytes, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if ((rc = check_t5(ctx))) return rc;
        for (int r = 0; r < B; ++r) {
            if (iters) iters[r0 + r] = it[r];
            if (est_error) est_error[r0 + r] = e[r];
            all_ok = all_ok && e[r] < tol;
        }
    }
    return all_ok ? IFGF2D_OK : IFGF2D_ERR_NOCONV;
}
}  // namespace

extern "C" int ifgf2d_solve_batch(ifgf2d_ctx* ctx, const double* rhs, double* x, int nrhs, int mode, double tol, int restart,
                                  int max_iters, int* iters, double* est_error) {
    if (!ctx || nrhs < 0 || (nrhs > 0 && (!rhs || !x)) || restart <= 0 || max_iters <= 0) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    return solve_batch(ctx, rhs, x, nrhs, mode, tol, restart, max_iters, iters, est_error, nullptr);
}

extern "C" int ifgf2d_solve_batch_flexible(ifgf2d_ctx* ctx, int precond, const double* rhs, double* x, int nrhs, int mode,
                                           double tol, int restart, int max_iters, int* iters, double* est_error) {
    if (!ctx || nrhs < 0 || (nrhs > 0 && (!rhs || !x)) || restart <= 0 || max_iters <= 0) return IFGF2D_ERR_ARG;
    if (precond != IFGF2D_PRECOND_SPECTRAL) return fail(ctx, IFGF2D_ERR_ARG, "batched solves take the spectral preconditioner only");
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_IFGF_MIXED) return fail(ctx, IFGF2D_ERR_ARG, "batched flexible solves are IFGF or IFGF_MIXED");
    AllocStream guard(ctx->stream);
    int rc = check_mode(ctx, mode);
    if (rc != IFGF2D_OK) return rc;
    if (!ctx->sw && (rc = spectral_setup(ctx, IFGF2D_SPECTRAL_DEFAULT_SCALE)) != IFGF2D_OK) return rc;
    return solve_batch(ctx, rhs, x, nrhs, mode, tol, restart, max_iters, iters, est_error, ctx->sw);
}
