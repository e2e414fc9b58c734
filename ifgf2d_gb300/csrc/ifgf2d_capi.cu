#include <atomic>
#include <mutex>
// ifgf2d_capi.cu -- the C ABI (include/ifgf2d.h): context, set-up, apply, GMRES, propagation.
//
// Host orchestration of the GB300 forward map.  The context owns every device buffer; set-up
// sizes them once, so an apply or a GMRES iteration allocates nothing.
#include <cuda_runtime.h>
#include <algorithm>
#include <complex>
#include <cstring>
#include <string>
#include <vector>
#include <memory>

#include "context.hpp"
#include "direct_view.hpp"
#include "host_threads.hpp"

using namespace ifgf;


// ------------------------------------------------------------------ create / destroy
extern "C" int ifgf2d_create(const ifgf2d_curve* curves, int ncurves, const ifgf2d_junction* junctions, int njunctions,
                             const ifgf2d_options* opts, ifgf2d_ctx** out) {
    if (!out || !opts) return IFGF2D_ERR_ARG;
    *out = nullptr;
    ifgf2d_ctx* ctx = new ifgf2d_ctx;
    ctx->opt = *opts;
    if (ctx->opt.Ps <= 0) ctx->opt.Ps = 5;
    if (ctx->opt.Pang <= 0) ctx->opt.Pang = 5;
    {
        // cone interpolants compiled for the device (IFGF_DISPATCH_P in ifgf2d_kernels.cu)
        const int ps = ctx->opt.Ps, pa = ctx->opt.Pang;
        const bool ok = (ps == 5 && pa == 5) || (ps == 5 && pa == 7) || (ps == 3 && pa == 5) || (ps == 3 && pa == 3) ||
                        (ps == 7 && pa == 7) || (ps == 4 && pa == 4) || (ps == 6 && pa == 6);
        if (!ok) { *out = ctx; ctx->err = "(Ps, Pang) must be one of (3,3) (3,5) (4,4) (5,5) (5,7) (6,6) (7,7)"; return IFGF2D_ERR_ARG; }
        if (ctx->opt.formulation != IFGF2D_SINGLE_LAYER && ctx->opt.formulation != IFGF2D_COMBINED) {
            *out = ctx; ctx->err = "formulation must be IFGF2D_SINGLE_LAYER or IFGF2D_COMBINED"; return IFGF2D_ERR_ARG;
        }
        ctx->form = ctx->opt.formulation;
    }
    std::string msg = discretise(curves, ncurves, junctions, njunctions, ctx->opt, ctx->D);
    if (!msg.empty()) {
        // report through a context so the caller can read the message, as the reference prints it
        *out = ctx; ctx->err = msg; return IFGF2D_ERR_GEOMETRY;
    }
    *out = ctx;
    return ifgf::init_host_tables(ctx);
}

// The host tables every context derives from its discretisation: per point its near-singular
// patches, the rectangular-polar columns and, per output row, the columns adding to it.
int ifgf::init_host_tables(ifgf2d_ctx* ctx) {
    const Discretisation& D = ctx->D;
    ctx->h_nsp.clear();
    ctx->hcols.clear();
    ctx->h_srow_col.clear();
    // per point: the patches it is near-singular to (ForwardMap.tpp:596-604)
    ctx->h_nsp_ptr.assign(D.N + 1, 0);
    {
        std::vector<std::vector<int>> per(D.N);
        for (long long p = 0; p < D.num_patches; ++p)
            for (int q = D.ns_ptr[p]; q < D.ns_ptr[p + 1]; ++q) per[D.ns_idx[q]].push_back((int)p);
        for (long long i = 0; i < D.N; ++i) {
            if (per[i].size() > 8) { ctx->err = "a point is near-singular to more than 8 patches (reduce delta)"; return IFGF2D_ERR_GEOMETRY; }
            for (int p : per[i]) ctx->h_nsp.push_back(p);
            ctx->h_nsp_ptr[i + 1] = (int)ctx->h_nsp.size();
        }
    }
    // rectangular-polar columns: per patch Np singular columns then its near-singular ones
    ctx->col_ptr.assign(D.num_patches + 1, 0);
    for (long long p = 0; p < D.num_patches; ++p) {
        ctx->col_ptr[p] = (int)ctx->hcols.size();
        for (int j = 0; j < D.Np; ++j) {
            const long long i = p * D.Np + j;
            ctx->hcols.push_back(RPColumn{(int)p, 0, D.t[i], D.x[i], D.y[i]});
        }
        for (int q = D.ns_ptr[p]; q < D.ns_ptr[p + 1]; ++q)
            ctx->hcols.push_back(RPColumn{(int)p, 0, D.ns_t[q], D.x[D.ns_idx[q]], D.y[D.ns_idx[q]]});
    }
    ctx->col_ptr[D.num_patches] = (int)ctx->hcols.size();
    // per output row: the columns that add to it, in patch order (ForwardMap.tpp:486-512)
    {
        std::vector<std::vector<std::pair<int, int>>> rows(D.N);
        for (long long p = 0; p < D.num_patches; ++p) {
            for (int j = 0; j < D.Np; ++j) rows[p * D.Np + j].push_back({(int)p, ctx->col_ptr[p] + j});
            for (int q = D.ns_ptr[p]; q < D.ns_ptr[p + 1]; ++q)
                rows[D.ns_idx[q]].push_back({(int)p, ctx->col_ptr[p] + D.Np + (q - D.ns_ptr[p])});
        }
        ctx->h_srow_ptr.assign(D.N + 1, 0);
        for (long long i = 0; i < D.N; ++i) {
            std::sort(rows[i].begin(), rows[i].end());
            for (auto& e : rows[i]) ctx->h_srow_col.push_back(e.second);
            ctx->h_srow_ptr[i + 1] = (int)ctx->h_srow_col.size();
        }
    }
    return IFGF2D_OK;
}

// Device-side copies of the discretisation; made on first use so that the constructor, like
// the reference's, is host work only.
static int ensure_device(ifgf2d_ctx* ctx) {
    if (ctx->device_ready) return IFGF2D_OK;
    CK(cudaGetDevice(&ctx->device));
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    keep_pool_memory(ctx->device);
    AllocStream guard(ctx->stream);
    const Discretisation& D = ctx->D;
    CK(ctx->x.upload(D.x)); CK(ctx->y.upload(D.y)); CK(ctx->wq.upload(D.wq)); CK(ctx->edge.upload(D.edge_jac));
    CK(ctx->nx.upload(D.nx)); CK(ctx->ny.upload(D.ny));
    CK(ctx->patch_of.upload(D.patch_of));
    std::vector<DevCurve> dc(D.curves.size());
    for (size_t c = 0; c < D.curves.size(); ++c) { dc[c].type = D.curves[c].type; dc[c].pad = 0; std::memcpy(dc[c].p, D.curves[c].p, sizeof(dc[c].p)); }
    CK(ctx->curves.upload(dc));
    std::vector<DevPatch> dp(D.num_patches);
    for (long long p = 0; p < D.num_patches; ++p) dp[p] = DevPatch{D.t1[p], D.t2[p], D.curve_of[p], D.ist1sing[p], D.ist2sing[p], 0};
    CK(ctx->patches.upload(dp));
    CK(ctx->nsn.upload(D.fej_ns_n)); CK(ctx->nsw.upload(D.fej_ns_w));
    CK(ctx->nsp_ptr.upload(ctx->h_nsp_ptr)); CK(ctx->nsp.upload(ctx->h_nsp));
    CK(ctx->cols.upload(ctx->hcols));
    CK(ctx->srow_ptr.upload(ctx->h_srow_ptr)); CK(ctx->srow_col.upload(ctx->h_srow_col));
    CK(ctx->rho.alloc(D.N)); CK(ctx->vin.alloc(D.N)); CK(ctx->vout.alloc(D.N));
    ctx->device_ready = true;
    return IFGF2D_OK;
}

double2* ifgf::pinned_scratch(size_t n) {
    struct Scratch {
        double2* p = nullptr;
        size_t n = 0;
        ~Scratch() { if (p) cudaFreeHost(p); }
    };
    static thread_local Scratch sc;
    if (sc.n < n) {
        if (sc.p) cudaFreeHost(sc.p);
        sc.p = nullptr;
        sc.n = 0;
        if (cudaMallocHost((void**)&sc.p, n * sizeof(double2)) != cudaSuccess) { sc.p = nullptr; return nullptr; }
        sc.n = n;
    }
    return sc.p;
}

void ifgf::keep_pool_memory(int device) {
    static std::mutex mu;
    static std::vector<int> done;
    std::lock_guard<std::mutex> lock(mu);
    if (std::find(done.begin(), done.end(), device) != done.end()) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = ~0ull;   // freed blocks stay in the pool for the next context's set-up
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done.push_back(device);
}

extern "C" int ifgf2d_destroy(ifgf2d_ctx* ctx) {
    if (!ctx) return IFGF2D_ERR_ARG;
    cudaStream_t s = ctx->stream;
    if (s) cudaStreamSynchronize(s);
    {
        AllocStream guard(s);
        free_batch(ctx);
        free_eval(ctx);
        free_spectral(ctx);
        delete ctx;   // buffers allocated on s are freed on s, before s goes
    }
    if (s) cudaStreamDestroy(s);
    return IFGF2D_OK;
}
extern "C" int ifgf2d_set_host_threads(int n) {
    if (n < 0) return IFGF2D_ERR_ARG;
    host_thread_limit().store(n);
    return IFGF2D_OK;
}
extern "C" const char* ifgf2d_last_error(const ifgf2d_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }
extern "C" long long ifgf2d_num_unknowns(const ifgf2d_ctx* ctx) { return ctx ? ctx->D.N : -1; }
extern "C" long long ifgf2d_num_patches(const ifgf2d_ctx* ctx) { return ctx ? ctx->D.num_patches : -1; }
extern "C" void* ifgf2d_stream(ifgf2d_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }
extern "C" int ifgf2d_get_nlevels(const ifgf2d_ctx* ctx) { return ctx ? ctx->nlevels : -1; }

extern "C" int ifgf2d_get_points(const ifgf2d_ctx* ctx, double* xs, double* ys, double* nxs, double* nys) {
    if (!ctx) return IFGF2D_ERR_ARG;
    const Discretisation& D = ctx->D;
    if (xs) std::copy(D.x.begin(), D.x.end(), xs);
    if (ys) std::copy(D.y.begin(), D.y.end(), ys);
    if (nxs) std::copy(D.nx.begin(), D.nx.end(), nxs);
    if (nys) std::copy(D.ny.begin(), D.ny.end(), nys);
    return IFGF2D_OK;
}
extern "C" int ifgf2d_get_patches(const ifgf2d_ctx* ctx, double* t1t2, long long* ns_count) {
    if (!ctx) return IFGF2D_ERR_ARG;
    const Discretisation& D = ctx->D;
    for (long long p = 0; p < D.num_patches; ++p) {
        if (t1t2) { t1t2[2 * p] = D.t1[p]; t1t2[2 * p + 1] = D.t2[p]; }
        if (ns_count) ns_count[p] = D.ns_ptr[p + 1] - D.ns_ptr[p];
    }
    return IFGF2D_OK;
}
extern "C" int ifgf2d_get_near_singular(const ifgf2d_ctx* ctx, long long* idx, double* t) {
    if (!ctx) return IFGF2D_ERR_ARG;
    for (size_t q = 0; q < ctx->D.ns_idx.size(); ++q) { if (idx) idx[q] = ctx->D.ns_idx[q]; if (t) t[q] = ctx->D.ns_t[q]; }
    return IFGF2D_OK;
}

// ------------------------------------------------------------------ rectangular-polar precomputation
// ForwardMap::compute_precomputations in two halves: the launch of the rectangular-polar
// weights on the context's stream, and the wait for them with the bookkeeping.  ifgf2d_setup
// builds the host tree between the two, while the GPU computes the weights.
static int precompute_launch(ifgf2d_ctx* ctx, double k) {
    if (!(k > 0)) return fail(ctx, IFGF2D_ERR_ARG, "wavenumber must be real and > 0");
    if (int rc = ensure_device(ctx)) return rc;
    AllocStream guard(ctx->stream);
    const Discretisation& D = ctx->D;
    const int ncols = (int)ctx->hcols.size();
    CK(ctx->M.alloc((size_t)ncols * D.Np));
    CK(ctx->W.alloc((size_t)ncols * D.Np));
    ctx->eta = ctx->opt.coupling > 0 ? ctx->opt.coupling : k;
    launch_rp_precompute(ctx->cols.p, ncols, ctx->patches.p, ctx->curves.p, ctx->nsn.p, ctx->nsw.p, D.Np, D.p, k, ctx->form,
                         ctx->eta, ctx->M.p, ctx->stream);
    CK(cudaGetLastError());
    launch_rp_fold(ctx->M.p, ctx->cols.p, ncols, ctx->edge.p, ctx->patches.p, D.Np, ctx->W.p, ctx->stream);
    CK(cudaGetLastError());
    return IFGF2D_OK;
}
static int precompute_finish(ifgf2d_ctx* ctx, double k) {
    AllocStream guard(ctx->stream);
    const Discretisation& D = ctx->D;
    const int ncols = (int)ctx->hcols.size();
    CK(cudaStreamSynchronize(ctx->stream));
    if (ifgf::noalloc_prepare(ctx->device) != IFGF2D_OK)
        return fail(ctx, IFGF2D_ERR_CUDA, "loading the scratch array of ifgf2d_apply_direct_noalloc failed");
    ctx->k = k;
    ctx->precomputed = true;
    ctx->ifgf_ready = false;
    if (ctx->gw) ctx->gw->drop_graphs();
    free_batch(ctx);
    free_eval(ctx);
    free_spectral(ctx);
    ctx->counts[6] = (long long)ncols * D.Np;
    return IFGF2D_OK;
}

extern "C" int ifgf2d_precompute(ifgf2d_ctx* ctx, double k) {
    if (!ctx) return IFGF2D_ERR_ARG;
    if (int rc = precompute_launch(ctx, k)) return rc;
    return precompute_finish(ctx, k);
}

extern "C" int ifgf2d_get_precomputations(ifgf2d_ctx* ctx, long long patch, double* out) {
    if (!ctx || !out || patch < 0 || patch >= ctx->D.num_patches) return IFGF2D_ERR_ARG;
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute first");
    const int c0 = ctx->col_ptr[patch], c1 = ctx->col_ptr[patch + 1];
    CK(cudaStreamSynchronize(ctx->stream));   // the table was written (and allocated) on the context's stream
    CK(cudaMemcpy(out, ctx->M.p + (size_t)c0 * ctx->D.Np, sizeof(double2) * (size_t)(c1 - c0) * ctx->D.Np, cudaMemcpyDeviceToHost));
    return IFGF2D_OK;
}

// ------------------------------------------------------------------ IFGF set-up
// BoxTree::CheckIfSingandNearSingInNeighborhood (BoxTree.h:1079-1161) on leaf box coordinates
// Every pair of a patch's points is adjacent exactly when the patch's leaf-box range spans at
// most two boxes in x and in y, and a near-singular point is adjacent to all of a patch's points
// exactly when it lies within one box of that whole range; so each patch needs its range only.
static bool neighbourhood_ok(const Discretisation& D, int nlevels) {
    double mx, my, size;
    tree_root_box(D.x, D.y, mx, my, size);
    const int lev = nlevels - 1;
    const double bs = size / (double)(1LL << lev);
    const long long side = 1LL << lev;
    auto box = [&](long long i, long long& bx, long long& by) {
        bx = (long long)((D.x[i] - mx) / bs); by = (long long)((D.y[i] - my) / bs);
        return bx >= 0 && by >= 0 && bx < side && by < side;
    };
    std::atomic<bool> ok{true};
    parallel_for(D.num_patches, [&](long long p0, long long p1) {
        for (long long p = p0; p < p1 && ok.load(std::memory_order_relaxed); ++p) {
            long long x0 = side, x1 = -1, y0 = side, y1 = -1, bx, by;
            for (long long i = p * D.Np; i < (p + 1) * D.Np; ++i) {
                if (!box(i, bx, by)) { ok = false; break; }
                x0 = std::min(x0, bx); x1 = std::max(x1, bx); y0 = std::min(y0, by); y1 = std::max(y1, by);
            }
            if (!ok.load(std::memory_order_relaxed)) break;
            if (x1 - x0 > 1 || y1 - y0 > 1) { ok = false; break; }
            for (int q = D.ns_ptr[p]; q < D.ns_ptr[p + 1]; ++q) {
                if (!box(D.ns_idx[q], bx, by) || bx > x0 + 1 || bx < x1 - 1 || by > y0 + 1 || by < y1 - 1) { ok = false; break; }
            }
        }
    }, 64);
    return ok.load();
}

// the tree depth: the requested one, checked, or (request <= 0) the deepest whose leaf
// neighbourhoods hold every singular and near-singular pair
static int choose_levels(ifgf2d_ctx* ctx, int& nlevels) {
    const Discretisation& D = ctx->D;
    if (nlevels <= 0) {
        nlevels = 0;
        for (int nl = 16; nl >= 3; --nl) if (neighbourhood_ok(D, nl)) { nlevels = nl; break; }
        if (!nlevels) return fail(ctx, IFGF2D_ERR_NEIGHBORHOOD, "no tree depth >= 3 keeps singular points in the leaf neighbourhood");
    } else {
        if (nlevels < 3) return fail(ctx, IFGF2D_ERR_NLEVELS, "IFGF accelerator requires at least 3 levels.");
        if (nlevels > 20) return fail(ctx, IFGF2D_ERR_NLEVELS, "nlevels too large");
        if (!neighbourhood_ok(D, nlevels)) return fail(ctx, IFGF2D_ERR_NEIGHBORHOOD, "Singular point not in neighborhood");
    }
    return IFGF2D_OK;
}

static void record_counts(ifgf2d_ctx* ctx, int nlevels) {
    const Tree& T = ctx->T;
    ctx->counts[0] = T.near_pairs; ctx->counts[1] = T.leaf_evals; ctx->counts[2] = T.prop_evals;
    ctx->counts[3] = T.interp_evals; ctx->counts[4] = T.total_cones; ctx->counts[5] = nlevels;
}

// the host part of the set-up: tree depth, neighbourhood check, tree and plans (no CUDA call)
extern "C" int ifgf2d_prepare(ifgf2d_ctx* ctx, double k, int nlevels) {
    if (!ctx) return IFGF2D_ERR_ARG;
    if (!(k > 0)) return fail(ctx, IFGF2D_ERR_ARG, "wavenumber must be real and > 0");
    const int request = nlevels;
    const Discretisation& D = ctx->D;
    if (int rc = choose_levels(ctx, nlevels)) return rc;
    // the device tables no longer match the host tree from here until ifgf2d_setup completes
    ctx->ifgf_ready = false;
    ctx->prep_ready = false;
    std::string msg = build_tree(D.x, D.y, nlevels, k, ctx->opt.Ps, ctx->opt.Pang, ctx->T);
    if (!msg.empty()) return fail(ctx, IFGF2D_ERR_GEOMETRY, msg);
    ctx->prep_ready = true;
    ctx->prep_k = k;
    ctx->prep_request = request;
    ctx->prep_nlevels = nlevels;
    ctx->nlevels = nlevels;
    record_counts(ctx, nlevels);
    return IFGF2D_OK;
}

static int setup_boxes(ifgf2d_ctx* ctx, double k, int nlevels, const SetupExtra* ex);
static int setup_cones(ifgf2d_ctx* ctx, double k, int nlevels, const SetupExtra* ex, DBuf<int>& perr,
                       PropPlanByLevel* by_level = nullptr);
static int setup_interp(ifgf2d_ctx* ctx, int nlevels, DBuf<int>& perr);

// ForwardMap::precomps_and_setup.  Host and GPU take turns so that each works while the other
// does: the host builds the tree's boxes; the GPU computes the near-field table, the
// rectangular-polar weights and, level by level on a second stream, the propagation plan while
// the host builds the cones; the GPU computes the leaf-cone tables while the host builds the
// interpolation plan.  A tree that ifgf2d_prepare built beforehand is used as it is.
extern "C" int ifgf2d_setup(ifgf2d_ctx* ctx, double k, int nlevels) {
    if (!ctx) return IFGF2D_ERR_ARG;
    if (!(k > 0)) return fail(ctx, IFGF2D_ERR_ARG, "wavenumber must be real and > 0");
    const bool pre = !ctx->precomputed || ctx->k != k;
    if (ctx->prep_ready && ctx->prep_k == k && ctx->prep_request == nlevels) {
        if (pre) {
            if (int rc = precompute_launch(ctx, k)) return rc;
            if (int rc = precompute_finish(ctx, k)) return rc;
        }
        AllocStream guard(ctx->stream);
        ctx->prep_ready = false;
        return ifgf::setup_tables(ctx, k, ctx->prep_nlevels, nullptr);
    }
    // a failed tree still leaves the weights computed, as the reference's order has them
    const Discretisation& D = ctx->D;
    int nl = nlevels;
    std::string msg;
    int rc = choose_levels(ctx, nl);
    if (rc == IFGF2D_OK) {
        ctx->ifgf_ready = false;
        ctx->prep_ready = false;
        msg = build_tree_boxes(D.x, D.y, nl, k, ctx->opt.Ps, ctx->opt.Pang, ctx->T);
        if (!msg.empty()) rc = fail(ctx, IFGF2D_ERR_GEOMETRY, msg);
    }
    if (int r = ensure_device(ctx)) return r;
    DBuf<int> perr;
    {   // the near-field table's uploads go first, while the stream is idle
        AllocStream guard(ctx->stream);
        if (pre) ctx->eta = ctx->opt.coupling > 0 ? ctx->opt.coupling : k;
        if (rc == IFGF2D_OK) rc = setup_boxes(ctx, k, nl, nullptr);
    }
    if (pre) {
        if (int r = precompute_launch(ctx, k)) return r;
    }
    AllocStream guard(ctx->stream);
    PropPlanByLevel by_level;
    if (rc == IFGF2D_OK) {
        msg = build_tree_cones(ctx->T, [&](int l) { if (l > 2) by_level.add(ctx->T, l); });
        if (!msg.empty()) rc = fail(ctx, IFGF2D_ERR_GEOMETRY, msg);
    }
    if (pre) {   // waits for the weights (and the near-field table)
        const std::string err = ctx->err;
        if (int r = precompute_finish(ctx, k)) return r;
        ctx->err = err;
    }
    if (rc != IFGF2D_OK) return rc;
    if (int rc2 = setup_cones(ctx, k, nl, nullptr, perr, &by_level)) return rc2;
    msg = build_tree_interp(ctx->T);
    if (!msg.empty()) {
        cudaStreamSynchronize(ctx->stream);
        return fail(ctx, IFGF2D_ERR_GEOMETRY, msg);
    }
    record_counts(ctx, nl);
    return setup_interp(ctx, nl, perr);
}

// The device tables of an IFGF set-up from the context's host tree (ctx->T) and discretisation,
// in three stages that follow the tree's (build_tree_boxes, _cones, _interp): setup_boxes needs
// the boxes, setup_cones the cones and the propagation slots, setup_interp the interpolation
// plan.  The first two only queue work on the context's stream, so the host can build the next
// stage of the tree meanwhile; setup_interp waits for all of it and then checks the
// propagation plan's error flag `perr`, which setup_cones clears.
// With `ex` (a group of obstacles, group.cu) the wavenumbers come per leaf box and leaf cone,
// the leaf-cone nodes from the members' trees, and the propagation plan from ex->build_plan.
static int setup_boxes(ifgf2d_ctx* ctx, double k, int nlevels, const SetupExtra* ex) {
    const Discretisation& D = ctx->D;
    free_batch(ctx);
    free_eval(ctx);
    ctx->ifgf_ready = false;
    Tree& T = ctx->T;
    ctx->nlevels = nlevels;
    const long long N = D.N;
    // sorted-order tables
    std::vector<int> patch_s(N), nptr(N + 1, 0), nl;
    for (long long i = 0; i < N; ++i) {
        const long long o = T.sorting[i];
        patch_s[i] = D.patch_of[o];
    }
    {   // per sorted point, the patches it is near-singular to, ascending: counted, then placed
        for (long long q = 0; q < (long long)D.ns_idx.size(); ++q) nptr[T.inverse[D.ns_idx[q]] + 1]++;
        for (long long i = 0; i < N; ++i) nptr[i + 1] += nptr[i];
        nl.resize(nptr[N]);
        std::vector<int> fill(nptr.begin(), nptr.end() - 1);
        for (long long p = 0; p < D.num_patches; ++p)
            for (int q = D.ns_ptr[p]; q < D.ns_ptr[p + 1]; ++q) nl[fill[T.inverse[D.ns_idx[q]]]++] = (int)p;
    }
    CK(ctx->sorting.upload(T.sorting)); CK(ctx->inverse.upload(T.inverse));
    CK(ctx->xs_s.upload(T.xs)); CK(ctx->ys_s.upload(T.ys));
    {
        std::vector<double> snx(N), sny(N);
        for (long long i = 0; i < N; ++i) { snx[i] = D.nx[T.sorting[i]]; sny[i] = D.ny[T.sorting[i]]; }
        CK(ctx->nxs_s.upload(snx)); CK(ctx->nys_s.upload(sny));
    }
    CK(ctx->patch_s.upload(patch_s)); CK(ctx->nsp_ptr_s.upload(nptr)); CK(ctx->nsp_s.upload(nl));
    CK(ctx->leaf_start.upload(T.leaf_start)); CK(ctx->leaf_count.upload(T.leaf_count)); CK(ctx->point_leaf.upload(T.point_leaf));
    CK(ctx->nbr_ptr.upload(T.nbr_ptr)); CK(ctx->nbr_box.upload(T.nbr_box));
    // near-field blocks
    const int nleaf = (int)T.leaf_start.size();
    std::vector<long long> noff(nleaf + 1, 0);
    for (int b = 0; b < nleaf; ++b) {
        long long nsrc = 0;
        for (int q = T.nbr_ptr[b]; q < T.nbr_ptr[b + 1]; ++q) nsrc += T.leaf_count[T.nbr_box[q]];
        noff[b + 1] = noff[b] + nsrc * T.leaf_count[b];
    }
    CK(ctx->near_off.upload(noff));
    {
        std::vector<int> rl(nleaf), soff(nleaf + 1, 0), src;
        for (int b = 0; b < nleaf; ++b) {
            rl[b] = (int)((noff[b + 1] - noff[b]) / std::max(1, T.leaf_count[b]));
            for (int q = T.nbr_ptr[b]; q < T.nbr_ptr[b + 1]; ++q)   // the row order of the near table
                for (int j = 0; j < T.leaf_count[T.nbr_box[q]]; ++j) src.push_back(T.leaf_start[T.nbr_box[q]] + j);
            soff[b + 1] = (int)src.size();
        }
        CK(ctx->near_rowlen.upload(rl));
        CK(ctx->near_src_off.upload(soff));
        CK(ctx->near_src.upload(src));
    }
    CK(ctx->near.alloc(noff[nleaf]));
    launch_near_setup(ctx->leaf_start.p, ctx->leaf_count.p, ctx->nbr_ptr.p, ctx->nbr_box.p, ctx->near_off.p, nleaf,
                      ctx->xs_s.p, ctx->ys_s.p, ctx->nxs_s.p, ctx->nys_s.p, ctx->patch_s.p, ctx->nsp_ptr_s.p, ctx->nsp_s.p, k,
                      ctx->form, ctx->eta, ctx->near.p, ctx->stream, ex ? ex->keta_leafbox : nullptr);
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

static int setup_cones(ifgf2d_ctx* ctx, double k, int nlevels, const SetupExtra* ex, DBuf<int>& perr,
                       PropPlanByLevel* by_level) {
    Tree& T = ctx->T;
    const int P = T.P, Dl = nlevels - 1;
    // values-to-coefficients matrix of the cone interpolant (Interpolator.h:81-120)
    {
        const int Ps = T.Ps, Pa = T.Pang;
        std::vector<double> xs(Ps), xa(Pa);
        for (int i = 0; i < Ps; ++i) xs[Ps - 1 - i] = std::cos(kPiH * (2.0 * i + 1.0) / (2.0 * Ps));
        for (int i = 0; i < Pa; ++i) xa[Pa - 1 - i] = std::cos(kPiH * (2.0 * i + 1.0) / (2.0 * Pa));
        auto Tn = [](int n, double x) { double a = 1.0, b = x; if (n == 0) return a; for (int i = 1; i < n; ++i) { double c = 2.0 * x * b - a; a = b; b = c; } return b; };
        std::vector<double> G((size_t)P * P);
        for (int m = 0; m < Ps; ++m)
            for (int n = 0; n < Pa; ++n)
                for (int kk = 0; kk < Ps; ++kk)
                    for (int l = 0; l < Pa; ++l) {
                        const double am = m == 0 ? 1.0 : 2.0, an = n == 0 ? 1.0 : 2.0;
                        G[(size_t)(n * Ps + m) * P + (l * Ps + kk)] = Tn(m, xs[kk]) * Tn(n, xa[l]) * (am * an / (Ps * Pa));
                    }
        CK(ctx->Gm.upload(G));
        // separable form: Gs[m][k] = (alpha_m / Ps) T_m(x_k), Ga[n][l] = (alpha_n / Pang) T_n(x_l)
        std::vector<double> Gs((size_t)Ps * Ps + (size_t)Pa * Pa);
        for (int m = 0; m < Ps; ++m)
            for (int kk = 0; kk < Ps; ++kk) Gs[(size_t)m * Ps + kk] = Tn(m, xs[kk]) * ((m == 0 ? 1.0 : 2.0) / Ps);
        for (int n = 0; n < Pa; ++n)
            for (int l = 0; l < Pa; ++l) Gs[(size_t)Ps * Ps + (size_t)n * Pa + l] = Tn(n, xa[l]) * ((n == 0 ? 1.0 : 2.0) / Pa);
        CK(ctx->Gsep.upload(Gs));
        std::vector<float> Gs32(Gs.begin(), Gs.end());
        CK(ctx->Gsep32.upload(Gs32));
    }
    // The uploads come before the kernels that follow them: a copy from pageable host memory
    // queued behind a running kernel holds the host until the kernel ends.  The leaf-cone nodes'
    // kernel is short; the propagation plan's uploads wait for it at most.
    const TreeLevel& LD = T.L[Dl];
    const int ncl = (int)LD.cone_nonrel.size();
    std::vector<long long> loff(ncl + 1, 0);
    for (int c = 0; c < ncl; ++c) loff[c + 1] = loff[c] + (long long)P * T.leaf_count[LD.cone_box[c]];
    CK(ctx->leaf_cone_box.upload(LD.cone_box)); CK(ctx->leaf_off.upload(loff));
    CK(ctx->leafL.alloc(loff[ncl]));
    CK(ctx->leaf_nodes_d.alloc((size_t)ncl * P));
    CK(ctx->pp.alloc((size_t)T.pp_total)); CK(ctx->pp32.alloc((size_t)T.pp_total));
    CK(ctx->pp_ptr.upload(T.pp_ptr)); CK(ctx->pp_nchild.upload(T.pp_nchild));
    CK(perr.alloc(1));
    CK(cudaMemsetAsync(perr.p, 0, sizeof(int), ctx->stream));
    // leaf-cone interpolation nodes, computed on the device
    if (ex) CK(ex->build_nodes(ctx->leaf_nodes_d.p, ctx->stream));
    else CK(build_leaf_nodes(T, ctx->leaf_nodes_d.p, ctx->stream));
    // propagation plan: the entries are computed on the device from the tree's slot form (or
    // were, level by level, while the host built the cones)
    if (ex) CK(ex->build_plan(ctx->pp.p, ctx->pp32.p, perr.p, ctx->stream));
    else if (by_level) CK(by_level->gather(ctx->pp.p, ctx->pp32.p, perr.p, ctx->stream));
    else CK(build_prop_plan(T, ctx->pp.p, ctx->pp32.p, perr.p, ctx->stream));
    // leaf-cone tables
    launch_leaf_setup(ctx->leaf_cone_box.p, ncl, ctx->leaf_start.p, ctx->leaf_count.p, ctx->leaf_off.p, ctx->leaf_nodes_d.p,
                      ctx->xs_s.p, ctx->ys_s.p, ctx->nxs_s.p, ctx->nys_s.p, T.Ps, T.Pang, k, ctx->form, ctx->eta, ctx->Gsep.p,
                      ctx->leafL.p, ctx->stream, ex ? ex->keta_leafcone : nullptr);
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

static int setup_interp(ifgf2d_ctx* ctx, int nlevels, DBuf<int>& perr) {
    const Discretisation& D = ctx->D;
    Tree& T = ctx->T;
    const long long N = D.N;
    const int P = T.P;
    const int nleaf = (int)T.leaf_start.size();
    {   // interpolation plan: the entries come from the host tree
        static_assert(sizeof(InterpEntry) == sizeof(InterpEntryD), "host and device plan layouts differ");
        CK(ctx->ip.upload(reinterpret_cast<const InterpEntryD*>(T.ip.data()), T.ip.size()));
        CK(ctx->ip_ptr.upload(T.ip_ptr));
        CK(ctx->ip32.alloc(T.ip.size()));
        launch_interp_to_c64(ctx->ip.p, (long long)T.ip.size(), ctx->ip32.p, ctx->stream);
        CK(cudaGetLastError());
    }
    {   // interpolation by leaf box: per box, chunks of 32 targets x pieces of kIbPiece terms
        std::vector<int4> items;
        std::vector<int2> nitems;
        int maxpc = 0;
        for (int b = 0; b < nleaf; ++b) {
            const int s0 = T.leaf_start[b], n = T.leaf_count[b];
            if (n <= 0) continue;
            for (int c0 = 0; c0 < n; c0 += kNearTargets) nitems.push_back(make_int2(b, c0));
            const int nt = T.ip_ptr[s0 + 1] - T.ip_ptr[s0];   // the same for every target of the box
            const int npc = (nt + kIbPiece - 1) / kIbPiece;
            maxpc = std::max(maxpc, npc);
            for (int c0 = 0; c0 < n; c0 += 32)
                for (int q = 0; q < npc; ++q) items.push_back(make_int4(b, c0, q * kIbPiece, std::min(nt, (q + 1) * kIbPiece)));
        }
        CK(ctx->ib_items.upload(items));
        CK(ctx->nb_items.upload(nitems));
        CK(ctx->ipT.alloc(T.ip.size())); CK(ctx->ip32T.alloc(T.ip.size()));
        launch_interp_transpose<double>((int)N, ctx->point_leaf.p, ctx->leaf_start.p, ctx->leaf_count.p, ctx->ip_ptr.p, ctx->ip.p,
                                        ctx->ipT.p, ctx->stream);
        launch_interp_transpose<float>((int)N, ctx->point_leaf.p, ctx->leaf_start.p, ctx->leaf_count.p, ctx->ip_ptr.p, ctx->ip.p,
                                       ctx->ip32T.p, ctx->stream);
        CK(cudaGetLastError());
        CK(ctx->ib_part.alloc((size_t)std::max(maxpc, 1) * N)); CK(ctx->ib_part32.alloc((size_t)std::max(maxpc, 1) * N));
    }
    CK(ctx->coef.alloc((size_t)T.total_cones * P));
    CK(ctx->coef32.alloc((size_t)T.total_cones * P));
    CK(ctx->rho32.alloc(N + 2));   // + padding: the TMA leaf kernel copies from 16-byte boundaries
    CK(ctx->near32.alloc(ctx->near.n));
    CK(ctx->leafL32.alloc(ctx->leafL.n + 2));   // + padding: the TMA leaf kernel copies from 16-byte boundaries
    CK(leaf_tma_init());
    CK(cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    if (!ctx->kerr.p) { CK(ctx->kerr.alloc(1)); CK(cudaMemsetAsync(ctx->kerr.p, 0, sizeof(int), ctx->stream)); }
    launch_d2f(ctx->near.p, (long long)ctx->near.n, ctx->near32.p, ctx->stream);
    launch_d2f(ctx->leafL.p, (long long)ctx->leafL.n, ctx->leafL32.p, ctx->stream);
    CK(cudaGetLastError());
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, perr.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (bad) return fail(ctx, IFGF2D_ERR_GEOMETRY, "internal: a propagation node's child cone is missing");
    ctx->counts[0] = T.near_pairs; ctx->counts[1] = T.leaf_evals; ctx->counts[2] = T.prop_evals;
    ctx->counts[3] = T.interp_evals; ctx->counts[4] = T.total_cones; ctx->counts[5] = nlevels;
    ctx->counts[7] = (long long)(ctx->near.n + ctx->leafL.n + ctx->coef.n + ctx->W.n) * 16 + (long long)ctx->pp.n * sizeof(PropEntryD) +
                     (long long)ctx->ip.n * sizeof(InterpEntryD);
    ctx->ifgf_ready = true;
    if (ctx->gw) ctx->gw->drop_graphs();
    return IFGF2D_OK;
}

int ifgf::setup_tables(ifgf2d_ctx* ctx, double k, int nlevels, const SetupExtra* ex) {
    DBuf<int> perr;
    if (int rc = setup_boxes(ctx, k, nlevels, ex)) return rc;
    if (int rc = setup_cones(ctx, k, nlevels, ex, perr)) return rc;
    return setup_interp(ctx, nlevels, perr);
}

extern "C" int ifgf2d_get_sorting(const ifgf2d_ctx* ctx, long long* s) {
    if (!ctx || !s) return IFGF2D_ERR_ARG;
    if (!ctx->ifgf_ready && !ctx->prep_ready) return IFGF2D_ERR_STATE;
    std::copy(ctx->T.sorting.begin(), ctx->T.sorting.end(), s);
    return IFGF2D_OK;
}
extern "C" int ifgf2d_last_refinements(const ifgf2d_ctx* ctx) { return ctx ? ctx->last_passes : -1; }
extern "C" int ifgf2d_work_counts(const ifgf2d_ctx* ctx, long long out[8]) {
    if (!ctx || !out) return IFGF2D_ERR_ARG;
    for (int i = 0; i < 8; ++i) out[i] = ctx->counts[i];
    return IFGF2D_OK;
}

// after a synchronisation: did a kernel give up on a bounded wait?
static int check_kerr(ifgf2d_ctx* ctx) {
    if (!ctx->kerr.p) return IFGF2D_OK;
    int v = 0;
    CK(cudaMemcpyAsync(&v, ctx->kerr.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (!v) return IFGF2D_OK;
    CK(cudaMemsetAsync(ctx->kerr.p, 0, sizeof(int), ctx->stream));
    return fail(ctx, IFGF2D_ERR_CUDA, "a kernel's bounded wait for a bulk copy ran out");
}

// ------------------------------------------------------------------ apply
// y += near field + cousin interpolants of every target (BoxTree.h:1049-1069).  By target:
// k_final_t, a warp per target.  By leaf box: the interpolation by k_interp_box (pieces per
// target), then the near field by k_near_box, which adds the pieces in order.
template <typename R>
static void launch_interp_final(ifgf2d_ctx* ctx, const V2<R>* rho, const V2<R>* near, const InterpE<R>* ip, const V2<R>* coef,
                                double2* y, bool by_box) {
    const Tree& T = ctx->T;
    const int N = (int)ctx->D.N;
    if (!by_box || ctx->nb_items.n == 0) {
        launch_final_t<R>(N, ctx->point_leaf.p, ctx->leaf_start.p, ctx->near_src_off.p, ctx->near_src.p, ctx->near_rowlen.p,
                          ctx->near_off.p, near, rho, ctx->ip_ptr.p, ip, coef, T.Ps, T.Pang, ctx->sorting.p, y, ctx->stream);
        return;
    }
    const V2<R>* part = nullptr;
    if (ctx->ib_items.n > 0) {
        V2<R>* pp;
        const InterpE<R>* ipT;
        if constexpr (sizeof(R) == 4) { pp = ctx->ib_part32.p; ipT = ctx->ip32T.p; }
        else { pp = ctx->ib_part.p; ipT = ctx->ipT.p; }
        launch_interp_box<R>(ctx->ib_items.p, (int)ctx->ib_items.n, N, ctx->leaf_start.p, ctx->leaf_count.p, ctx->ip_ptr.p, ipT,
                             coef, T.Ps, T.Pang, pp, ctx->stream);
        part = pp;
    }
    launch_near_box<R>(ctx->nb_items.p, (int)ctx->nb_items.n, ctx->leaf_start.p, ctx->leaf_count.p, ctx->near_src_off.p,
                       ctx->near_src.p, ctx->near_rowlen.p, ctx->near_off.p, near, rho, ctx->ip_ptr.p, part, N, ctx->sorting.p, y,
                       ctx->stream);
}

// y += far field of the Morton-ordered intensities (rho / rho32), BoxTree.h:1037-1061
template <typename R>
static void far_ifgf_t(ifgf2d_ctx* ctx, const V2<R>* rho, const V2<R>* near, const V2<R>* leafL, const PropE<R>* pp,
                       const InterpE<R>* ip, const R* Gsep, V2<R>* coef, double2* y, cudaEvent_t* ev) {
    const Tree& T = ctx->T;
    const int Dl = ctx->nlevels - 1, P = T.P;
    const TreeLevel& LD = T.L[Dl];
    cudaStream_t s = ctx->stream;
    const int pr = sizeof(R) == 4 ? 1 : 0;
    bool leaf_done = false;
    if constexpr (sizeof(R) == 4) {
        if (ctx->tune_leaf[1] == 0)
            leaf_done = launch_leaf_tma(ctx->leaf_cone_box.p, (int)LD.cone_nonrel.size(), LD.cone_base, ctx->leaf_start.p,
                                        ctx->leaf_count.p, ctx->leaf_off.p, leafL, rho, P, coef, ctx->kerr.p, ctx->nsm, s);
    }
    if (!leaf_done)
        launch_leaf_apply_t<R>(ctx->leaf_cone_box.p, (int)LD.cone_nonrel.size(), LD.cone_base, ctx->leaf_start.p, ctx->leaf_count.p,
                               ctx->leaf_off.p, leafL, rho, P, coef, s, ctx->tune_leaf[pr]);
    if (ev) cudaEventRecord(ev[0], s);
    for (int l = Dl; l >= 3; --l) {
        const TreeLevel& Lp = T.L[l - 1];
        launch_propagate_t<R>(Lp.cone_base, Lp.cone_base + (int)Lp.cone_nonrel.size(), ctx->pp_ptr.p, ctx->pp_nchild.p, pp,
                              T.Ps, T.Pang, Gsep, coef, s, l < kTuneLevels ? ctx->tune_prop[pr][l] : 0);
    }
    if (ev) cudaEventRecord(ev[1], s);
    launch_interp_final<R>(ctx, rho, near, ip, coef, y, (ctx->tune_batch_tc & (pr ? kSingleInterpBox32 : kSingleInterpBox64)) != 0);
}

// the IFGF far field in the precision of `mode`; x in original order, y += result.  With
// rho_ready the Morton-ordered intensities were already written (by the fused singular pass).
static int far_apply(ifgf2d_ctx* ctx, const double2* x, const double* wq, double2* y, int mode, cudaEvent_t* ev,
                     bool rho_ready = false) {
    const int N = (int)ctx->D.N;
    if (mode == IFGF2D_APPLY_IFGF_MIXED) {
        if (!rho_ready) launch_intensities_t<float>(x, wq, ctx->sorting.p, N, ctx->rho32.p, ctx->stream);
        if (ev) cudaEventRecord(ev[0], ctx->stream);
        far_ifgf_t<float>(ctx, ctx->rho32.p, ctx->near32.p, ctx->leafL32.p, ctx->pp32.p, ctx->ip32.p, ctx->Gsep32.p,
                          ctx->coef32.p, y, ev ? ev + 1 : nullptr);
    } else {
        if (!rho_ready) launch_intensities_t<double>(x, wq, ctx->sorting.p, N, ctx->rho.p, ctx->stream);
        if (ev) cudaEventRecord(ev[0], ctx->stream);
        far_ifgf_t<double>(ctx, ctx->rho.p, ctx->near.p, ctx->leafL.p, ctx->pp.p, ctx->ip.p, ctx->Gsep.p, ctx->coef.p, y,
                           ev ? ev + 1 : nullptr);
    }
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

static int apply_dev(ifgf2d_ctx* ctx, const double2* x, double2* y, int mode) {
    const Discretisation& D = ctx->D;
    const int N = (int)D.N;
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) before apply");
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_DIRECT && mode != IFGF2D_APPLY_IFGF_MIXED)
        return fail(ctx, IFGF2D_ERR_ARG, "unknown apply mode");
    if (mode != IFGF2D_APPLY_DIRECT && !ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup before an IFGF apply");
    const double half = ctx->form == IFGF2D_COMBINED ? 0.5 : 0.0;
    if (mode != IFGF2D_APPLY_DIRECT) {
        launch_sing_intens(x, ctx->W.p, ctx->srow_ptr.p, ctx->srow_col.p, ctx->cols.p, N, D.Np, half, y, ctx->wq.p,
                           ctx->inverse.p, mode == IFGF2D_APPLY_IFGF_MIXED ? nullptr : ctx->rho.p,
                           mode == IFGF2D_APPLY_IFGF_MIXED ? ctx->rho32.p : nullptr, ctx->stream);
        return far_apply(ctx, x, ctx->wq.p, y, mode, nullptr, true);
    }
    launch_sing_intens(x, ctx->W.p, ctx->srow_ptr.p, ctx->srow_col.p, ctx->cols.p, N, D.Np, half, y, ctx->wq.p, nullptr,
                       ctx->rho.p, nullptr, ctx->stream);
    launch_direct_far(ctx->x.p, ctx->y.p, N, ctx->patch_of.p, ctx->nsp_ptr.p, ctx->nsp.p, ctx->x.p, ctx->y.p, ctx->nx.p, ctx->ny.p,
                      ctx->patch_of.p, ctx->rho.p, N, ctx->k, ctx->form, ctx->eta, y, 1, ctx->stream);
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

int ifgf::apply_single(ifgf2d_ctx* ctx, const double2* x, double2* y, int mode) { return apply_dev(ctx, x, y, mode); }
int ifgf::ensure_device_ctx(ifgf2d_ctx* ctx) { return ensure_device(ctx); }

extern "C" int ifgf2d_apply_timed(ifgf2d_ctx* ctx, const void* d_x, void* d_y, int mode, double ms[5]) {
    if (!ctx || !d_x || !d_y || !ms) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) before apply");
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_DIRECT && mode != IFGF2D_APPLY_IFGF_MIXED)
        return fail(ctx, IFGF2D_ERR_ARG, "unknown apply mode");
    if (mode != IFGF2D_APPLY_DIRECT && !ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup before an IFGF apply");
    const double2* x = (const double2*)d_x;
    double2* y = (double2*)d_y;
    const Discretisation& D = ctx->D;
    const int N = (int)D.N;
    cudaEvent_t ev[6];
    for (int i = 0; i < 6; ++i) CK(cudaEventCreate(&ev[i]));
    cudaStream_t s = ctx->stream;
    CK(cudaEventRecord(ev[0], s));
    launch_sing_apply(x, ctx->W.p, ctx->srow_ptr.p, ctx->srow_col.p, ctx->cols.p, N, D.Np,
                      ctx->form == IFGF2D_COMBINED ? 0.5 : 0.0, y, s);
    CK(cudaEventRecord(ev[1], s));
    if (mode != IFGF2D_APPLY_DIRECT) {
        int rc = far_apply(ctx, x, ctx->wq.p, y, mode, ev + 2);
        if (rc != IFGF2D_OK) return rc;
    } else {
        launch_intensities(x, ctx->wq.p, nullptr, N, ctx->rho.p, s);
        CK(cudaEventRecord(ev[2], s));
        CK(cudaEventRecord(ev[3], s));
        CK(cudaEventRecord(ev[4], s));
        launch_direct_far(ctx->x.p, ctx->y.p, N, ctx->patch_of.p, ctx->nsp_ptr.p, ctx->nsp.p, ctx->x.p, ctx->y.p, ctx->nx.p,
                          ctx->ny.p, ctx->patch_of.p, ctx->rho.p, N, ctx->k, ctx->form, ctx->eta, y, 1, s);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(ev[5], s));
    CK(cudaEventSynchronize(ev[5]));
    for (int i = 0; i < 5; ++i) { float t = 0; CK(cudaEventElapsedTime(&t, ev[i], ev[i + 1])); ms[i] = t; }
    for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
    return IFGF2D_OK;
}

// ------------------------------------------------------------------ launch-shape autotuner
// Times every launch shape of the leaf kernel (source chunks 1, 2, 5, 10) and of each level's
// propagation (2, 4 or the most cones per block) on this context's own tables, both
// precisions, and keeps the fastest (median of `reps` CUDA-event timings).  choices (may be
// NULL) receives the table: leaf FP64, leaf complex64, then kTuneLevels propagation entries
// per precision, then the batched complex64 kernels on the tcgen05 tensor cores (bit 0 leaf
// cones in 3xTF32, bit 1 propagation, bit 2 leaf cones with three TF32 terms per operand; FP32
// FMA otherwise) and bit 3, the FMA propagation with TMA-staged child coefficients.
static void write_tuning(const ifgf2d_ctx* ctx, int* c) {
    c[0] = ctx->tune_leaf[0]; c[1] = ctx->tune_leaf[1];
    for (int p = 0; p < 2; ++p)
        for (int l = 0; l < kTuneLevels; ++l) c[2 + p * kTuneLevels + l] = ctx->tune_prop[p][l];
    c[2 + 2 * kTuneLevels] = ctx->tune_batch_tc;
}
extern "C" int ifgf2d_tuning_size(void) { return 3 + 2 * kTuneLevels; }
extern "C" int ifgf2d_get_tuning(const ifgf2d_ctx* ctx, int* choices) {
    if (!ctx || !choices) return IFGF2D_ERR_ARG;
    write_tuning(ctx, choices);
    return IFGF2D_OK;
}
extern "C" int ifgf2d_set_tuning(ifgf2d_ctx* ctx, const int* c) {
    if (!ctx || !c) return IFGF2D_ERR_ARG;
    ctx->tune_leaf[0] = c[0]; ctx->tune_leaf[1] = c[1];
    for (int p = 0; p < 2; ++p)
        for (int l = 0; l < kTuneLevels; ++l) ctx->tune_prop[p][l] = c[2 + p * kTuneLevels + l];
    ctx->tune_batch_tc = c[2 + 2 * kTuneLevels] & kKernelBits;
    if (ctx->gw) ctx->gw->drop_graphs();   // the captured iterations hold the old launch shapes
    return IFGF2D_OK;
}
template <typename R>
static int tune_precision(ifgf2d_ctx* ctx, int reps, const V2<R>* rho, const V2<R>* leafL, const PropE<R>* pp, const R* Gsep,
                          V2<R>* coef) {
    const Tree& T = ctx->T;
    const int Dl = ctx->nlevels - 1, P = T.P, pr = sizeof(R) == 4 ? 1 : 0;
    const TreeLevel& LD = T.L[Dl];
    cudaStream_t s = ctx->stream;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    auto time_it = [&](auto&& launch) -> float {
        std::vector<float> t(reps);
        launch();   // warm
        for (int q = 0; q < reps; ++q) {
            cudaEventRecord(e0, s); launch(); cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&t[q], e0, e1);
        }
        std::sort(t.begin(), t.end());
        return t[reps / 2];
    };
    float best = 1e30f; int bestc = 5;
    for (int ch : {1, 2, 5, 10, 0}) {   // 0: complex64 only, the table streamed by TMA bulk copies
        if (ch == 0 && sizeof(R) != 4) continue;
        const float ms = time_it([&] {
            bool done = false;
            if constexpr (sizeof(R) == 4) {
                if (ch == 0)
                    done = launch_leaf_tma(ctx->leaf_cone_box.p, (int)LD.cone_nonrel.size(), LD.cone_base, ctx->leaf_start.p,
                                           ctx->leaf_count.p, ctx->leaf_off.p, leafL, rho, P, coef, ctx->kerr.p, ctx->nsm, s);
            }
            if (!done)
                launch_leaf_apply_t<R>(ctx->leaf_cone_box.p, (int)LD.cone_nonrel.size(), LD.cone_base, ctx->leaf_start.p,
                                       ctx->leaf_count.p, ctx->leaf_off.p, leafL, rho, P, coef, s, ch);
        });
        if (ms < best) { best = ms; bestc = ch; }
    }
    ctx->tune_leaf[pr] = bestc;
    for (int l = Dl; l >= 3 && l < kTuneLevels; --l) {
        const TreeLevel& Lp = T.L[l - 1];
        best = 1e30f; int bestp = 0;
        for (int cpb : {2, 4, 0, kPropStaged}) {
            const float ms = time_it([&] {
                launch_propagate_t<R>(Lp.cone_base, Lp.cone_base + (int)Lp.cone_nonrel.size(), ctx->pp_ptr.p, ctx->pp_nchild.p, pp,
                                      T.Ps, T.Pang, Gsep, coef, s, cpb);
            });
            if (ms < best) { best = ms; bestp = cpb; }
        }
        ctx->tune_prop[pr][l] = bestp;
    }
    {   // the interpolation by leaf box or by target (y: the context's output vector, overwritten later)
        const int bit = pr ? kSingleInterpBox32 : kSingleInterpBox64;
        const V2<R>* near;
        const InterpE<R>* ip;
        if constexpr (sizeof(R) == 4) { near = ctx->near32.p; ip = ctx->ip32.p; }
        else { near = ctx->near.p; ip = ctx->ip.p; }
        const float tb = time_it([&] { launch_interp_final<R>(ctx, rho, near, ip, coef, ctx->vout.p, true); });
        const float tt = time_it([&] { launch_interp_final<R>(ctx, rho, near, ip, coef, ctx->vout.p, false); });
        if (tb < tt) ctx->tune_batch_tc |= bit;
        else ctx->tune_batch_tc &= ~bit;
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    CK(cudaGetLastError());
    return IFGF2D_OK;
}
extern "C" int ifgf2d_autotune(ifgf2d_ctx* ctx, int reps, int* choices) {
    if (!ctx || reps <= 0 || reps > 1000) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    if (!ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup before autotuning");
    // realistic intensities in both precisions from one apply of each form on the stored vector
    CK(cudaMemsetAsync(ctx->vin.p, 0, sizeof(double2) * ctx->D.N, ctx->stream));
    int rc;
    if ((rc = apply_dev(ctx, ctx->vin.p, ctx->vout.p, IFGF2D_APPLY_IFGF))) return rc;
    if ((rc = apply_dev(ctx, ctx->vin.p, ctx->vout.p, IFGF2D_APPLY_IFGF_MIXED))) return rc;
    if ((rc = tune_precision<double>(ctx, reps, ctx->rho.p, ctx->leafL.p, ctx->pp.p, ctx->Gsep.p, ctx->coef.p))) return rc;
    if ((rc = tune_precision<float>(ctx, reps, ctx->rho32.p, ctx->leafL32.p, ctx->pp32.p, ctx->Gsep32.p, ctx->coef32.p))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->gw) ctx->gw->drop_graphs();
    if (choices) write_tuning(ctx, choices);
    return IFGF2D_OK;
}

extern "C" int ifgf2d_measure_fp64_peak(double* tflops) {
    if (!tflops) return IFGF2D_ERR_ARG;
    return launch_fp64_peak(tflops) ? IFGF2D_OK : IFGF2D_ERR_CUDA;
}

extern "C" int ifgf2d_apply_device(ifgf2d_ctx* ctx, const void* d_x, void* d_y, int mode) {
    if (!ctx || !d_x || !d_y) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    return apply_dev(ctx, (const double2*)d_x, (double2*)d_y, mode);
}

extern "C" int ifgf2d_apply(ifgf2d_ctx* ctx, const double* x, double* y, int mode) {
    if (!ctx || !x || !y) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    // state and mode before any copy (apply_dev repeats the checks for the device entry point)
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) before apply");
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_DIRECT && mode != IFGF2D_APPLY_IFGF_MIXED)
        return fail(ctx, IFGF2D_ERR_ARG, "unknown apply mode");
    if (mode != IFGF2D_APPLY_DIRECT && !ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup before an IFGF apply");
    if (!all_finite(x, 2 * ctx->D.N)) return fail(ctx, IFGF2D_ERR_NONFINITE, "non-finite value in the density");
    const size_t bytes = sizeof(double2) * ctx->D.N;
    CK(cudaMemcpyAsync(ctx->vin.p, x, bytes, cudaMemcpyHostToDevice, ctx->stream));
    // the device part on the context's own vectors, captured once per mode as a CUDA graph (one
    // launch instead of one per kernel); set-up, precomputation and tuning changes drop it
    if (!ctx->gw) ctx->gw.reset(new GmresWork);
    cudaGraphExec_t& ex = ctx->gw->apply_exec[mode];
    if (!ex) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = apply_dev(ctx, ctx->vin.p, ctx->vout.p, mode);
        const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &graph);
        if (rc != IFGF2D_OK) { if (ec == cudaSuccess) cudaGraphDestroy(graph); return rc; }
        CK(ec);
        const cudaError_t ei = cudaGraphInstantiate(&ex, graph, 0);
        cudaGraphDestroy(graph);
        CK(ei);
    }
    CK(cudaGraphLaunch(ex, ctx->stream));
    CK(cudaMemcpyAsync(y, ctx->vout.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    // of the single-vector kernels only the TMA-streamed complex64 leaf kernel can set the
    // bounded-wait flag; the other applies skip the flag's read-back round trip
    if (mode == IFGF2D_APPLY_IFGF_MIXED && ctx->tune_leaf[1] == 0)
        if (int rk = check_kerr(ctx)) return rk;
    if (!all_finite(y, 2 * ctx->D.N)) return fail(ctx, IFGF2D_ERR_NONFINITE, "non-finite value in the result");
    return IFGF2D_OK;
}

extern "C" int ifgf2d_ifgf_far(ifgf2d_ctx* ctx, const double* intens, double* y) {
    if (!ctx || !intens || !y) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    if (!ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup first");
    const size_t bytes = sizeof(double2) * ctx->D.N;
    CK(cudaMemcpyAsync(ctx->vin.p, intens, bytes, cudaMemcpyHostToDevice, ctx->stream));
    // rho = intensities in Morton order (unit weights)
    std::vector<double> ones(ctx->D.N, 1.0);
    DBuf<double> w1; CK(w1.upload(ones));
    CK(cudaMemsetAsync(ctx->vout.p, 0, bytes, ctx->stream));
    int rc = far_apply(ctx, ctx->vin.p, w1.p, ctx->vout.p, IFGF2D_APPLY_IFGF, nullptr);
    if (rc != IFGF2D_OK) return rc;
    CK(cudaMemcpyAsync(y, ctx->vout.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return IFGF2D_OK;
}

// ------------------------------------------------------------------ propagation (off-surface)
extern "C" int ifgf2d_propagate(ifgf2d_ctx* ctx, long long m, const double* xp, const double* yp, const double* dens, double* out) {
    if (!ctx || m < 0 || (m > 0 && (!xp || !yp || !out)) || !dens) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) first: the wavenumber is set there");
    if (m == 0) return IFGF2D_OK;
    const int N = (int)ctx->D.N;
    DBuf<double> tx, ty; DBuf<double2> o;
    CK(tx.upload(xp, m)); CK(ty.upload(yp, m)); CK(o.alloc(m));
    CK(cudaMemcpyAsync(ctx->vin.p, dens, sizeof(double2) * N, cudaMemcpyHostToDevice, ctx->stream));
    launch_intensities(ctx->vin.p, ctx->wq.p, nullptr, N, ctx->rho.p, ctx->stream);
    launch_direct_far(tx.p, ty.p, (int)m, nullptr, nullptr, nullptr, ctx->x.p, ctx->y.p, ctx->nx.p, ctx->ny.p, nullptr, ctx->rho.p, N,
                      ctx->k, ctx->form, ctx->eta, o.p, 0, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, o.p, sizeof(double2) * m, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return IFGF2D_OK;
}

// ------------------------------------------------------------------ GMRES on the device

// GMRES core on device vectors: x = A^{-1} b from the initial guess 0 (the reference's guess,
// opGMRES.hpp:383-392).  Arnoldi with classical Gram-Schmidt twice (CGS2), Givens rotations and
// the residual estimate on the device (gmres_device.cu).  One restart cycle is one launch of a
// captured CUDA graph: a while-loop whose body is one iteration -- copy of v_j, the whole apply,
// CGS2 into the Hessenberg column, ||w||, v_{j+1} = w / ||w||, the Givens step -- and whose
// condition the Givens step clears when the cycle ends.  The kernels read j from device memory,
// so the same graph serves every iteration and every cycle.  After the loop one warp solves the
// triangular system, x += V y, and the host reads the cycle's state (a few bytes) once.  Stops
// when |g_{j+1}| / ||r0|| < tol (the first ||r0||, opGMRES.hpp:207) or after max_iters
// iterations.
// The right preconditioner of a flexible GMRES: the learned network, the spectral preconditioner
// (spectral_precond.cu), or the spectral one corrected by the network (z = M_s r + N(r) - 2 r:
// the network trained on the spectral preconditioner's errors)
struct RightPrecond {
    ifgf2d_net* net = nullptr;
    SpectralWork* spec = nullptr;
    int kind() const { return (net ? 1 : 0) | (spec ? 2 : 0); }
};

static int gmres_core(ifgf2d_ctx* ctx, const double2* b, double2* x, int mode, double tol, int restart,
                      int max_iters, int& iters, double& est, const RightPrecond* P = nullptr) {
    const long long N = ctx->D.N;
    const int m = restart, ldh = m + 1;
    cudaStream_t s = ctx->stream;
    if (!ctx->gw) ctx->gw.reset(new GmresWork);
    GmresWork& G = *ctx->gw;
    if (G.n != N || G.m != m) {
        G.drop_graphs();
        CK(G.V.alloc((size_t)N * (m + 1))); CK(G.w.alloc(N)); CK(G.h.alloc(m + 2)); CK(G.t.alloc(N)); CK(G.vin.alloc(N));
        CK(G.H.alloc((size_t)ldh * m)); CK(G.y.alloc(m)); CK(G.nrm2.alloc(1)); CK(G.jdev.alloc(1));
        CK(G.part.alloc((size_t)arnoldi_part_size(N, m)));
        CK(G.lsR.alloc((size_t)ldh * m)); CK(G.lsg.alloc(m + 1)); CK(G.lsgc.alloc(m)); CK(G.lsgs.alloc(m));
        CK(G.lsst.alloc(4)); CK(G.lssc.alloc(3));
        G.Z.release(); G.zt.release(); G.zt2.release(); G.zt3.release();
        G.n = N; G.m = m;
    }
    const int pk = P ? P->kind() : 0;
    if (pk && !G.Z.p) { CK(G.Z.alloc((size_t)N * m)); CK(G.zt.alloc(N)); }
    if (pk == 3 && !G.zt2.p) { CK(G.zt2.alloc(N)); CK(G.zt3.alloc(N)); }
    const LsqDev L{G.lsR.p, G.lsg.p, G.lsgc.p, G.lsgs.p, G.lsst.p, G.lssc.p, m};
    const int gi = mode + 3 * pk;
    if (!G.exec[gi]) {
        cudaGraph_t graph;
        CK(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle cond;
        cudaError_t e = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = cond;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(s, np.conditional.phGraph_out[0], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            return fail(ctx, IFGF2D_ERR_CUDA, std::string("building the GMRES cycle graph: ") + cudaGetErrorString(e));
        }
        launch_copy_col(G.V.p, N, G.jdev.p, G.vin.p, G.nrm2.p, s);
        int rc;
        if (pk) {
            // flexible GMRES: z_j = M(v_j) into Z[:, j], then w = A z_j
            if (pk == 1) {
                net_precondition_launch(P->net, G.vin.p, G.zt.p, s);
            } else {
                spectral_launch(P->spec, G.vin.p, G.zt.p, ctx->D.Np, s);
                if (pk == 3) {
                    net_precondition_launch(P->net, G.vin.p, G.zt2.p, s);
                    if (net_weighted(P->net)) {   // zt += Op(1/|sigma|) (zt2 - 2 v)
                        launch_axpby(G.zt2.p, 1.0, G.zt2.p, -2.0, G.vin.p, N, s);
                        spectral_launch(P->spec, G.zt2.p, G.zt3.p, ctx->D.Np, s, 2);
                        launch_axpby(G.zt.p, 1.0, G.zt.p, 1.0, G.zt3.p, N, s);
                    } else {
                        launch_precond_sum(G.zt.p, G.zt2.p, G.vin.p, N, s);   // zt += zt2 - 2 v
                    }
                }
            }
            launch_store_col(G.zt.p, N, G.jdev.p, G.Z.p, s);
            rc = apply_dev(ctx, G.zt.p, G.w.p, mode);
        } else {
            rc = apply_dev(ctx, G.vin.p, G.w.p, mode);
        }
        // the complex64 inner solves of the refinement take one Gram-Schmidt pass, as the batched
        // ones do: each correction is checked by the FP64 residual, and a short one costs one more
        // refinement pass, not a wrong answer
        launch_arnoldi_step(G.V.p, N, m, G.jdev.p, G.w.p, G.h.p, G.H.p, G.nrm2.p, G.part.p, s,
                            mode == IFGF2D_APPLY_IFGF_MIXED ? 1 : 2, &L, cond, true);
        cudaGraph_t body = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(s, &body);
        if (rc != IFGF2D_OK || ec != cudaSuccess) {
            cudaGraphDestroy(graph);
            if (rc != IFGF2D_OK) return rc;
            CK(ec);
        }
        e = cudaGraphInstantiate(&G.exec[gi], graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { G.exec[gi] = nullptr; CK(e); }
    }
    double2 *V = G.V.p, *w = G.w.p, *h = G.h.p, *t = G.t.p;
    // the cycle state read back after each cycle: estimate (double), then [stopped, columns,
    // limit, iterations] (ints)
    double2* rb = pinned_scratch(4);
    if (!rb) return fail(ctx, IFGF2D_ERR_CUDA, "cudaMallocHost of the GMRES read-back buffer failed");
    double* rb_est = reinterpret_cast<double*>(rb);
    int* rb_st = reinterpret_cast<int*>(rb + 2);
    CK(cudaMemsetAsync(x, 0, sizeof(double2) * N, s));
    auto dnorm = [&](const double2* v, double& out) -> int {
        launch_multidot(v, N, 1, v, N, h + m + 1, s);
        double2 r; CK(cudaMemcpyAsync(&r, h + m + 1, sizeof(double2), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        out = std::sqrt(std::max(r.x, 0.0));
        return IFGF2D_OK;
    };
    int rc;
    iters = 0; est = 0.0;
    double bn; if ((rc = dnorm(b, bn))) return rc;
    if (bn <= 2.2250738585072014e-308) return IFGF2D_OK;
    // r0 = b - A x0 = b for the initial guess x0 = 0 (the reference applies the operator to the
    // zero guess, which gives exactly 0)
    CK(cudaMemcpyAsync(w, b, sizeof(double2) * N, cudaMemcpyDeviceToDevice, s));
    double beta; if ((rc = dnorm(w, beta))) return rc;
    const double r0n = beta;
    est = 1.0;
    if (beta == 0.0) { est = 0.0; return IFGF2D_OK; }
    for (;;) {
        const long long limit = std::min<long long>(max_iters, N) - iters;
        if (limit <= 0) break;
        launch_scale(w, make_double2(1.0 / beta, 0.0), N, V, s);
        CK(cudaMemsetAsync(G.H.p, 0, sizeof(double2) * ldh * m, s));
        launch_lsq_init(L, G.jdev.p, beta, r0n, tol, (int)std::min<long long>(limit, 1 << 30), s);
        CK(cudaGraphLaunch(G.exec[gi], s));
        launch_lsq_solve(L, ldh, G.y.p, s);
        launch_multi_axpy_dyn(pk ? G.Z.p : V, N, G.lsst.p + 1, G.y.p, N, x, s);   // x += V y, or Z y (flexible)
        CK(cudaMemcpyAsync(rb_est, G.lssc.p, sizeof(double), cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(rb_st, G.lsst.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        CK(cudaGetLastError());
        iters += rb_st[3];
        est = *rb_est;
        if (rb_st[0] || rb_st[3] <= 0) break;   // converged, out of iterations or broken down
        // restart: r = b - A x (the residual estimate keeps the first ||r0||, opGMRES.hpp:207)
        if ((rc = apply_dev(ctx, x, t, mode))) return rc;
        launch_sub(b, t, N, w, s);
        if ((rc = dnorm(w, beta))) return rc;
        if (beta == 0.0) { est = 0.0; break; }
    }
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

extern "C" int ifgf2d_solve(ifgf2d_ctx* ctx, const double* rhs, double* xout, int mode, double tol, int restart, int max_iters,
                            int* iters_out, double* err_out) {
    if (!ctx || !rhs || !xout || restart <= 0 || max_iters <= 0) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) before solve");
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_DIRECT && mode != IFGF2D_APPLY_IFGF_MIXED)
        return fail(ctx, IFGF2D_ERR_ARG, "unknown solve mode");
    if (mode != IFGF2D_APPLY_DIRECT && !ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup before an IFGF solve");
    const long long N = ctx->D.N;
    if (!all_finite(rhs, 2 * N)) return fail(ctx, IFGF2D_ERR_NONFINITE, "non-finite value in the right-hand side");
    cudaStream_t s = ctx->stream;
    if (!ctx->gw) ctx->gw.reset(new GmresWork);
    GmresWork& GW = *ctx->gw;
    if (GW.sn != N) {
        CK(GW.sb.alloc(N)); CK(GW.sx.alloc(N)); CK(GW.sr.alloc(N)); CK(GW.sd.alloc(N)); CK(GW.st.alloc(N)); CK(GW.shb.alloc(1));
        GW.sn = N;
    }
    DBuf<double2>& b = GW.sb;
    DBuf<double2>& x = GW.sx;
    CK(cudaMemcpyAsync(b.p, rhs, sizeof(double2) * N, cudaMemcpyHostToDevice, s));
    int iters = 0, rc;
    double est = 0.0;
    if (mode != IFGF2D_APPLY_IFGF_MIXED) {
        if ((rc = gmres_core(ctx, b.p, x.p, mode, tol, restart, max_iters, iters, est))) return rc;
    } else {
        // FP64 iterative refinement: r = b - A x with the FP64 IFGF operator, inner GMRES on the
        // complex64 operator for the correction, x += d, until ||r|| / ||b|| < tol
        DBuf<double2>& r = GW.sr;
        DBuf<double2>& d = GW.sd;
        DBuf<double2>& t = GW.st;
        DBuf<double2>& hb = GW.shb;
        CK(cudaMemsetAsync(x.p, 0, sizeof(double2) * N, s));
        auto nrm = [&](const double2* v, double& out) -> int {
            launch_multidot(v, N, 1, v, N, hb.p, s);
            double2 q; CK(cudaMemcpyAsync(&q, hb.p, sizeof(double2), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            out = std::sqrt(std::max(q.x, 0.0));
            return IFGF2D_OK;
        };
        double bn; if ((rc = nrm(b.p, bn))) return rc;
        CK(cudaMemcpyAsync(r.p, b.p, sizeof(double2) * N, cudaMemcpyDeviceToDevice, s));
        double rn = bn;
        est = bn > 0 ? 1.0 : 0.0;
        ctx->last_passes = 0;
        for (int outer = 0; outer < 30 && est >= tol && iters < max_iters; ++outer) {
            ++ctx->last_passes;
            // inner solves run to 0.3 of what is left of the tolerance, but not below the
            // complex64 operator's own accuracy (~6e-8 relative on the kite at k = 500)
            const double inner_tol = std::max(2e-7, 0.3 * tol * bn / rn);
            int it = 0; double e = 0.0;
            if ((rc = gmres_core(ctx, r.p, d.p, IFGF2D_APPLY_IFGF_MIXED, inner_tol, restart, max_iters - iters, it, e))) return rc;
            iters += it;
            {
                double2 one = make_double2(1.0, 0.0);
                CK(cudaMemcpyAsync(hb.p, &one, sizeof(double2), cudaMemcpyHostToDevice, s));
                launch_multi_axpy(d.p, N, 1, hb.p, 1.0, N, x.p, s);   // x += d
            }
            if ((rc = apply_dev(ctx, x.p, t.p, IFGF2D_APPLY_IFGF))) return rc;
            launch_sub(b.p, t.p, N, r.p, s);
            if ((rc = nrm(r.p, rn))) return rc;
            est = rn / bn;
        }
    }
    CK(cudaMemcpyAsync(xout, x.p, sizeof(double2) * N, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (iters_out) *iters_out = iters;
    if (err_out) *err_out = est;
    if (int rk = check_kerr(ctx)) return rk;
    return est < tol ? IFGF2D_OK : IFGF2D_ERR_NOCONV;
}

// ------------------------------------------------------------------ right preconditioners
// Flexible GMRES with z_j = M(v_j) (the network, the spectral preconditioner or both) inside FP64
// iterative refinement: the residual b - A x with the FP64 operator (the stop test), corrections
// from flexible GMRES on the operator of `mode`.  A preconditioned correction that misses its
// tolerance (a stall) switches the rest of the solve to plain GMRES.
static int solve_flexible(ifgf2d_ctx* ctx, RightPrecond P, const double* rhs, double* xout, int mode, double tol, int restart,
                          int max_iters, int* iters_out, double* err_out) {
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) before solve");
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_DIRECT && mode != IFGF2D_APPLY_IFGF_MIXED)
        return fail(ctx, IFGF2D_ERR_ARG, "unknown solve mode");
    if (mode != IFGF2D_APPLY_DIRECT && !ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup before an IFGF solve");
    const Discretisation& D = ctx->D;
    const long long N = D.N;
    if (!all_finite(rhs, 2 * N)) return fail(ctx, IFGF2D_ERR_NONFINITE, "non-finite value in the right-hand side");
    cudaStream_t s = ctx->stream;
    if (!ctx->gw) ctx->gw.reset(new GmresWork);
    GmresWork& GW = *ctx->gw;
    if (P.net) {
        std::vector<double> geom((size_t)N * 4);
        for (long long i = 0; i < N; ++i) {
            geom[4 * i] = D.kappa[i]; geom[4 * i + 1] = -D.ny[i]; geom[4 * i + 2] = D.nx[i]; geom[4 * i + 3] = D.wq[i];
        }
        CK(cudaStreamSynchronize(s));
        std::string msg;
        int rc = net_prepare_single(P.net, N, geom.data(), ctx->k, msg);
        if (rc != IFGF2D_OK) return fail(ctx, rc, msg);
        // the network's buffers may have moved since the last capture: recapture its iterations
        for (int q = 3; q < 12; ++q)
            if (((q / 3) & 1) && GW.exec[q]) { cudaGraphExecDestroy(GW.exec[q]); GW.exec[q] = nullptr; }
    }
    if (GW.sn != N) {
        CK(GW.sb.alloc(N)); CK(GW.sx.alloc(N)); CK(GW.sr.alloc(N)); CK(GW.sd.alloc(N)); CK(GW.st.alloc(N)); CK(GW.shb.alloc(1));
        GW.sn = N;
    }
    double2 *b = GW.sb.p, *x = GW.sx.p, *r = GW.sr.p, *d = GW.sd.p, *t = GW.st.p, *hb = GW.shb.p;
    CK(cudaMemcpyAsync(b, rhs, sizeof(double2) * N, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(x, 0, sizeof(double2) * N, s));
    auto nrm = [&](const double2* v, double& out) -> int {
        launch_multidot(v, N, 1, v, N, hb, s);
        double2 q; CK(cudaMemcpyAsync(&q, hb, sizeof(double2), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        out = std::sqrt(std::max(q.x, 0.0));
        return IFGF2D_OK;
    };
    const int outer_mode = mode == IFGF2D_APPLY_DIRECT ? IFGF2D_APPLY_DIRECT : IFGF2D_APPLY_IFGF;
    int rc, iters = 0;
    double bn; if ((rc = nrm(b, bn))) return rc;
    CK(cudaMemcpyAsync(r, b, sizeof(double2) * N, cudaMemcpyDeviceToDevice, s));
    double rn = bn, est = bn > 0 ? 1.0 : 0.0;
    bool use_p = true;
    ctx->last_passes = 0;
    for (int outer = 0; outer < 30 && est >= tol && iters < max_iters; ++outer) {
        ++ctx->last_passes;
        const double want = tol * bn / rn;
        const double inner_tol = mode == IFGF2D_APPLY_IFGF_MIXED ? std::max(2e-7, 0.3 * want) : 0.5 * want;
        int it = 0; double e = 0.0;
        if ((rc = gmres_core(ctx, r, d, mode, inner_tol, restart, max_iters - iters, it, e, use_p ? &P : nullptr))) return rc;
        iters += it;
        if (use_p && e >= inner_tol) use_p = false;   // stalled: plain GMRES from here on
        double2 one = make_double2(1.0, 0.0);
        CK(cudaMemcpyAsync(hb, &one, sizeof(double2), cudaMemcpyHostToDevice, s));
        launch_multi_axpy(d, N, 1, hb, 1.0, N, x, s);   // x += d
        if ((rc = apply_dev(ctx, x, t, outer_mode))) return rc;
        launch_sub(b, t, N, r, s);
        if ((rc = nrm(r, rn))) return rc;
        est = rn / bn;
    }
    CK(cudaMemcpyAsync(xout, x, sizeof(double2) * N, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (iters_out) *iters_out = iters;
    if (err_out) *err_out = est;
    if (int rk = check_kerr(ctx)) return rk;
    if (P.net && net_kernel_error(P.net) != IFGF2D_OK)
        return fail(ctx, IFGF2D_ERR_CUDA, "learned preconditioner: a tensor-core completion wait ran out");
    return est < tol ? IFGF2D_OK : IFGF2D_ERR_NOCONV;
}

extern "C" int ifgf2d_solve_precond(ifgf2d_ctx* ctx, ifgf2d_net* net, const double* rhs, double* xout, int mode, double tol,
                                    int restart, int max_iters, int* iters_out, double* err_out) {
    if (!ctx || !net || !rhs || !xout || restart <= 0 || max_iters <= 0) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    RightPrecond P;
    P.net = net;
    return solve_flexible(ctx, P, rhs, xout, mode, tol, restart, max_iters, iters_out, err_out);
}

extern "C" int ifgf2d_solve_flexible(ifgf2d_ctx* ctx, ifgf2d_net* net, int precond, const double* rhs, double* xout, int mode,
                                     double tol, int restart, int max_iters, int* iters_out, double* err_out) {
    if (!ctx || !rhs || !xout || restart <= 0 || max_iters <= 0) return IFGF2D_ERR_ARG;
    if (precond <= 0 || (precond & ~(IFGF2D_PRECOND_NET | IFGF2D_PRECOND_SPECTRAL)))
        return fail(ctx, IFGF2D_ERR_ARG, "precond: IFGF2D_PRECOND_NET, IFGF2D_PRECOND_SPECTRAL or both");
    if ((precond & IFGF2D_PRECOND_NET) && !net) return fail(ctx, IFGF2D_ERR_ARG, "IFGF2D_PRECOND_NET needs a network");
    AllocStream guard(ctx->stream);
    RightPrecond P;
    if (precond & IFGF2D_PRECOND_NET) P.net = net;
    if (precond & IFGF2D_PRECOND_SPECTRAL) {
        if (!ctx->sw) {
            const int rc = spectral_setup(ctx, IFGF2D_SPECTRAL_DEFAULT_SCALE);
            if (rc != IFGF2D_OK) return rc;
        }
        P.spec = ctx->sw;
    }
    return solve_flexible(ctx, P, rhs, xout, mode, tol, restart, max_iters, iters_out, err_out);
}

// ------------------------------------------------------------------ Hankel test entry
extern "C" int ifgf2d_hankel(int order, long long n, const double* x, double* out) {
    if (order < 0 || order > 3 || n < 0 || (n > 0 && (!x || !out))) return IFGF2D_ERR_ARG;
    if (n == 0) return IFGF2D_OK;
    if (n > (1LL << 30)) return IFGF2D_ERR_ARG;
    DBuf<double> dx; DBuf<double2> dout;
    if (dx.upload(x, n) != cudaSuccess || dout.alloc(n) != cudaSuccess) return IFGF2D_ERR_CUDA;
    launch_hankel(order, dx.p, (int)n, dout.p, 0);
    if (cudaGetLastError() != cudaSuccess) return IFGF2D_ERR_CUDA;
    if (cudaMemcpy(out, dout.p, sizeof(double2) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return IFGF2D_ERR_CUDA;
    return IFGF2D_OK;
}

// ------------------------------------------------------------------ views for other translation units

int ifgf::direct_view(ifgf2d_ctx* ctx, ifgf::DirectView* v) {
    if (!ctx || !v) return IFGF2D_ERR_ARG;
    if (!ctx->precomputed) return fail(ctx, IFGF2D_ERR_STATE, "precompute (or setup) before apply");
    v->N = (int)ctx->D.N; v->Np = ctx->D.Np; v->device = ctx->device; v->k = ctx->k; v->stream = ctx->stream;
    v->W = ctx->W.p; v->srow_ptr = ctx->srow_ptr.p; v->srow_col = ctx->srow_col.p; v->cols = ctx->cols.p;
    v->wq = ctx->wq.p; v->x = ctx->x.p; v->y = ctx->y.p; v->patch_of = ctx->patch_of.p;
    v->nsp_ptr = ctx->nsp_ptr.p; v->nsp = ctx->nsp.p;
    v->nx = ctx->nx.p; v->ny = ctx->ny.p; v->form = ctx->form; v->eta = ctx->eta;
    v->half = ctx->form == IFGF2D_COMBINED ? 0.5 : 0.0;
    return IFGF2D_OK;
}

void ifgf::set_error(ifgf2d_ctx* ctx, const char* msg) { if (ctx) ctx->err = msg; }
