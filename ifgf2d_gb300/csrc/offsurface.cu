// offsurface.cu -- the IFGF-accelerated off-surface field (C ABI ifgf2d_eval_offsurface_*).
//
// The reference evaluates the layer potential at off-surface points directly, O(M N)
// (ForwardMap::propagate_unacc, ForwardMap.tpp:701-727).  Here the sources' cone
// coefficients are built for the cones the targets need (build_target_tree: the surface
// tree's boxes, cones reaching the farthest target), and each target sums
//   * the direct Green function over the sources of its adjacent leaf boxes, and
//   * the cone interpolants of the boxes in its interaction lists, level by level,
// which covers every source once.  Targets may lie anywhere, also outside the root box.
#include "context.hpp"
#include "hankel.cuh"
#include "ifgf_device.cuh"

struct EvalWork {
    Tree E;
    long long M = 0;
    DBuf<double> tx, ty;
    DBuf<int> leaf_cone_box;
    DBuf<long long> leaf_off;
    DBuf<LeafNode> nodes;
    DBuf<double2> leafL;
    DBuf<long long> pp_ptr;
    DBuf<int> pp_nchild;
    DBuf<PropEntryD> pp;
    DBuf<int> ip_ptr, nb_ptr, nb_box;
    DBuf<InterpEntryD> ip;
    DBuf<double2> coef, out;
};

void ifgf::free_eval(ifgf2d_ctx* ctx) {
    delete ctx->ew;
    ctx->ew = nullptr;
}

namespace {

// warp = one target: lanes share its near sources (direct Green function, the formulation's
// kernel with the source normal) and its interpolation entries, then a warp sum
template <int PS, int PA>
__global__ void __launch_bounds__(256) k_eval_targets(long long M, const double* __restrict__ tx, const double* __restrict__ ty,
                                                      const int* __restrict__ nb_ptr, const int* __restrict__ nb_box,
                                                      const int* __restrict__ leaf_start, const int* __restrict__ leaf_count,
                                                      const double* __restrict__ xs, const double* __restrict__ ys,
                                                      const double* __restrict__ nxs, const double* __restrict__ nys,
                                                      const double2* __restrict__ rho, double k, int form, double eta,
                                                      const int* __restrict__ ip_ptr, const InterpEntryD* __restrict__ ip,
                                                      const double2* __restrict__ coef, double2* __restrict__ out) {
    constexpr int P = PS * PA;
    const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= M) return;
    const double x = tx[t], y = ty[t];
    double2 acc = make_double2(0.0, 0.0);
    for (int q = nb_ptr[t]; q < nb_ptr[t + 1]; ++q) {
        const int b = nb_box[q];
        const int s0 = leaf_start[b], n = leaf_count[b];
        for (int s = lane; s < n; s += 32) {
            const int j = s0 + s;
            const double2 g = green_form(form, x - xs[j], y - ys[j], nxs[j], nys[j], k, eta);
            cmac<double>(acc, g, rho[j]);
        }
    }
    for (int e = ip_ptr[t] + lane; e < ip_ptr[t + 1]; e += 32) {
        const InterpEntryD E = ip[e];
        const double2 it = interp_eval<double, PS, PA>(coef + (long long)E.cone * P, E.s, E.th);
        cmac<double>(acc, it, make_double2(E.fr, E.fi));
    }
    acc.x = warp_sum_r<double>(acc.x);
    acc.y = warp_sum_r<double>(acc.y);
    if (lane == 0) out[t] = acc;
}

void launch_eval_targets(long long M, const double* tx, const double* ty, const int* nb_ptr, const int* nb_box,
                         const int* leaf_start, const int* leaf_count, const double* xs, const double* ys, const double* nxs,
                         const double* nys, const double2* rho, double k, int form, double eta, const int* ip_ptr,
                         const InterpEntryD* ip, const double2* coef, int Ps, int Pang, double2* out, cudaStream_t s) {
    if (M <= 0) return;
    const unsigned grid = (unsigned)((M * 32 + 255) / 256);
    IFGF_DISPATCH_P(Ps, Pang, (k_eval_targets<PS, PA><<<grid, 256, 0, s>>>(M, tx, ty, nb_ptr, nb_box, leaf_start, leaf_count, xs,
                                                                          ys, nxs, nys, rho, k, form, eta, ip_ptr, ip, coef,
                                                                          out)));
}

}  // namespace

extern "C" int ifgf2d_eval_offsurface_setup(ifgf2d_ctx* ctx, long long m, const double* xp, const double* yp) {
    if (!ctx || m < 0 || (m > 0 && (!xp || !yp))) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    if (!ctx->ifgf_ready) return fail(ctx, IFGF2D_ERR_STATE, "setup before an off-surface evaluation plan");
    free_eval(ctx);
    ctx->ew = new EvalWork;
    EvalWork& W = *ctx->ew;
    W.M = m;
    if (m == 0) return IFGF2D_OK;
    const std::vector<double> tx(xp, xp + m), ty(yp, yp + m);
    for (long long t = 0; t < m; ++t)
        if (!std::isfinite(tx[t]) || !std::isfinite(ty[t])) return fail(ctx, IFGF2D_ERR_ARG, "non-finite target coordinate");
    Tree& E = W.E;
    std::string msg = build_target_tree(ctx->T, tx, ty, E);
    if (!msg.empty()) { free_eval(ctx); return fail(ctx, IFGF2D_ERR_GEOMETRY, msg); }
    const int D = E.nlevels - 1, P = E.P;
    const TreeLevel& LD = E.L[D];
    const int ncl = (int)LD.cone_nonrel.size();
    cudaStream_t s = ctx->stream;
    CK(W.tx.upload(tx)); CK(W.ty.upload(ty));
    if (ncl > 0) {
        std::vector<long long> loff(ncl + 1, 0);
        for (int c = 0; c < ncl; ++c) loff[c + 1] = loff[c] + (long long)P * E.leaf_count[LD.cone_box[c]];
        CK(W.nodes.alloc((size_t)ncl * P));
        CK(build_leaf_nodes(E, W.nodes.p, s));
        CK(W.leaf_cone_box.upload(LD.cone_box)); CK(W.leaf_off.upload(loff));
        CK(W.leafL.alloc(loff[ncl]));
        launch_leaf_setup(W.leaf_cone_box.p, ncl, ctx->leaf_start.p, ctx->leaf_count.p, W.leaf_off.p, W.nodes.p, ctx->xs_s.p,
                          ctx->ys_s.p, ctx->nxs_s.p, ctx->nys_s.p, ctx->T.Ps, ctx->T.Pang, ctx->k, ctx->form, ctx->eta, ctx->Gsep.p,
                          W.leafL.p, s);
        CK(cudaGetLastError());
    }
    static_assert(sizeof(InterpEntry) == sizeof(InterpEntryD), "host and device plan layouts differ");
    CK(W.pp.alloc((size_t)E.pp_total));
    CK(W.pp_ptr.upload(E.pp_ptr)); CK(W.pp_nchild.upload(E.pp_nchild));
    {
        DBuf<int> perr;
        CK(perr.alloc(1));
        CK(cudaMemsetAsync(perr.p, 0, sizeof(int), s));
        CK(build_prop_plan(E, W.pp.p, nullptr, perr.p, s));
        int bad = 0;
        CK(cudaMemcpyAsync(&bad, perr.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (bad) { free_eval(ctx); return fail(ctx, IFGF2D_ERR_GEOMETRY, "internal: a propagation node's child cone is missing"); }
    }
    CK(W.ip.upload(reinterpret_cast<const InterpEntryD*>(E.ip.data()), E.ip.size()));
    CK(W.ip_ptr.upload(E.ip_ptr));
    CK(W.nb_ptr.upload(E.nbr_ptr)); CK(W.nb_box.upload(E.nbr_box));
    CK(W.coef.alloc((size_t)std::max(1, E.total_cones) * P));
    CK(W.out.alloc(m));
    CK(cudaStreamSynchronize(s));
    return IFGF2D_OK;
}

extern "C" int ifgf2d_eval_offsurface(ifgf2d_ctx* ctx, const double* density, double* out) {
    if (!ctx || !density) return IFGF2D_ERR_ARG;
    AllocStream guard(ctx->stream);
    if (!ctx->ew) return fail(ctx, IFGF2D_ERR_STATE, "ifgf2d_eval_offsurface_setup first");
    EvalWork& W = *ctx->ew;
    if (W.M == 0) return IFGF2D_OK;
    if (!out) return IFGF2D_ERR_ARG;
    const Tree& E = W.E;
    const int N = (int)ctx->D.N, D = E.nlevels - 1, P = E.P;
    cudaStream_t s = ctx->stream;
    // weighted density in Morton order (ForwardMap::compute_intensities, BoxTree.h:954-963)
    CK(cudaMemcpyAsync(ctx->vin.p, density, sizeof(double2) * N, cudaMemcpyHostToDevice, s));
    launch_intensities(ctx->vin.p, ctx->wq.p, ctx->sorting.p, N, ctx->rho.p, s);
    const TreeLevel& LD = E.L[D];
    launch_leaf_apply_t<double>(W.leaf_cone_box.p, (int)LD.cone_nonrel.size(), LD.cone_base, ctx->leaf_start.p, ctx->leaf_count.p,
                                W.leaf_off.p, W.leafL.p, ctx->rho.p, P, W.coef.p, s);
    for (int l = D; l >= 3; --l) {
        const TreeLevel& Lp = E.L[l - 1];
        launch_propagate_t<double>(Lp.cone_base, Lp.cone_base + (int)Lp.cone_nonrel.size(), W.pp_ptr.p, W.pp_nchild.p, W.pp.p,
                                   E.Ps, E.Pang, ctx->Gsep.p, W.coef.p, s);
    }
    launch_eval_targets(W.M, W.tx.p, W.ty.p, W.nb_ptr.p, W.nb_box.p, ctx->leaf_start.p, ctx->leaf_count.p, ctx->xs_s.p,
                        ctx->ys_s.p, ctx->nxs_s.p, ctx->nys_s.p, ctx->rho.p, ctx->k, ctx->form, ctx->eta, W.ip_ptr.p, W.ip.p,
                        W.coef.p, E.Ps, E.Pang, W.out.p, s);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, W.out.p, sizeof(double2) * W.M, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return IFGF2D_OK;
}

extern "C" int ifgf2d_eval_offsurface_counts(const ifgf2d_ctx* ctx, long long out[4]) {
    if (!ctx || !out) return IFGF2D_ERR_ARG;
    if (!ctx->ew) return IFGF2D_ERR_STATE;
    const Tree& E = ctx->ew->E;
    out[0] = E.near_pairs; out[1] = E.leaf_evals; out[2] = E.prop_evals; out[3] = E.interp_evals;
    return IFGF2D_OK;
}
