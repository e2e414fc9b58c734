// group.cu -- many obstacles as one block-diagonal operator (C ABI ifgf2d_group_*).
//
// The reference solves one obstacle per ForwardMap::solve (ForwardMap.tpp:658-697).  A group
// merges the discretisations and IFGF trees of many prepared contexts into one context whose
// tables hold every member side by side, so that each phase of the set-up and of an apply is
// one launch over all members, however uneven their sizes:
// * points, patches and rectangular-polar columns are concatenated (member offsets);
// * tree levels are aligned from the leaves: merged level m holds member o's level
//   m - (Dmax - D_o), D_o its leaf level and Dmax the deepest, so every propagation step of
//   every member is one range of parent cones;
// * the set-up kernels take each member's wavenumber per item (leaf box, leaf cone, column),
//   and the propagation plan is built member by member into the merged arrays.
// GMRES then runs for all members at once with per-member (segmented) Gram-Schmidt sums,
// rotations, estimates and stop tests (ifgf2d_group_solve).
#include "context.hpp"
#include "host_threads.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

struct ifgf2d_group {
    ifgf2d_ctx* g = nullptr;            // the merged context
    int n = 0;                          // members
    std::vector<long long> off;         // per member: first point (n + 1 entries)
    std::vector<double> k, eta;         // per member
    std::string err;
    // segmented GMRES workspace (group_gmres)
    int m = 0;
    DBuf<double2> V, w, vin, t, H, hh, part, Y, hn, b, x, r, d;
    DBuf<int> seg_of, chunk_seg, seg_chunk_ptr, jdev, act;
    DBuf<long long> chunk_lo;
    DBuf<double> par;
    DBuf<double2> lsR, lsg, lsgs;
    DBuf<double> lsgc, lssc;
    DBuf<int> lsst;
    int nchunk = 0;
    // flexible GMRES with the spectral preconditioner: the preconditioned columns and z_j
    DBuf<double2> Z, zt;
    // per apply mode (FP64, complex64) x (plain, spectral preconditioner): one restart cycle
    cudaGraphExec_t exec[4] = {nullptr, nullptr, nullptr, nullptr};
    void drop_graphs() { for (auto& e : exec) if (e) { cudaGraphExecDestroy(e); e = nullptr; } }
    ~ifgf2d_group() {
        drop_graphs();
        // the workspace was allocated in order on the merged context's stream: free it before
        // that stream goes with the context
        for (DBuf<double2>* b : {&V, &w, &vin, &t, &H, &hh, &part, &Y, &hn, &this->b, &x, &r, &d, &lsR, &lsg, &lsgs, &Z, &zt}) b->release();
        for (DBuf<int>* b : {&seg_of, &chunk_seg, &seg_chunk_ptr, &jdev, &act, &lsst}) b->release();
        for (DBuf<double>* b : {&par, &lsgc, &lssc}) b->release();
        chunk_lo.release();
        if (g) ifgf2d_destroy(g);
    }
};

namespace {

int gfail(ifgf2d_group* G, int code, const std::string& msg) {
    G->err = msg;
    return code;
}

// the merged discretisation: members' arrays side by side with their indices shifted
void merge_discretisation(ifgf2d_ctx* const* mem, int n, Discretisation& D, std::vector<long long>& off) {
    const Discretisation& D0 = mem[0]->D;
    D = Discretisation();
    D.Np = D0.Np; D.delta = D0.delta; D.p = D0.p;
    D.fej_n = D0.fej_n; D.fej_w = D0.fej_w; D.fej_ns_n = D0.fej_ns_n; D.fej_ns_w = D0.fej_ns_w;
    off.assign(n + 1, 0);
    D.ns_ptr.assign(1, 0);
    for (int o = 0; o < n; ++o) {
        const Discretisation& M = mem[o]->D;
        const long long p0 = D.num_patches, i0 = D.N;
        const int c0 = (int)D.curves.size();
        D.curves.insert(D.curves.end(), M.curves.begin(), M.curves.end());
        auto app = [](std::vector<double>& a, const std::vector<double>& b) { a.insert(a.end(), b.begin(), b.end()); };
        app(D.x, M.x); app(D.y, M.y); app(D.nx, M.nx); app(D.ny, M.ny); app(D.t, M.t); app(D.wq, M.wq);
        app(D.edge_jac, M.edge_jac); app(D.kappa, M.kappa); app(D.t1, M.t1); app(D.t2, M.t2);
        for (int p : M.patch_of) D.patch_of.push_back((int)(p + p0));
        for (int c : M.curve_of) D.curve_of.push_back(c + c0);
        D.ist1sing.insert(D.ist1sing.end(), M.ist1sing.begin(), M.ist1sing.end());
        D.ist2sing.insert(D.ist2sing.end(), M.ist2sing.begin(), M.ist2sing.end());
        const int q0 = (int)D.ns_idx.size();
        for (long long p = 0; p < M.num_patches; ++p) D.ns_ptr.push_back(q0 + M.ns_ptr[p + 1]);
        for (long long i : M.ns_idx) D.ns_idx.push_back(i + i0);
        D.ns_t.insert(D.ns_t.end(), M.ns_t.begin(), M.ns_t.end());
        D.N += M.N;
        D.num_patches += M.num_patches;
        off[o + 1] = D.N;
    }
}

// the merged tree, levels aligned from the leaves; fills per member and level its first global
// cone id (cbase[o][l]) and the first plan entry of its slots with children at level l
// (ebase[o][l])
std::string merge_trees(ifgf2d_ctx* const* mem, int n, const std::vector<long long>& off, Tree& T,
                        std::vector<std::vector<int>>& cbase, std::vector<std::vector<long long>>& ebase) {
    const Tree& T0 = mem[0]->T;
    int Dmax = 0;
    for (int o = 0; o < n; ++o) Dmax = std::max(Dmax, mem[o]->T.nlevels - 1);
    T = Tree();
    T.nlevels = Dmax + 1; T.Ps = T0.Ps; T.Pang = T0.Pang; T.P = T0.P; T.k = 0.0;
    T.N = off[n];
    T.L.resize(T.nlevels);
    cbase.assign(n, {});
    ebase.assign(n, {});
    for (int o = 0; o < n; ++o) { cbase[o].assign(mem[o]->T.nlevels, 0); ebase[o].assign(mem[o]->T.nlevels, 0); }
    auto lev = [&](int o, int m) { return m - (Dmax - (mem[o]->T.nlevels - 1)); };   // member level of merged level m
    // cones, merged level by merged level (ids ascend with the level, as in one tree)
    int total = 0;
    for (int m = 2; m <= Dmax; ++m) {
        TreeLevel& L = T.L[m];
        L.level = m;
        L.cone_base = total;
        int boxes = 0;
        for (int o = 0; o < n; ++o) {
            const int l = lev(o, m);
            if (l < 2) continue;
            const TreeLevel& Lo = mem[o]->T.L[l];
            cbase[o][l] = total + (int)L.cone_nonrel.size();
            L.cone_nonrel.insert(L.cone_nonrel.end(), Lo.cone_nonrel.begin(), Lo.cone_nonrel.end());
            for (int b : Lo.cone_box) L.cone_box.push_back(b + boxes);
            boxes += (int)Lo.boxes.size();
        }
        total += (int)L.cone_nonrel.size();
    }
    T.total_cones = total;
    // points in Morton order, member by member, and the leaf boxes
    T.sorting.resize(T.N); T.inverse.resize(T.N); T.xs.resize(T.N); T.ys.resize(T.N);
    T.point_leaf.resize(T.N);
    T.ip_ptr.assign(T.N + 1, 0);
    T.nbr_ptr.assign(1, 0);
    int leaf0 = 0;
    for (int o = 0; o < n; ++o) {
        const Tree& To = mem[o]->T;
        const long long i0 = off[o];
        for (long long i = 0; i < To.N; ++i) {
            T.sorting[i0 + i] = i0 + To.sorting[i];
            T.inverse[i0 + i] = i0 + To.inverse[i];
            T.xs[i0 + i] = To.xs[i];
            T.ys[i0 + i] = To.ys[i];
            T.point_leaf[i0 + i] = leaf0 + To.point_leaf[i];
        }
        for (size_t b = 0; b < To.leaf_start.size(); ++b) {
            T.leaf_start.push_back((int)(To.leaf_start[b] + i0));
            T.leaf_count.push_back(To.leaf_count[b]);
            for (int q = To.nbr_ptr[b]; q < To.nbr_ptr[b + 1]; ++q) T.nbr_box.push_back(To.nbr_box[q] + leaf0);
            T.nbr_ptr.push_back((int)T.nbr_box.size());
        }
        leaf0 += (int)To.leaf_start.size();
        T.near_pairs += To.near_pairs; T.leaf_evals += To.leaf_evals;
        T.prop_evals += To.prop_evals; T.interp_evals += To.interp_evals;
    }
    // the leaf level's boxes per cone index the merged leaf boxes
    {
        TreeLevel& LD = T.L[Dmax];
        LD.cone_box.clear();
        int lb0 = 0;
        for (int o = 0; o < n; ++o) {
            const Tree& To = mem[o]->T;
            for (int b : To.L[To.nlevels - 1].cone_box) LD.cone_box.push_back(b + lb0);
            lb0 += (int)To.leaf_start.size();
        }
        LD.cone_ptr.assign(1, 0);
    }
    // interpolation plan: member entries with their cones renumbered
    T.ip.resize((size_t)T.interp_evals);
    {
        long long e0 = 0;
        for (int o = 0; o < n; ++o) {
            const Tree& To = mem[o]->T;
            const long long i0 = off[o];
            for (long long i = 0; i < To.N; ++i) T.ip_ptr[i0 + i + 1] = e0 + To.ip_ptr[i + 1];
            const std::vector<int>& cb = cbase[o];
            const Tree* Tp = &To;
            InterpEntry* out = T.ip.data() + e0;
            bool bad = false;
            parallel_for((long long)To.ip.size(), [&](long long a, long long b) {
                for (long long e = a; e < b; ++e) {
                    InterpEntry q = Tp->ip[e];
                    const int l = q.pad;
                    if (l < 2 || l >= Tp->nlevels) { bad = true; continue; }
                    q.cone = cb[l] + (q.cone - Tp->L[l].cone_base);
                    out[e] = q;
                }
            }, 1 << 14);
            if (bad) return "internal: interpolation entry without a level";
            e0 += (long long)To.ip.size();
        }
    }
    // propagation CSR over merged parent cone ids, and each member's entry bases
    T.pp_ptr.assign(1, 0);
    for (int m = 2; m <= Dmax; ++m)
        for (int o = 0; o < n; ++o) {
            const int l = lev(o, m);
            if (l < 2) continue;
            const Tree& To = mem[o]->T;
            const TreeLevel& Lo = To.L[l];
            if (l + 1 < To.nlevels) ebase[o][l + 1] = T.pp_ptr.back();
            for (size_t c = 0; c < Lo.cone_nonrel.size(); ++c) {
                const int nch = To.pp_nchild[Lo.cone_base + c];
                T.pp_nchild.push_back(nch);
                T.pp_ptr.push_back(T.pp_ptr.back() + (long long)nch * T.P);
            }
        }
    T.pp_total = T.pp_ptr.back();
    return "";
}

}  // namespace

extern "C" int ifgf2d_group_create(ifgf2d_ctx* const* members, int n, ifgf2d_group** out) {
    if (!out || !members || n <= 0 || n > 1024) return IFGF2D_ERR_ARG;   // one thread per member in the Givens step
    *out = nullptr;
    ifgf2d_group* G = new ifgf2d_group;
    *out = G;
    G->n = n;
    const ifgf2d_ctx* m0 = members[0];
    for (int o = 0; o < n; ++o) {
        const ifgf2d_ctx* c = members[o];
        if (!c) return gfail(G, IFGF2D_ERR_ARG, "a member context is NULL");
        if (!c->prep_ready) return gfail(G, IFGF2D_ERR_STATE, "every member must be prepared (ifgf2d_prepare) before grouping");
        if (c->D.Np != m0->D.Np || c->T.Ps != m0->T.Ps || c->T.Pang != m0->T.Pang || c->form != m0->form || c->D.p != m0->D.p)
            return gfail(G, IFGF2D_ERR_ARG, "members must share Np, Ps, Pang, p and the formulation");
        G->k.push_back(c->prep_k);
        G->eta.push_back(c->opt.coupling > 0 ? c->opt.coupling : c->prep_k);
    }
    // the merged context: host tables from the merged discretisation and trees
    ifgf2d_ctx* g = new ifgf2d_ctx;
    G->g = g;
    g->opt = m0->opt;
    g->form = m0->form;
    merge_discretisation(members, n, g->D, G->off);
    if (int rc = init_host_tables(g)) { G->err = g->err; return rc; }
    std::vector<std::vector<int>> cbase;
    std::vector<std::vector<long long>> ebase;
    std::string msg = merge_trees(members, n, G->off, g->T, cbase, ebase);
    if (!msg.empty()) return gfail(G, IFGF2D_ERR_GEOMETRY, msg);
    const Tree& T = g->T;
    const Discretisation& D = g->D;
    // device: discretisation, rectangular-polar weights with each member's wavenumber
    if (int rc = ensure_device_ctx(g)) { G->err = g->err; return rc; }
    ifgf2d_ctx* ctx = g;   // for CK
    AllocStream guard(g->stream);
    std::vector<int> member_of_patch(D.num_patches);
    for (int o = 0; o < n; ++o)
        for (long long p = G->off[o] / D.Np; p < G->off[o + 1] / D.Np; ++p) member_of_patch[p] = o;
    std::vector<double2> kc(g->hcols.size());
    for (size_t c = 0; c < g->hcols.size(); ++c) {
        const int o = member_of_patch[g->hcols[c].patch];
        kc[c] = make_double2(G->k[o], G->eta[o]);
    }
    DBuf<double2> keta_col, keta_box, keta_cone;
    CK(keta_col.upload(kc));
    const int ncols = (int)g->hcols.size();
    CK(g->M.alloc((size_t)ncols * D.Np));
    CK(g->W.alloc((size_t)ncols * D.Np));
    launch_rp_precompute(g->cols.p, ncols, g->patches.p, g->curves.p, g->nsn.p, g->nsw.p, D.Np, D.p, 0.0, g->form, 0.0, g->M.p,
                         g->stream, keta_col.p);
    CK(cudaGetLastError());
    launch_rp_fold(g->M.p, g->cols.p, ncols, g->edge.p, g->patches.p, D.Np, g->W.p, g->stream);
    CK(cudaGetLastError());
    g->precomputed = true;
    g->counts[6] = (long long)ncols * D.Np;
    // IFGF tables: (k, eta) per leaf box and leaf cone; the members' leaf nodes and plans on the device
    std::vector<double2> kb, kl;
    std::vector<long long> node_off(n + 1, 0);
    for (int o = 0; o < n; ++o) {
        const Tree& To = members[o]->T;
        const double2 ke = make_double2(G->k[o], G->eta[o]);
        kb.insert(kb.end(), To.leaf_start.size(), ke);
        kl.insert(kl.end(), To.L[To.nlevels - 1].cone_nonrel.size(), ke);
        node_off[o + 1] = node_off[o] + (long long)To.L[To.nlevels - 1].cone_nonrel.size() * To.P;
    }
    CK(keta_box.upload(kb));
    CK(keta_cone.upload(kl));
    SetupExtra ex;
    ex.keta_leafbox = keta_box.p;
    ex.keta_leafcone = keta_cone.p;
    ex.build_nodes = [&](LeafNode* out, cudaStream_t s) -> cudaError_t {
        for (int o = 0; o < n; ++o) {
            const cudaError_t e = build_leaf_nodes(members[o]->T, out + node_off[o], s);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    ex.build_plan = [&](PropE<double>* pp64, PropE<float>* pp32, int* err, cudaStream_t s) -> cudaError_t {
        for (int o = 0; o < n; ++o) {
            const cudaError_t e = build_prop_plan(members[o]->T, pp64, pp32, err, s, cbase[o].data(), ebase[o].data());
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    if (int rc = setup_tables(g, 0.0, T.nlevels, &ex)) { G->err = g->err; return rc; }
    CK(cudaStreamSynchronize(g->stream));
    return IFGF2D_OK;
}

extern "C" int ifgf2d_group_destroy(ifgf2d_group* G) {
    if (!G) return IFGF2D_ERR_ARG;
    delete G;
    return IFGF2D_OK;
}
extern "C" const char* ifgf2d_group_last_error(const ifgf2d_group* G) {
    if (!G) return "NULL group";
    if (G->err.empty() && G->g) return G->g->err.c_str();   // a CUDA error recorded on the merged context
    return G->err.c_str();
}
extern "C" long long ifgf2d_group_num_unknowns(const ifgf2d_group* G) { return G && G->g ? G->g->D.N : -1; }
extern "C" int ifgf2d_group_offsets(const ifgf2d_group* G, long long* off) {
    if (!G || !off) return IFGF2D_ERR_ARG;
    std::copy(G->off.begin(), G->off.end(), off);
    return IFGF2D_OK;
}

// y = A x for all members at once, host vectors in member order
extern "C" int ifgf2d_group_apply(ifgf2d_group* G, const double* x, double* y, int mode) {
    if (!G || !x || !y) return IFGF2D_ERR_ARG;
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_IFGF_MIXED) return gfail(G, IFGF2D_ERR_ARG, "group applies are IFGF or IFGF_MIXED");
    ifgf2d_ctx* ctx = G->g;
    if (!ctx || !ctx->ifgf_ready) return gfail(G, IFGF2D_ERR_STATE, "group not set up");
    const long long N = ctx->D.N;
    if (!all_finite(x, 2 * N)) return gfail(G, IFGF2D_ERR_NONFINITE, "non-finite value in the density");
    AllocStream guard(ctx->stream);
    CK(cudaMemcpyAsync(ctx->vin.p, x, sizeof(double2) * N, cudaMemcpyHostToDevice, ctx->stream));
    if (int rc = apply_single(ctx, ctx->vin.p, ctx->vout.p, mode)) { G->err = ctx->err; return rc; }
    CK(cudaMemcpyAsync(y, ctx->vout.p, sizeof(double2) * N, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->kerr.p) {
        int v = 0;
        CK(cudaMemcpy(&v, ctx->kerr.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (v) return gfail(G, IFGF2D_ERR_CUDA, "a kernel's bounded wait for a bulk copy ran out");
    }
    return IFGF2D_OK;
}

// ---------------------------------------------------------------- segmented GMRES
namespace {

constexpr long long kSegChunk = 2048;

// workspace for restart length m; the segment layout (chunks never cross a member's range)
int group_workspace(ifgf2d_group* G, int m) {
    ifgf2d_ctx* ctx = G->g;
    const long long N = ctx->D.N;
    const int B = G->n;
    if (!G->seg_of.p) {
        std::vector<int> seg(N), sc(B + 1, 0);
        std::vector<long long> lo;
        for (int s = 0; s < B; ++s) {
            for (long long i = G->off[s]; i < G->off[s + 1]; ++i) seg[i] = s;
            sc[s] = (int)lo.size();
            for (long long a = G->off[s]; a < G->off[s + 1]; a += kSegChunk) lo.push_back(a);
        }
        sc[B] = (int)lo.size();
        lo.push_back(N);
        G->nchunk = (int)lo.size() - 1;
        CK(G->seg_of.upload(seg)); CK(G->seg_chunk_ptr.upload(sc)); CK(G->chunk_lo.upload(lo));
    }
    if (G->m != m) {
        G->drop_graphs();
        const size_t ldh = (size_t)m + 1;
        CK(G->V.alloc((size_t)N * ldh)); CK(G->w.alloc(N)); CK(G->vin.alloc(N)); CK(G->t.alloc(N));
        CK(G->H.alloc(ldh * m * B)); CK(G->hh.alloc(ldh * B)); CK(G->part.alloc(ldh * G->nchunk));
        CK(G->Y.alloc((size_t)m * B)); CK(G->hn.alloc(B)); CK(G->jdev.alloc(1)); CK(G->act.alloc(m));
        CK(G->par.alloc((size_t)3 * B));
        CK(G->lsR.alloc((size_t)B * ldh * m)); CK(G->lsg.alloc((size_t)B * ldh)); CK(G->lsgc.alloc((size_t)B * m));
        CK(G->lsgs.alloc((size_t)B * m)); CK(G->lssc.alloc((size_t)3 * B)); CK(G->lsst.alloc((size_t)4 * B));
        G->m = m;
    }
    return IFGF2D_OK;
}

SegDesc seg_desc(ifgf2d_group* G) {
    return SegDesc{G->g->D.N, G->n, G->nchunk, G->chunk_lo.p, G->seg_chunk_ptr.p, G->seg_of.p, G->part.p};
}

// per-member norms of a device vector, to the host
int seg_norms_host(ifgf2d_group* G, const double2* v, std::vector<double>& out) {
    ifgf2d_ctx* ctx = G->g;
    launch_seg_norms(seg_desc(G), v, G->hn.p, ctx->stream);
    std::vector<double2> h(G->n);
    CK(cudaMemcpyAsync(h.data(), G->hn.p, sizeof(double2) * G->n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    out.resize(G->n);
    for (int s = 0; s < G->n; ++s) out[s] = h[s].x;
    return IFGF2D_OK;
}

// x = A^{-1} b for every member, initial guess 0: GMRES per member (segment) in lock step.  One
// restart cycle is one launch of a captured graph whose while-loop body is an iteration (copy of
// v_j, the group apply, per-member Gram-Schmidt and norms, per-member Givens step); member s stops
// when |g_{j+1}| / ||r0_s|| < tol[s], after its iteration limit, or at the start when skip[s].
int group_gmres(ifgf2d_group* G, const double2* b, double2* x, int mode, const std::vector<double>& tol, int restart, int max_iters,
                const std::vector<char>& skip, std::vector<int>& iters, std::vector<double>& est, int passes,
                SpectralWork* spec = nullptr) {
    ifgf2d_ctx* ctx = G->g;
    const long long N = ctx->D.N;
    const int B = G->n;
    long long minseg = N;
    for (int s = 0; s < B; ++s) minseg = std::min(minseg, G->off[s + 1] - G->off[s]);
    const int m = (int)std::max<long long>(1, std::min<long long>(restart, N));
    if (int rc = group_workspace(G, m)) return rc;
    cudaStream_t s = ctx->stream;
    const SegDesc S = seg_desc(G);
    const LsqBatchDev L{G->lsR.p, G->lsg.p, G->lsgc.p, G->lsgs.p, G->lsst.p, G->lssc.p, m, B};
    const int gi = (mode == IFGF2D_APPLY_IFGF_MIXED ? 1 : 0) + (spec ? 2 : 0);
    if (spec && G->Z.n != (size_t)N * m) { CK(G->Z.alloc((size_t)N * m)); CK(G->zt.alloc(N)); }
    if (!G->exec[gi]) {
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
            return gfail(G, IFGF2D_ERR_CUDA, std::string("building the group GMRES graph: ") + cudaGetErrorString(e));
        }
        launch_copy_col(G->V.p, N, G->jdev.p, G->vin.p, nullptr, s);
        const double2* src = G->vin.p;
        if (spec) {   // flexible GMRES: z_j = M v_j into Z[:, j], then w = A z_j
            spectral_launch(spec, G->vin.p, G->zt.p, ctx->D.Np, s);
            launch_store_col(G->zt.p, N, G->jdev.p, G->Z.p, s);
            src = G->zt.p;
        }
        const int rc = apply_single(ctx, src, G->w.p, mode);
        launch_seg_arnoldi(S, G->V.p, m, G->jdev.p, G->w.p, G->hh.p, G->H.p, G->hn.p, passes, s);
        launch_lsq_givens_batch_dev(G->H.p, G->jdev.p, L, G->act.p, cond, s);
        cudaGraph_t body = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(s, &body);
        if (rc != IFGF2D_OK || ec != cudaSuccess) {
            cudaGraphDestroy(graph);
            if (rc != IFGF2D_OK) { G->err = ctx->err; return rc; }
            CK(ec);
        }
        e = cudaGraphInstantiate(&G->exec[gi], graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { G->exec[gi] = nullptr; CK(e); }
    }
    CK(cudaMemsetAsync(x, 0, sizeof(double2) * N, s));
    iters.assign(B, 0);
    est.assign(B, 0.0);
    std::vector<double> beta, r0n;
    CK(cudaMemcpyAsync(G->w.p, b, sizeof(double2) * N, cudaMemcpyDeviceToDevice, s));
    if (int rc = seg_norms_host(G, G->w.p, beta)) return rc;
    r0n = beta;
    std::vector<char> done(B, 0);
    for (int r = 0; r < B; ++r) { done[r] = skip[r] || beta[r] == 0.0; est[r] = done[r] ? 0.0 : 1.0; }
    std::vector<double> hpar(3 * B);
    std::vector<int> hst(4 * B);
    std::vector<double> hsc(3 * B);
    auto all_done = [&]() { for (int r = 0; r < B; ++r) if (!done[r]) return false; return true; };
    while (!all_done()) {
        // v_0 = r / ||r|| per member (G->hn holds the norms)
        launch_seg_scale0(S, G->w.p, G->hn.p, G->V.p, s);
        CK(cudaMemsetAsync(G->H.p, 0, sizeof(double2) * (size_t)(m + 1) * m * B, s));
        for (int r = 0; r < B; ++r) {
            const long long cap = std::min<long long>(max_iters, G->off[r + 1] - G->off[r]);
            hpar[3 * r] = r0n[r];
            hpar[3 * r + 1] = tol[r];
            hpar[3 * r + 2] = done[r] ? 0.0 : (double)std::max<long long>(0, cap - iters[r]);
        }
        CK(cudaMemcpyAsync(G->par.p, hpar.data(), sizeof(double) * 3 * B, cudaMemcpyHostToDevice, s));
        launch_lsq_init_batch(L, G->hn.p, G->par.p, s);
        CK(cudaMemsetAsync(G->jdev.p, 0, sizeof(int), s));
        CK(cudaGraphLaunch(G->exec[gi], s));
        launch_lsq_solve_batch(L, m, G->Y.p, s);
        CK(cudaMemcpyAsync(hst.data(), G->lsst.p, sizeof(int) * 4 * B, cudaMemcpyDeviceToHost, s));
        CK(cudaMemcpyAsync(hsc.data(), G->lssc.p, sizeof(double) * 3 * B, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        CK(cudaGetLastError());
        int ncols = 0;
        bool progress = false;
        for (int r = 0; r < B; ++r) {
            ncols = std::max(ncols, hst[4 * r + 1]);
            if (done[r]) continue;
            iters[r] += hst[4 * r + 3];
            est[r] = hsc[3 * r];
            progress = progress || hst[4 * r + 3] > 0;
            if (hst[4 * r] || hst[4 * r + 3] <= 0) done[r] = 1;
        }
        launch_seg_axpy(S, spec ? G->Z.p : G->V.p, ncols, G->Y.p, x, s);   // x += V Y (or Z Y, flexible) per member
        if (all_done() || !progress) break;
        // restart: r = b - A x; the estimate keeps the first ||r0|| (opGMRES.hpp:207)
        if (int rc = apply_single(ctx, x, G->t.p, mode)) { G->err = ctx->err; return rc; }
        launch_sub(b, G->t.p, N, G->w.p, s);
        if (int rc = seg_norms_host(G, G->w.p, beta)) return rc;
        for (int r = 0; r < B; ++r) if (!done[r] && beta[r] == 0.0) { done[r] = 1; est[r] = 0.0; }
    }
    CK(cudaStreamSynchronize(s));
    CK(cudaGetLastError());
    return IFGF2D_OK;
}

}  // namespace

// GMRES for every member at once (ForwardMap::solve, ForwardMap.tpp:658-697, per member):
// host vectors of all members' unknowns in member order; per member its iterations and
// estimated error.  IFGF2D_APPLY_IFGF_MIXED: FP64 iterative refinement around complex64 inner
// solves, each member stopping on its own FP64 relative residual.
namespace {
int group_solve(ifgf2d_group* G, const double* rhs, double* xout, int mode, double tol, int restart, int max_iters, int* iters_out,
                double* est_out, SpectralWork* spec) {
    if (mode != IFGF2D_APPLY_IFGF && mode != IFGF2D_APPLY_IFGF_MIXED) return gfail(G, IFGF2D_ERR_ARG, "group solves are IFGF or IFGF_MIXED");
    ifgf2d_ctx* ctx = G->g;
    if (!ctx || !ctx->ifgf_ready) return gfail(G, IFGF2D_ERR_STATE, "group not set up");
    const long long N = ctx->D.N;
    const int B = G->n;
    if (!all_finite(rhs, 2 * N)) return gfail(G, IFGF2D_ERR_NONFINITE, "non-finite value in the right-hand side");
    AllocStream guard(ctx->stream);
    cudaStream_t s = ctx->stream;
    if (int rc = group_workspace(G, (int)std::max<long long>(1, std::min<long long>(restart, N)))) return rc;
    if (G->b.n != (size_t)N) { CK(G->b.alloc(N)); CK(G->x.alloc(N)); CK(G->r.alloc(N)); CK(G->d.alloc(N)); }
    CK(cudaMemcpyAsync(G->b.p, rhs, sizeof(double2) * N, cudaMemcpyHostToDevice, s));
    std::vector<int> iters(B, 0);
    std::vector<double> est(B, 0.0);
    std::vector<char> skip(B, 0);
    int rc;
    if (mode == IFGF2D_APPLY_IFGF) {
        std::vector<double> tv(B, tol);
        if ((rc = group_gmres(G, G->b.p, G->x.p, mode, tv, restart, max_iters, skip, iters, est, 2, spec))) return rc;
    } else {
        // FP64 iterative refinement per member: residual with the FP64 operator, correction from
        // GMRES on the complex64 operator (one Gram-Schmidt pass, as the batched inner solves)
        std::vector<double> bn, rn;
        if ((rc = seg_norms_host(G, G->b.p, bn))) return rc;
        rn = bn;
        std::vector<char> done(B, 0);
        for (int r = 0; r < B; ++r) { est[r] = bn[r] > 0 ? 1.0 : 0.0; done[r] = est[r] < tol; }
        CK(cudaMemsetAsync(G->x.p, 0, sizeof(double2) * N, s));
        CK(cudaMemcpyAsync(G->r.p, G->b.p, sizeof(double2) * N, cudaMemcpyDeviceToDevice, s));
        std::vector<double> itol(B);
        std::vector<int> it;
        std::vector<double> e;
        ctx->last_passes = 0;
        for (int outer = 0; outer < 30; ++outer) {
            bool any = false;
            int most = 0;
            for (int r = 0; r < B; ++r) {
                skip[r] = done[r] || iters[r] >= max_iters;
                any = any || !skip[r];
                most = std::max(most, iters[r]);
                itol[r] = std::max(2e-7, 0.3 * tol * bn[r] / std::max(rn[r], 1e-300));
            }
            if (!any) break;
            ++ctx->last_passes;
            if ((rc = group_gmres(G, G->r.p, G->d.p, IFGF2D_APPLY_IFGF_MIXED, itol, restart, std::max(1, max_iters - most), skip, it, e, 1,
                                  spec)))
                return rc;
            for (int r = 0; r < B; ++r) iters[r] += it[r];
            {
                const double2 one = make_double2(1.0, 0.0);
                CK(cudaMemcpyAsync(G->hh.p, &one, sizeof(double2), cudaMemcpyHostToDevice, s));
                launch_multi_axpy(G->d.p, N, 1, G->hh.p, 1.0, N, G->x.p, s);   // x += d (skipped members have d = 0)
            }
            if ((rc = apply_single(ctx, G->x.p, G->t.p, IFGF2D_APPLY_IFGF))) { G->err = ctx->err; return rc; }
            launch_sub(G->b.p, G->t.p, N, G->r.p, s);
            if ((rc = seg_norms_host(G, G->r.p, rn))) return rc;
            for (int r = 0; r < B; ++r) {
                est[r] = bn[r] > 0 ? rn[r] / bn[r] : 0.0;
                done[r] = est[r] < tol;
            }
        }
    }
    CK(cudaMemcpyAsync(xout, G->x.p, sizeof(double2) * N, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    bool ok = true;
    for (int r = 0; r < B; ++r) {
        if (iters_out) iters_out[r] = iters[r];
        if (est_out) est_out[r] = est[r];
        ok = ok && est[r] < tol;
    }
    return ok ? IFGF2D_OK : IFGF2D_ERR_NOCONV;
}
}  // namespace

extern "C" int ifgf2d_group_solve(ifgf2d_group* G, const double* rhs, double* xout, int mode, double tol, int restart,
                                  int max_iters, int* iters_out, double* est_out) {
    if (!G || !rhs || !xout || restart <= 0 || max_iters <= 0) return IFGF2D_ERR_ARG;
    return group_solve(G, rhs, xout, mode, tol, restart, max_iters, iters_out, est_out, nullptr);
}

// the spectral preconditioner of the merged context, each curve with its own member's k and eta
extern "C" int ifgf2d_group_solve_flexible(ifgf2d_group* G, int precond, const double* rhs, double* xout, int mode, double tol,
                                           int restart, int max_iters, int* iters_out, double* est_out) {
    if (!G || !rhs || !xout || restart <= 0 || max_iters <= 0) return IFGF2D_ERR_ARG;
    if (precond != IFGF2D_PRECOND_SPECTRAL) return gfail(G, IFGF2D_ERR_ARG, "group solves take the spectral preconditioner only");
    ifgf2d_ctx* ctx = G->g;
    if (!ctx || !ctx->ifgf_ready) return gfail(G, IFGF2D_ERR_STATE, "group not set up");
    if (!ctx->sw) {
        const Discretisation& D = ctx->D;
        std::vector<double> kc(D.curves.size(), 0.0), ec(D.curves.size(), 0.0);
        for (long long p = 0; p < D.num_patches; ++p) {
            const long long first = p * D.Np;
            const int o = (int)(std::upper_bound(G->off.begin(), G->off.end(), first) - G->off.begin()) - 1;
            kc[D.curve_of[p]] = G->k[o];
            ec[D.curve_of[p]] = G->eta[o];
        }
        AllocStream guard(ctx->stream);
        const int rc = spectral_setup(ctx, IFGF2D_SPECTRAL_DEFAULT_SCALE, kc.data(), ec.data());
        if (rc != IFGF2D_OK) { G->err = ctx->err; return rc; }
        G->drop_graphs();
    }
    return group_solve(G, rhs, xout, mode, tol, restart, max_iters, iters_out, est_out, ctx->sw);
}
