// oracle_capi.cpp -- CPU ORACLE (test infrastructure only; never linked into the product).
//
// extern "C" surface of the CPU restatement so that the pytest suite and bench.py's
// CPU-baseline leg can drive it through ctypes.  Complex vectors are interleaved
// (re, im) doubles.  Functions follow ForwardMap/ForwardMap.tpp and IFGF_Source/BoxTree.h;
// see the headers for the line-by-line citations.
#include "oracle_ifgf.hpp"
#include "oracle_gmres.hpp"
#include <chrono>
#include <cstring>

using namespace orc;

namespace {
struct OracleFM {
    std::unique_ptr<ForwardMap> fm;
    std::unique_ptr<BoxTree> tree;
    std::vector<std::unordered_set<long long>> sort_sing;   // ForwardMap.tpp:567-607
    std::string err;
};
static std::vector<cd> to_c(const double* v, long long n) {
    std::vector<cd> o(n); for (long long i = 0; i < n; ++i) o[i] = cd(v[2 * i], v[2 * i + 1]); return o;
}
static void from_c(const std::vector<cd>& v, double* o) {
    for (size_t i = 0; i < v.size(); ++i) { o[2 * i] = v[i].real(); o[2 * i + 1] = v[i].imag(); }
}
}

extern "C" {

void orc_hankel(int order, long long n, const double* x, double* out) {
    for (long long i = 0; i < n; ++i) { cd h = hankel1(order, x[i]); out[2 * i] = h.real(); out[2 * i + 1] = h.imag(); }
}

// curves: types[c], closed[c], tlims[2c..2c+1], params[16c..16c+15]; junctions: triples
void* orc_fm_create(int ncurves, const int* types, const int* closed, const double* tlims, const double* params,
                    int njunc, const int* junc, int Np, double delta, double wl_per_patch, double split_k,
                    double p, int patches_per_curve, int form, double coupling) {
    std::vector<Curve> cs(ncurves);
    for (int c = 0; c < ncurves; ++c) {
        cs[c].type = types[c]; cs[c].is_closed = closed[c] != 0;
        cs[c].tlim1 = tlims[2 * c]; cs[c].tlim2 = tlims[2 * c + 1];
        std::memcpy(cs[c].p, params + 16 * c, 16 * sizeof(double));
    }
    std::vector<std::vector<Junction>> touch;
    if (njunc > 0) {
        touch.resize(ncurves);
        for (int j = 0; j < njunc; ++j) touch[junc[3 * j]].push_back({junc[3 * j + 1], junc[3 * j + 2] != 0});
    }
    OracleFM* h = new OracleFM;
    h->fm.reset(new ForwardMap(Np, delta, cs, touch, wl_per_patch, split_k, p, patches_per_curve));
    h->fm->form = form; h->fm->coupling = coupling;
    return h;
}
void orc_fm_destroy(void* h) { delete (OracleFM*)h; }
long long orc_fm_N(void* h) { return ((OracleFM*)h)->fm->N; }
long long orc_fm_num_patches(void* h) { return ((OracleFM*)h)->fm->num_patches; }

void orc_fm_points(void* h, double* xs, double* ys, double* nxs, double* nys) {
    ForwardMap& F = *((OracleFM*)h)->fm;
    for (long long i = 0; i < F.N; ++i) { xs[i] = F.xs[i]; ys[i] = F.ys[i]; nxs[i] = F.nxs[i]; nys[i] = F.nys[i]; }
}
void orc_fm_patch_info(void* h, double* t1t2, long long* ns_count) {
    ForwardMap& F = *((OracleFM*)h)->fm;
    for (long long p = 0; p < F.num_patches; ++p) {
        t1t2[2 * p] = F.patches[p].t1; t1t2[2 * p + 1] = F.patches[p].t2;
        ns_count[p] = (long long)F.patches[p].ns_idx.size();
    }
}
// per patch, concatenated: near-singular point index and t value
void orc_fm_ns_lists(void* h, long long* idx, double* t) {
    ForwardMap& F = *((OracleFM*)h)->fm;
    long long o = 0;
    for (auto& P : F.patches) for (size_t j = 0; j < P.ns_idx.size(); ++j) { idx[o] = P.ns_idx[j]; t[o] = P.ns_t[j]; ++o; }
}
// per-point factor (t2-t1)/2 * w_j * curve_jac_j and the edge jacobian
void orc_fm_point_weights(void* h, double* wq, double* edge) {
    ForwardMap& F = *((OracleFM*)h)->fm;
    for (long long p = 0; p < F.num_patches; ++p)
        for (int j = 0; j < F.Np; ++j) {
            wq[p * F.Np + j] = ab2cdjac(-1, 1, F.patches[p].t1, F.patches[p].t2) * F.fej_w[j] * F.patches[p].curve_jac[j];
            edge[p * F.Np + j] = F.patches[p].edge_sing_jac[j];
        }
}
void orc_fm_precompute(void* h, double k) { ((OracleFM*)h)->fm->compute_precomputations(k); }
// Np x (Np + n_ns) column-major, interleaved complex
void orc_fm_precomp_matrix(void* h, long long p, double* out) { from_c(((OracleFM*)h)->fm->patches[p].precomp, out); }

void orc_fm_apply_unacc(void* h, const double* in, double* out) {
    ForwardMap& F = *((OracleFM*)h)->fm;
    from_c(F.apply_unacc(to_c(in, F.N)), out);
}
void orc_fm_apply_sing(void* h, const double* in, double* out) {
    ForwardMap& F = *((OracleFM*)h)->fm;
    from_c(F.sing_near_sing(to_c(in, F.N)), out);
}

// ForwardMap.tpp:542-565 (precomputations are taken from orc_fm_precompute).  Returns 0,
// 1 when a singular or near-singular point is outside the leaf neighbourhood, 2 on other errors.
int orc_fm_setup_ifgf(void* hh, double k, int nlevels, int Ps, int Pang) {
    OracleFM* h = (OracleFM*)hh; ForwardMap& F = *h->fm;
    // the far-field kernel's wavenumber and coupling, also when no precomputation ran (far-field
    // and exclusion-matched direct sums need no rectangular-polar weights)
    F.wavenumber = k;
    F.eta = F.coupling > 0 ? F.coupling : k;
    try {
        h->tree.reset(new BoxTree(Ps, Pang));
        h->tree->Reinitialize(F.xs, F.ys, F.nxs, F.nys, nlevels, k, F.form, F.coupling > 0 ? F.coupling : k);
        h->tree->CheckIfSingandNearSingInNeighborhood(F.xs, F.ys, F.patches, F.Np);
    } catch (std::logic_error& e) {
        h->err = e.what();
        return std::string(e.what()).find("neighborhood") != std::string::npos ? 1 : 2;
    }
    const std::vector<long long>& inv = h->tree->inverse;
    h->sort_sing.assign(F.N, {});
    for (long long p = 0; p < F.num_patches; ++p) {
        std::unordered_set<long long> s;
        for (long long i = p * F.Np; i < p * F.Np + F.Np; ++i) s.insert(inv[i]);
        for (long long i = p * F.Np; i < p * F.Np + F.Np; ++i) h->sort_sing[inv[i]] = s;
    }
    for (long long p = 0; p < F.num_patches; ++p)
        for (long long i : F.patches[p].ns_idx)
            for (long long j = p * F.Np; j < p * F.Np + F.Np; ++j) h->sort_sing[inv[i]].insert(inv[j]);
    return 0;
}
const char* orc_fm_last_error(void* h) { return ((OracleFM*)h)->err.c_str(); }
void orc_fm_sorting(void* h, long long* s) { auto& t = *((OracleFM*)h)->tree; for (long long i = 0; i < t.N; ++i) s[i] = t.sorting[i]; }
// near_pairs, leaf_evals, prop_evals, interp_evals, cones, cone_levels
void orc_fm_work(void* h, long long* c) {
    auto& w = ((OracleFM*)h)->tree->wc;
    c[0] = w.near_pairs; c[1] = w.leaf_evals; c[2] = w.prop_evals; c[3] = w.interp_evals; c[4] = w.cones; c[5] = w.cone_levels;
}
// per level l = 2..nlevels-1: number of relevant boxes and relevant cones
void orc_fm_level_stats(void* h, long long* boxes, long long* cones) {
    auto& t = *((OracleFM*)h)->tree;
    for (int l = 2; l < t.nlevels; ++l) { boxes[l] = (long long)t.levels[l]->relboxes.size(); cones[l] = (long long)t.levels[l]->rel2box.size(); }
}

// ForwardMap.tpp:609-646
void orc_fm_apply_acc(void* hh, const double* in, double* out) {
    OracleFM* h = (OracleFM*)hh; ForwardMap& F = *h->fm;
    std::vector<cd> d = to_c(in, F.N);
    std::vector<cd> sns = F.sing_near_sing(d);
    F.compute_intensities(d);
    h->tree->Solve(d, &h->sort_sing);
    for (long long i = 0; i < F.N; ++i) sns[i] += d[i];
    F.add_jump(to_c(in, F.N), sns);
    from_c(sns, out);
}
// BoxTree::Solve on given intensities (original order in and out), with the exclusion sets
void orc_fm_ifgf_far(void* hh, const double* in, double* out) {
    OracleFM* h = (OracleFM*)hh; ForwardMap& F = *h->fm;
    std::vector<cd> d = to_c(in, F.N);
    h->tree->Solve(d, &h->sort_sing);
    from_c(d, out);
}
// O(N^2) sum excluding the same pairs as sort_sing_point (tests/IFGF/IgnoreSingNSing.cpp:65-117),
// on given intensities, original order in and out.  Rows [row0, row1) only.
void orc_fm_direct_excluded(void* hh, const double* in, double* out, long long row0, long long row1) {
    OracleFM* h = (OracleFM*)hh; ForwardMap& F = *h->fm;
    const std::vector<long long>& inv = h->tree->inverse;
    std::vector<cd> d = to_c(in, F.N);
    for (long long t = row0; t < row1; ++t) {
        cd s = 0.0;
        for (long long j = 0; j < F.N; ++j) {
            if (j == t || h->sort_sing[inv[t]].count(inv[j])) continue;
            s += GF_form(F.form, F.xs[t], F.ys[t], F.xs[j], F.ys[j], F.nxs[j], F.nys[j], F.wavenumber, F.eta) * d[j];
        }
        out[2 * (t - row0)] = s.real(); out[2 * (t - row0) + 1] = s.imag();
    }
}

// ForwardMap.tpp:658-697 (precomputations / IFGF set-up must have been done)
int orc_fm_solve(void* hh, const double* rhs, double* x, int accelerated, double tol, long long restart,
                 long long maxit, long long* iters, double* err, long long* matvecs, int exact_adjoint) {
    OracleFM* h = (OracleFM*)hh; ForwardMap& F = *h->fm;
    auto A = [&](const std::vector<cd>& in, std::vector<cd>& o) {
        if (accelerated) {
            std::vector<cd> d = in;
            std::vector<cd> sns = F.sing_near_sing(d);
            F.compute_intensities(d);
            h->tree->Solve(d, &h->sort_sing);
            for (long long i = 0; i < F.N; ++i) sns[i] += d[i];
            F.add_jump(in, sns);
            o = sns;
        } else {
            o = F.apply_unacc(in);
        }
    };
    std::vector<cd> xv;
    GmresResult R = householder_gmres(A, to_c(rhs, F.N), xv, restart, maxit, tol, exact_adjoint != 0);
    from_c(xv, x);
    *iters = R.iters; *err = R.error; *matvecs = R.matvecs;
    return R.ok ? (R.error <= tol ? 0 : 1) : 2;
}

void orc_fm_propagate(void* hh, long long M, const double* xp, const double* yp, const double* dens, double* out) {
    ForwardMap& F = *((OracleFM*)hh)->fm;
    std::vector<double> X(xp, xp + M), Y(yp, yp + M);
    from_c(F.propagate_unacc(X, Y, to_c(dens, F.N), F.wavenumber), out);
}

}  // extern "C"
