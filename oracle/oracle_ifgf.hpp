// oracle_ifgf.hpp -- CPU ORACLE (test infrastructure only; never linked into the product).
//
// Restatement of the IFGF accelerator of IFGF2D:
//   IFGF_Source/Level.h:18-455        (per-level cones, Morton codes, coordinate maps)
//   IFGF_Source/Interpolator.h:7-122  (2D tensor Chebyshev interpolation)
//   IFGF_Source/Chebyshev.h:10-68, PolarCoordinates.h:8-57, Vector.h:13-41
//   IFGF_Source/BoxTree.h:24-1171     (tree set-up, SingularInteractions, LevelDEvaluations,
//                                      Propagation, Interpolation, Solve, neighbourhood check)
// Deviations: Level.h uses uint64_t without <cstdint> (fixed); Ps/Pang are run-time values;
// `levels_` are owned (BoxTree.h:223 leaks them); work counters are added for the roofline.
#pragma once

#include "oracle_fm.hpp"
#include <cstdint>
#include <map>
#include <set>

namespace orc {

// PolarCoordinates.h:8-27
static inline double Atan2_0_2pi(double y, double x) {
    if (x > 0 && y >= 0) return std::atan(y / x);
    else if (x > 0 && y < 0) return std::atan(y / x) + 2.0 * PI;
    else if (x < 0 && y > 0) return std::atan(y / x) + PI;
    else if (x < 0 && y == 0) return PI;
    else if (x < 0 && y < 0) return std::atan(y / x) + PI;
    else if (x == 0 && y > 0) return PI / 2;
    else if (x == 0 && y < 0) return 3.0 * PI / 2;
    return 0;
}
static inline void CartToPol(double& x, double& y) {
    const double r = std::sqrt(x * x + y * y);
    if (r == 0.0) { x = 0.0; y = 0.0; return; }
    const double th = Atan2_0_2pi(y, x);
    x = r; y = th;
}
static inline void PolToCart(double& r, double& th) {
    const double x = r * std::cos(th), y = r * std::sin(th);
    r = x; th = y;
}

// Level.h:190-226
static inline uint64_t splitBy2(unsigned int a, int level) {
    uint64_t x = a;
    x &= (static_cast<uint64_t>(1) << (level + 1)) - 1;
    x = (x | (x << 16)) & 0xFFFF0000FFFFull;
    x = (x | (x << 8)) & 0xFF00FF00FF00FFull;
    x = (x | (x << 4)) & 0xF0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}
static inline unsigned int mergeFrom2(uint64_t x) {
    x &= 0x5555555555555555ull;
    x = (x ^ (x >> 1)) & 0x3333333333333333ull;
    x = (x ^ (x >> 2)) & 0xF0F0F0F0F0F0F0Full;
    x = (x ^ (x >> 4)) & 0xFF00FF00FF00FFull;
    x = (x ^ (x >> 8)) & 0xFFFF0000FFFFull;
    x = (x ^ (x >> 16)) & 0xffffffffull;
    return (unsigned int)x;
}

// Chebyshev.h:10-24 (ascending nodes) and Interpolator.h
struct Interp2D {
    int Ps, Pang, P;
    std::vector<double> xs, xang;                   // ascending nodes
    std::vector<std::vector<double>> Ts, Tang;      // [n][i]
    Interp2D(int ps, int pang) : Ps(ps), Pang(pang), P(ps * pang) {
        xs = nodes(Ps); xang = nodes(Pang); Ts = tn(Ps); Tang = tn(Pang);
    }
    static std::vector<double> nodes(int N) {
        std::vector<double> x(N);
        for (int i = 0; i < N; ++i) x[N - 1 - i] = std::cos(PI * (2.0 * i + 1.0) / (2.0 * N));
        return x;
    }
    static std::vector<std::vector<double>> tn(int N) {
        std::vector<double> x = nodes(N);
        std::vector<std::vector<double>> T(N, std::vector<double>(N));
        for (int i = 0; i < N; ++i) { T[0][i] = 1.0; if (N > 1) T[1][i] = x[i]; }
        for (int n = 2; n < N; ++n) for (int i = 0; i < N; ++i) T[n][i] = 2.0 * x[i] * T[n - 1][i] - T[n - 2][i];
        return T;
    }
    void point(int it, double& x, double& y) const { x = xs[it % Ps]; y = xang[it / Ps]; }
    // Interpolator.h:55-77
    cd interpolate(double x, double y, const cd* c) const {
        double ts[16], tt[16];
        ts[0] = 1.0; if (Ps > 1) ts[1] = x; for (int i = 2; i < Ps; ++i) ts[i] = 2.0 * x * ts[i - 1] - ts[i - 2];
        tt[0] = 1.0; if (Pang > 1) tt[1] = y; for (int i = 2; i < Pang; ++i) tt[i] = 2.0 * y * tt[i - 1] - tt[i - 2];
        cd r = 0.0;
        for (int a = 0; a < Pang; ++a) for (int s = 0; s < Ps; ++s) r += (tt[a] * ts[s]) * c[a * Ps + s];
        return r;
    }
    // Interpolator.h:81-120
    void generate(cd* arr) const {
        std::vector<cd> C(P);
        for (int m = 0; m < Ps; ++m) for (int n = 0; n < Pang; ++n) {
            cd s = 0.0;
            for (int k = 0; k < Ps; ++k) for (int l = 0; l < Pang; ++l) s += arr[l * Ps + k] * Ts[m][k] * Tang[n][l];
            C[m * Pang + n] = s;
        }
        for (int m = 0; m < Ps; ++m) for (int n = 0; n < Pang; ++n) {
            const double an = n == 0 ? 1.0 : 2.0, am = m == 0 ? 1.0 : 2.0;
            arr[n * Ps + m] = C[m * Pang + n] * (am * an / (Ps * Pang));
        }
    }
};

struct Level {
    int level, nlevels;
    double min_x, min_y, boxsize;
    long long nside;
    std::vector<long long> rel2box, rel2nonrel;
    double scaling_r2s = 0;
    long long ntheta = 0;
    std::vector<double> radial;
    std::unordered_set<long long> relboxes;
    std::unordered_map<long long, std::array<long long, 2>> box2pts;
    std::unordered_map<long long, std::unordered_map<long long, long long>> boxnonrel2rel;
    std::unordered_map<long long, std::array<std::unordered_map<long long, std::vector<int>>, 4>> protobox;

    Level(int l, int nl, double mx, double my, double bs, double k)
        : level(l), nlevels(nl), min_x(mx), min_y(my), boxsize(bs), nside(1LL << l) { init_cones(k); }

    // Level.h:88-142 (Helmholtz strategy)
    void init_cones(double k) {
        const double minsize = (3.0 / 2.0 * boxsize) * (1.0 - 1e-10);
        const double maxsize = (std::sqrt(2.0) * boxsize * nside - std::sqrt(2.0) / 2.0 * boxsize) * (1.0 + 1e-10);
        long long scal = 1;
        if (level > 1) scal = std::max<long long>(1, (long long)std::ceil(k * boxsize * (1.0 / PI) * 1.2));
        ntheta = scal * 2;
        const long long nrad_level = scal * 1;
        scaling_r2s = std::sqrt(2.0) / 2.0 * boxsize;
        const double eta = std::sqrt(2.0) / 3.0 - 1e-5;
        const double tmpr = (maxsize - minsize + 1e-10);
        const double tmps = std::min(eta / nrad_level, scaling_r2s * (1.0 / minsize - 1.0 / (minsize + tmpr)));
        const long long nact = (long long)std::ceil(scaling_r2s * (1.0 / minsize - 1.0 / maxsize) / tmps);
        radial.assign(nact + 1, 0.0);
        radial[0] = minsize;
        const double fin = scaling_r2s * (1.0 / minsize - 1.0 / maxsize) / nact;
        for (long long i = nact - 1; i >= 0; --i) {
            const long long it = nact - i;
            radial[it] = scaling_r2s * maxsize / (scaling_r2s + maxsize * i * fin);
        }
    }
    static long long Box2Morton(long long x, long long y, int level) {
        return (long long)(splitBy2((unsigned)x, level) | (splitBy2((unsigned)y, level) << 1));
    }
    long long Box2Morton(long long x, long long y) const { return Box2Morton(x, y, level); }
    static long long Point2Morton(double x, double y, double mx, double my, double bs, int level) {
        const long long px = (long long)((x - mx) / bs), py = (long long)((y - my) / bs);
        if (px < 0 || py < 0 || px >= (1LL << level) || py >= (1LL << level))
            throw std::logic_error("The 2D box index cannot be < 0 or larger than the number of boxes");
        return Box2Morton(px, py, level);
    }
    long long Point2Morton(double x, double y) const { return Point2Morton(x, y, min_x, min_y, boxsize, level); }
    void Morton2Box(long long m, long long& x, long long& y) const { x = mergeFrom2((uint64_t)m); y = mergeFrom2((uint64_t)m >> 1); }
    bool IsRelevant(long long m) const { return relboxes.count(m) > 0; }
    static long long even(long long x) { return (x / 2) * 2; }
    // Level.h:261-289
    std::vector<long long> GetCousins(long long m) const {
        std::vector<long long> c; long long x, y; Morton2Box(m, x, y);
        const long long xlo = std::max<long long>(even(x) - 2, 0), xup = std::min<long long>(nside - 1, even(x) + 3);
        const long long ylo = std::max<long long>(even(y) - 2, 0), yup = std::min<long long>(nside - 1, even(y) + 3);
        for (long long j = ylo; j <= yup; ++j) for (long long i = xlo; i <= xup; ++i)
            if (std::llabs(i - x) > 1 || std::llabs(j - y) > 1) {
                const long long cm = Box2Morton(i, j); if (IsRelevant(cm)) c.push_back(cm);
            }
        std::sort(c.begin(), c.end());
        return c;
    }
    // Level.h:378-404
    std::vector<long long> GetNeighbours(long long m) const {
        std::vector<long long> nb; long long x, y; Morton2Box(m, x, y);
        const long long xlo = std::max<long long>(0, x - 1), xup = std::min<long long>(nside - 1, x + 1);
        const long long ylo = std::max<long long>(0, y - 1), yup = std::min<long long>(nside - 1, y + 1);
        for (long long j = ylo; j <= yup; ++j) for (long long i = xlo; i <= xup; ++i) {
            const long long nm = Box2Morton(i, j); if (IsRelevant(nm)) nb.push_back(nm);
        }
        std::sort(nb.begin(), nb.end());
        return nb;
    }
    void GetBoxCenter(long long m, double& x, double& y) const {
        long long px, py; Morton2Box(m, px, py);
        x = min_x + px * boxsize + 0.5 * boxsize; y = min_y + py * boxsize + 0.5 * boxsize;
    }
    long long nrad() const { return (long long)radial.size() - 1; }
    long long twod2nonrel(long long r, long long th) const { return th * nrad() + r; }
    long long radial_pos(double r) const {
        return (long long)(std::upper_bound(radial.begin(), radial.end(), r) - radial.begin()) - 1;
    }
    // Level.h:310-323
    long long Cart2Nonrelcone(long long m, double x, double y) const {
        double cx, cy; GetBoxCenter(m, cx, cy); x -= cx; y -= cy; CartToPol(x, y);
        const long long pr = radial_pos(x);
        const long long pt = (long long)(y * ntheta / PI);
        return twod2nonrel(pr, pt);
    }
    // Level.h:347-356
    double ChebPosr2Radius(long long pr, double r) const {
        const double mn = radial[pr];
        const double rmin = scaling_r2s / radial[pr + 1];
        const double dr = scaling_r2s / mn - rmin;
        return scaling_r2s / ((r + 1.0) / 2.0 * dr + rmin);
    }
    double Cheb2Radius(long long nonrel, double r) const { return ChebPosr2Radius(nonrel % nrad(), r); }
    // Level.h:358-375
    void Cheb2Cart(long long m, long long nonrel, double& x, double& y) const {
        const long long pr = nonrel % nrad(), pt = nonrel / nrad();
        const double da = PI / ntheta;
        x = ChebPosr2Radius(pr, x);
        y = (y + 1.0) / 2.0 * da + da * pt;
        double cx, cy; GetBoxCenter(m, cx, cy);
        PolToCart(x, y); x += cx; y += cy;
    }
    // Level.h:413-422
    double PolRadius2ChebRadius(long long pr, double r) const {
        const double mn = radial[pr];
        const double rmin = scaling_r2s / radial[pr + 1];
        const double dr = scaling_r2s / mn - rmin;
        return (scaling_r2s / r - rmin) / dr * 2.0 - 1.0;
    }
    // Level.h:424-437
    void Cart2Cheb(long long m, long long nonrel, double& x, double& y) const {
        double cx, cy; GetBoxCenter(m, cx, cy); x -= cx; y -= cy; CartToPol(x, y);
        const long long pr = nonrel % nrad(), pt = nonrel / nrad();
        const double da = PI / ntheta;
        x = PolRadius2ChebRadius(pr, x);
        y = (y - da * pt) / da * 2.0 - 1.0;
    }
    // Level.h:439-453
    void Cart2Cheb(long long m, double& x, double& y, long long& nonrel) const {
        double cx, cy; GetBoxCenter(m, cx, cy); x -= cx; y -= cy; CartToPol(x, y);
        const long long pr = radial_pos(x);
        const long long pt = (long long)(y * ntheta / PI);
        nonrel = twod2nonrel(pr, pt);
        const double da = PI / ntheta;
        x = PolRadius2ChebRadius(pr, x);
        y = (y - da * pt) / da * 2.0 - 1.0;
    }
};

struct WorkCounts { long long near_pairs = 0, leaf_evals = 0, prop_evals = 0, interp_evals = 0, cones = 0, cone_levels = 0; };

struct BoxTree {
    std::vector<double> x, y, nx, ny;
    int form = FORM_SINGLE_LAYER;
    double eta = 0.0;
    std::vector<long long> sorting, inverse;
    int nlevels = 0;
    double k = 0.0;
    long long N = 0;
    Interp2D ip;
    std::vector<std::unique_ptr<Level>> levels;
    std::vector<cd> solution, cur, prev;
    WorkCounts wc;

    BoxTree(int Ps, int Pang) : ip(Ps, Pang) {}

    // BoxTree.h:995-1008
    void Reinitialize(const std::vector<double>& xx, const std::vector<double>& yy, const std::vector<double>& nxx,
                      const std::vector<double>& nyy, int nl, double kk, int form_, double eta_) {
        x = xx; y = yy; nx = nxx; ny = nyy; N = (long long)x.size(); nlevels = nl; k = kk; form = form_; eta = eta_;
        inverse.assign(N, 0); sorting.clear(); levels.clear();
        InitializeBoxesAndLevels();
        InitializeRelevantConeSegments();
        solution.assign(N, 0.0);
        long long mx = 0;
        for (int l = 2; l < nlevels; ++l) mx = std::max<long long>(mx, (long long)levels[l]->rel2nonrel.size());
        cur.assign(mx * ip.P, 0.0); prev.assign(mx * ip.P, 0.0);
        count_work();
    }

    // BoxTree.h:205-231 with ComputeBB (:179-202), SortBox (:73-106) and the level-D data (:111-174)
    void InitializeBoxesAndLevels() {
        double mn[2] = {1e308, 1e308}, mxv[2] = {-1e308, -1e308};
        for (long long i = 0; i < N; ++i) {
            mn[0] = std::min(mn[0], x[i]); mn[1] = std::min(mn[1], y[i]);
            mxv[0] = std::max(mxv[0], x[i]); mxv[1] = std::max(mxv[1], y[i]);
        }
        mxv[0] += 1e-10; mxv[1] += 1e-10; mn[0] -= 1e-10; mn[1] -= 1e-10;
        const double boxsize = std::max(mxv[0] - mn[0], mxv[1] - mn[1]);
        // SortBox: stable sort of point indices by leaf Morton code
        std::vector<long long> code(N);
        for (long long i = 0; i < N; ++i)
            code[i] = Level::Point2Morton(x[i], y[i], mn[0], mn[1], boxsize / (1 << (nlevels - 1)), nlevels - 1);
        sorting.resize(N);
        for (long long i = 0; i < N; ++i) sorting[i] = i;
        std::stable_sort(sorting.begin(), sorting.end(), [&](long long a, long long b) { return code[a] < code[b]; });
        std::vector<double> tx(N), ty(N), tnx(N), tny(N);
        for (long long i = 0; i < N; ++i) { tx[i] = x[sorting[i]]; ty[i] = y[sorting[i]]; tnx[i] = nx[sorting[i]]; tny[i] = ny[sorting[i]]; }
        x = tx; y = ty; nx = tnx; ny = tny;
        for (long long i = 0; i < N; ++i) inverse[sorting[i]] = i;
        levels.resize(nlevels);
        for (int i = 1; i < nlevels; ++i)
            levels[i].reset(new Level(i, nlevels, mn[0], mn[1], boxsize / (1 << i), k));
        Level& D = *levels.back();
        long long old = -1, np = -1;
        for (long long i = 0; i < N; ++i) {
            const long long m = D.Point2Morton(x[i], y[i]);
            if (m != old) {
                if (i != 0) D.box2pts[old] = {i - np, np};
                old = m; np = 1; D.relboxes.insert(m);
            } else np++;
        }
        D.box2pts[old] = {N - np, np};
        std::unordered_set<long long> rel = D.relboxes, par;
        for (int i = nlevels - 1; i >= 2; --i) {
            if (i != nlevels - 1) levels[i]->relboxes.insert(rel.begin(), rel.end());
            for (long long m : rel) par.insert(m / 4);
            std::swap(rel, par); par.clear();
        }
    }

    std::vector<long long> RelChildren(int level, long long m) const {
        std::vector<long long> ch;
        if (level >= nlevels - 1) return ch;
        for (long long c = m * 4; c < (m + 1) * 4; ++c) if (levels[level + 1]->IsRelevant(c)) ch.push_back(c);
        return ch;
    }

    // BoxTree.h:235-277
    void ConesDueToCousins(int level, std::unordered_map<long long, std::vector<long long>>& out) const {
        std::unordered_map<long long, std::unordered_set<long long>> tmp;
        long long old = -1; std::vector<long long> cous;
        const Level& L = *levels[level];
        for (long long i = 0; i < N; ++i) {
            const long long m = L.Point2Morton(x[i], y[i]);
            if (m != old) { cous = L.GetCousins(m); old = m; }
            for (long long c : cous) tmp[c].insert(L.Cart2Nonrelcone(c, x[i], y[i]));
        }
        for (auto& kv : tmp) { std::vector<long long> v(kv.second.begin(), kv.second.end()); std::sort(v.begin(), v.end()); out[kv.first] = v; }
    }

    // BoxTree.h:299-428 (builds the protobox routing table of level `level`)
    void ConesDueToParents(int level, std::unordered_map<long long, std::vector<long long>>& out) {
        Level& Lp = *levels[level - 1];
        Level& Lc = *levels[level];
        long long old = -1; std::vector<long long> ch;
        for (size_t rc = 0; rc < Lp.rel2nonrel.size(); ++rc) {
            const long long box = Lp.rel2box[rc], nonrel = Lp.rel2nonrel[rc];
            if (box != old) {
                ch = RelChildren(level - 1, box);
                if (ch.empty()) throw std::logic_error("Every cocentered morton box must have children");
                old = box;
            }
            auto& entry = Lc.protobox[nonrel];
            for (long long c : ch) {
                const long long pos = c % 4;
                if (!entry[pos].empty()) continue;
                for (int it = 0; it < ip.P; ++it) {
                    double px, py; ip.point(it, px, py);
                    Lp.Cheb2Cart(box, nonrel, px, py);
                    entry[pos][Lc.Cart2Nonrelcone(c, px, py)].push_back(it);
                }
            }
        }
        std::unordered_map<long long, std::unordered_set<long long>> all;
        old = -1;
        for (size_t rc = 0; rc < Lp.rel2nonrel.size(); ++rc) {
            const long long box = Lp.rel2box[rc], nonrel = Lp.rel2nonrel[rc];
            if (box != old) { ch = RelChildren(level - 1, box); old = box; }
            for (long long c : ch)
                for (auto& kv : Lc.protobox.at(nonrel)[c % 4]) all[c].insert(kv.first);
        }
        for (auto& kv : all) { std::vector<long long> v(kv.second.begin(), kv.second.end()); std::sort(v.begin(), v.end()); out[kv.first] = v; }
    }

    // BoxTree.h:430-514, 553-583 (merged cone lists; relevant cones numbered box by box)
    void InitializeRelevantConeSegments() {
        for (int level = 2; level < nlevels; ++level) {
            std::unordered_map<long long, std::vector<long long>> a, b;
            ConesDueToCousins(level, a);
            if (level > 2) ConesDueToParents(level, b);
            if (a.empty() && b.empty()) throw std::logic_error("The number of cone segments on any level cannot be 0");
            std::map<long long, std::set<long long>> merged;
            for (auto& kv : a) merged[kv.first].insert(kv.second.begin(), kv.second.end());
            for (auto& kv : b) merged[kv.first].insert(kv.second.begin(), kv.second.end());
            Level& L = *levels[level];
            L.rel2box.clear(); L.rel2nonrel.clear(); L.boxnonrel2rel.clear();
            for (auto& kv : merged) for (long long c : kv.second) {
                L.boxnonrel2rel[kv.first][c] = (long long)L.rel2box.size();
                L.rel2box.push_back(kv.first); L.rel2nonrel.push_back(c);
            }
        }
    }

    // BoxTree.h:614-683
    void SingularInteractions(const std::vector<cd>& dens, const std::vector<std::unordered_set<long long>>* excl) {
        const Level& D = *levels.back();
        long long old = -1; std::vector<long long> nb;
        for (long long i = 0; i < N; ++i) {
            const long long m = D.Point2Morton(x[i], y[i]);
            cd res = solution[i];
            if (m != old) { nb = D.GetNeighbours(m); if (nb.size() > 9) throw std::logic_error("Cannot have more than 9 neighbours."); old = m; }
            for (long long b : nb) {
                const auto& pd = D.box2pts.at(b);
                for (long long s = 0; s < pd[1]; ++s) {
                    const long long j = pd[0] + s;
                    if (j == i) continue;
                    if (excl && (*excl)[i].count(j)) continue;
                    res += GF_form(form, x[i], y[i], x[j], y[j], nx[j], ny[j], k, eta) * dens[j];
                }
            }
            solution[i] = res;
        }
    }

    // BoxTree.h:685-762
    void LevelDEvaluations(const std::vector<cd>& dens) {
        const Level& D = *levels.back();
        for (size_t i = 0; i < D.rel2nonrel.size(); ++i) {
            const long long box = D.rel2box[i], nonrel = D.rel2nonrel[i];
            const auto& pd = D.box2pts.at(box);
            cd* co = &prev[i * ip.P];
            for (int j = 0; j < ip.P; ++j) {
                double px, py; ip.point(j, px, py);
                const double rad = D.Cheb2Radius(nonrel, px);
                D.Cheb2Cart(box, nonrel, px, py);
                cd res = 0.0;
                for (long long s = 0; s < pd[1]; ++s) {
                    const long long j = pd[0] + s;
                    res += GF_form(form, px, py, x[j], y[j], nx[j], ny[j], k, eta) * dens[j];
                }
                co[j] = res / factorization(rad, k);
            }
            ip.generate(co);
        }
        cur = prev;
    }

    // BoxTree.h:767-868
    void Propagation(int level) {
        const Level& Lp = *levels[level - 1];
        const Level& Lc = *levels[level];
        std::vector<double> X(ip.P), Y(ip.P), R(ip.P);
        std::vector<cd> val(ip.P);
        long long old = -1; std::vector<long long> ch;
        for (size_t rc = 0; rc < Lp.rel2nonrel.size(); ++rc) {
            const long long box = Lp.rel2box[rc], nonrel = Lp.rel2nonrel[rc];
            if (box != old) { ch = RelChildren(level - 1, box); old = box; }
            const auto& proto = Lc.protobox.at(nonrel);
            for (int it = 0; it < ip.P; ++it) {
                ip.point(it, X[it], Y[it]);
                R[it] = Lp.Cheb2Radius(nonrel, X[it]);
                Lp.Cheb2Cart(box, nonrel, X[it], Y[it]);
                val[it] = 0.0;
            }
            for (long long c : ch) {
                const auto& cones = proto.at(c % 4);
                for (auto& kv : cones) {
                    const long long crel = Lc.boxnonrel2rel.at(c).at(kv.first);
                    const cd* cc = &prev[crel * ip.P];
                    for (int it : kv.second) {
                        double lx = X[it], ly = Y[it];
                        Lc.Cart2Cheb(c, kv.first, lx, ly);
                        const double lr = Lc.Cheb2Radius(kv.first, lx);
                        val[it] += ip.interpolate(lx, ly, cc) * factorization(lr, k);
                    }
                }
            }
            cd* co = &cur[rc * ip.P];
            for (int it = 0; it < ip.P; ++it) co[it] = val[it] / factorization(R[it], k);
            ip.generate(co);
        }
    }

    // BoxTree.h:876-937
    void Interpolation(int level) {
        const Level& L = *levels[level];
        long long old = -1; std::vector<long long> cous;
        for (long long i = 0; i < N; ++i) {
            cd v = solution[i];
            const long long m = L.Point2Morton(x[i], y[i]);
            if (m != old) { cous = L.GetCousins(m); old = m; }
            for (long long c : cous) {
                double lx = x[i], ly = y[i]; long long nonrel;
                L.Cart2Cheb(c, lx, ly, nonrel);
                const long long rel = L.boxnonrel2rel.at(c).at(nonrel);
                const double r = L.Cheb2Radius(nonrel, lx);
                v += ip.interpolate(lx, ly, &prev[rel * ip.P]) * factorization(r, k);
            }
            solution[i] = v;
        }
    }

    // BoxTree.h:1020-1071; density in original order, replaced by the result
    void Solve(std::vector<cd>& density, const std::vector<std::unordered_set<long long>>* excl) {
        if (nlevels < 3) throw std::invalid_argument("IFGF accelerator requires at least 3 levels.");
        std::fill(solution.begin(), solution.end(), cd(0.0, 0.0));
        std::vector<cd> d(N);
        for (long long i = 0; i < N; ++i) d[i] = density[sorting[i]];
        SingularInteractions(d, excl);
        LevelDEvaluations(d);
        for (int level = nlevels - 1; level >= 2; --level) {
            if (level > 2) Propagation(level);
            Interpolation(level);
            std::swap(cur, prev);
        }
        for (long long i = 0; i < N; ++i) density[sorting[i]] = solution[i];
    }

    // BoxTree.h:1079-1161 (throws when a singular / near-singular point is not a leaf neighbour)
    void CheckIfSingandNearSingInNeighborhood(const std::vector<double>& xr, const std::vector<double>& yr,
                                              const std::vector<Patch>& patches, int Np) const {
        const Level& D = *levels.back();
        auto inhood = [&](double xt, double yt, const std::vector<long long>& nb) {
            const long long m = D.Point2Morton(xt, yt);
            return std::find(nb.begin(), nb.end(), m) != nb.end();
        };
        for (long long i = 0; i < N; ++i) {
            const long long pi = i / Np;
            std::vector<long long> nb = D.GetNeighbours(D.Point2Morton(xr[i], yr[i]));
            for (long long j = pi * Np; j < pi * Np + Np; ++j)
                if (j != i && !inhood(xr[j], yr[j], nb)) throw std::logic_error("Singular point not in neighborhood");
        }
        for (size_t pi = 0; pi < patches.size(); ++pi)
            for (long long ns : patches[pi].ns_idx) {
                std::vector<long long> nb = D.GetNeighbours(D.Point2Morton(xr[ns], yr[ns]));
                for (long long j = (long long)pi * Np; j < (long long)pi * Np + Np; ++j)
                    if (!inhood(xr[j], yr[j], nb)) throw std::logic_error("Near singular point not in neighborhood");
            }
    }

    // algorithmic work of one Solve (not in the reference; used for the roofline figures)
    void count_work() {
        wc = WorkCounts();
        const Level& D = *levels.back();
        for (auto& kv : D.box2pts) {
            long long nsrc = 0;
            for (long long b : D.GetNeighbours(kv.first)) nsrc += D.box2pts.at(b)[1];
            wc.near_pairs += kv.second[1] * nsrc;
        }
        for (size_t i = 0; i < D.rel2box.size(); ++i) wc.leaf_evals += (long long)ip.P * D.box2pts.at(D.rel2box[i])[1];
        for (int l = 2; l < nlevels; ++l) {
            const Level& L = *levels[l];
            wc.cones += (long long)L.rel2box.size();
            long long old = -1, nc = 0;
            for (long long i = 0; i < N; ++i) {
                const long long m = L.Point2Morton(x[i], y[i]);
                if (m != old) { nc = (long long)L.GetCousins(m).size(); old = m; }
                wc.interp_evals += nc;
            }
            if (l > 2) {
                const Level& Lp = *levels[l - 1];
                for (size_t rc = 0; rc < Lp.rel2box.size(); ++rc)
                    wc.prop_evals += (long long)ip.P * (long long)RelChildren(l - 1, Lp.rel2box[rc]).size();
            }
        }
        wc.cone_levels = nlevels - 2;
    }
};

}  // namespace orc
