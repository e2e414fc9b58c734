// tree.cpp -- host build of the flattened IFGF tree (see tree.hpp).
#include "tree.hpp"
#include <algorithm>
#include <cmath>
#include <numeric>
#include <unordered_map>
#include <array>
#include "host_threads.hpp"

namespace ifgf {

static constexpr double kPiT = 3.14159265358979323846;

// ---------------------------------------------------------------- Morton codes (Level.h:172-245)
static inline uint64_t spread_bits(uint64_t x) {
    x &= 0xFFFFFFFFull;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}
static inline uint64_t gather_bits(uint64_t x) {
    x &= 0x5555555555555555ull;
    x = (x ^ (x >> 1)) & 0x3333333333333333ull;
    x = (x ^ (x >> 2)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x ^ (x >> 4)) & 0x00FF00FF00FF00FFull;
    x = (x ^ (x >> 8)) & 0x0000FFFF0000FFFFull;
    x = (x ^ (x >> 16)) & 0xFFFFFFFFull;
    return x;
}
static inline long long morton_of(long long bx, long long by) { return (long long)(spread_bits((uint64_t)bx) | (spread_bits((uint64_t)by) << 1)); }
static inline void box_of(long long m, long long& bx, long long& by) { bx = (long long)gather_bits((uint64_t)m); by = (long long)gather_bits((uint64_t)m >> 1); }

long long point_morton(double x, double y, double min_x, double min_y, double boxsize, int level) {
    const long long px = (long long)((x - min_x) / boxsize), py = (long long)((y - min_y) / boxsize);
    if (px < 0 || py < 0 || px >= (1LL << level) || py >= (1LL << level)) return -1;
    return morton_of(px, py);
}

void tree_root_box(const std::vector<double>& x, const std::vector<double>& y, double& min_x, double& min_y, double& size) {
    double x0 = 1e308, y0 = 1e308, x1 = -1e308, y1 = -1e308;
    for (size_t i = 0; i < x.size(); ++i) { x0 = std::min(x0, x[i]); y0 = std::min(y0, y[i]); x1 = std::max(x1, x[i]); y1 = std::max(y1, y[i]); }
    x1 += 1e-10; y1 += 1e-10; x0 -= 1e-10; y0 -= 1e-10;   // BoxTree.h:196-200
    min_x = x0; min_y = y0; size = std::max(x1 - x0, y1 - y0);
}

int TreeLevel::find_box(long long m) const {
    auto it = std::lower_bound(boxes.begin(), boxes.end(), m);
    return (it != boxes.end() && *it == m) ? (int)(it - boxes.begin()) : -1;
}
int TreeLevel::find_cone(int b, long long nonrel) const {
    auto first = cone_nonrel.begin() + cone_ptr[b], last = cone_nonrel.begin() + cone_ptr[b + 1];
    auto it = std::lower_bound(first, last, nonrel);
    return (it != last && *it == nonrel) ? (int)(it - cone_nonrel.begin()) : -1;
}

// ---------------------------------------------------------------- host threads
namespace {
void sort_unique(std::vector<unsigned long long>& v) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
}
// union of sorted, duplicate-free lists: pairwise merges, in parallel per round
std::vector<unsigned long long> merge_unique(std::vector<std::vector<unsigned long long>>& parts) {
    if (parts.empty()) return {};
    while (parts.size() > 1) {
        const long long np = (long long)(parts.size() + 1) / 2;
        std::vector<std::vector<unsigned long long>> next(np);
        parallel_for(np, [&](long long q0, long long q1) {
            for (long long q = q0; q < q1; ++q) {
                if (2 * q + 1 >= (long long)parts.size()) { next[q].swap(parts[2 * q]); continue; }
                auto& a = parts[2 * q];
                auto& b = parts[2 * q + 1];
                next[q].resize(a.size() + b.size());
                auto e = std::set_union(a.begin(), a.end(), b.begin(), b.end(), next[q].begin());
                next[q].resize(e - next[q].begin());
                std::vector<unsigned long long>().swap(a);
                std::vector<unsigned long long>().swap(b);
            }
        }, 1);
        parts.swap(next);
    }
    return std::move(parts[0]);
}
}  // namespace

// ---------------------------------------------------------------- per-level geometry
namespace {
struct LevelGeo {
    const TreeLevel* L; double min_x, min_y;
    void center(long long m, double& cx, double& cy) const {   // Level.h:291-298
        long long bx, by; box_of(m, bx, by);
        cx = min_x + bx * L->boxsize + 0.5 * L->boxsize;
        cy = min_y + by * L->boxsize + 0.5 * L->boxsize;
    }
    static double atan_0_2pi(double y, double x) {             // PolarCoordinates.h:8-27
        if (x > 0 && y >= 0) return std::atan(y / x);
        if (x > 0 && y < 0) return std::atan(y / x) + 2.0 * kPiT;
        if (x < 0 && y > 0) return std::atan(y / x) + kPiT;
        if (x < 0 && y == 0) return kPiT;
        if (x < 0 && y < 0) return std::atan(y / x) + kPiT;
        if (x == 0 && y > 0) return kPiT / 2;
        if (x == 0 && y < 0) return 3.0 * kPiT / 2;
        return 0;
    }
    static void to_polar(double& x, double& y) {
        const double r = std::sqrt(x * x + y * y);
        if (r == 0.0) { x = 0.0; y = 0.0; return; }
        const double th = atan_0_2pi(y, x);
        x = r; y = th;
    }
    long long rpos(double r) const {
        return (long long)(std::upper_bound(L->radial.begin(), L->radial.end(), r) - L->radial.begin()) - 1;
    }
    // rpos(r) from a guess h: the interval [radial[h], radial[h + 1]) that holds r is the one
    // upper_bound finds, so a right guess gives the same index without the search
    long long rpos(double r, long long h) const {
        const double* R = L->radial.data();
        if (h >= 0 && h + 1 < (long long)L->radial.size() && R[h] <= r && r < R[h + 1]) return h;
        return rpos(r);
    }
    long long nonrel_of(long long m, double x, double y) const {   // Level.h:310-323
        double cx, cy; center(m, cx, cy); x -= cx; y -= cy; to_polar(x, y);
        return (long long)(y * L->ntheta / kPiT) * L->nrad + rpos(x);
    }
    // nonrel_of with a guess of the radial interval, updated to the one found
    long long nonrel_of(long long m, double x, double y, long long& h) const {
        double cx, cy; center(m, cx, cy); x -= cx; y -= cy; to_polar(x, y);
        h = rpos(x, h);
        return (long long)(y * L->ntheta / kPiT) * L->nrad + h;
    }
    double cheb_to_radius(long long pr, double s) const {          // Level.h:347-356
        const double rmin = L->scaling_r2s / L->radial[pr + 1];
        const double dr = L->scaling_r2s / L->radial[pr] - rmin;
        return L->scaling_r2s / ((s + 1.0) / 2.0 * dr + rmin);
    }
    double radius_to_cheb(long long pr, double r) const {          // Level.h:413-422
        const double rmin = L->scaling_r2s / L->radial[pr + 1];
        const double dr = L->scaling_r2s / L->radial[pr] - rmin;
        return (L->scaling_r2s / r - rmin) / dr * 2.0 - 1.0;
    }
    void cheb_to_cart(long long m, long long nonrel, double& x, double& y) const {   // Level.h:358-375
        const long long pr = nonrel % L->nrad, pt = nonrel / L->nrad;
        const double da = kPiT / L->ntheta;
        const double r = cheb_to_radius(pr, x);
        const double th = (y + 1.0) / 2.0 * da + da * pt;
        double cx, cy; center(m, cx, cy);
        x = r * std::cos(th) + cx; y = r * std::sin(th) + cy;
    }
    void cart_to_cheb(long long m, long long nonrel, double& x, double& y) const {   // Level.h:424-437
        double cx, cy; center(m, cx, cy); x -= cx; y -= cy; to_polar(x, y);
        const long long pr = nonrel % L->nrad, pt = nonrel / L->nrad;
        const double da = kPiT / L->ntheta;
        x = radius_to_cheb(pr, x);
        y = (y - da * pt) / da * 2.0 - 1.0;
    }
    long long cart_to_cheb_cone(long long m, double& x, double& y) const {
        long long h = -1;
        return cart_to_cheb_cone(m, x, y, h);
    }
    // with a guess of the radial interval, updated to the one found
    long long cart_to_cheb_cone(long long m, double& x, double& y, long long& h) const {   // Level.h:439-453
        double cx, cy; center(m, cx, cy); x -= cx; y -= cy; to_polar(x, y);
        const long long pr = h = rpos(x, h), pt = (long long)(y * L->ntheta / kPiT);
        const double da = kPiT / L->ntheta;
        x = radius_to_cheb(pr, x);
        y = (y - da * pt) / da * 2.0 - 1.0;
        return pt * L->nrad + pr;
    }
};

// Level.h:88-142 (Helmholtz cone refinement).  The cone segments cover box-centre distances
// from 1.5 box sizes to the farthest point of the root box; `reach` (> 0 for off-surface
// targets) extends the outer radius to cover targets outside it.
void init_cones(TreeLevel& L, double k, double reach = 0.0) {
    const double minsize = (3.0 / 2.0 * L.boxsize) * (1.0 - 1e-10);
    const double maxsize = std::max(reach, (std::sqrt(2.0) * L.boxsize * L.nside - std::sqrt(2.0) / 2.0 * L.boxsize) * (1.0 + 1e-10));
    long long scal = 1;
    if (L.level > 1) scal = std::max<long long>(1, (long long)std::ceil(k * L.boxsize * (1.0 / kPiT) * 1.2));
    L.ntheta = 2 * scal;
    L.scaling_r2s = std::sqrt(2.0) / 2.0 * L.boxsize;
    const double eta = std::sqrt(2.0) / 3.0 - 1e-5;
    const double span = maxsize - minsize + 1e-10;
    const double ds = std::min(eta / scal, L.scaling_r2s * (1.0 / minsize - 1.0 / (minsize + span)));
    const long long n = (long long)std::ceil(L.scaling_r2s * (1.0 / minsize - 1.0 / maxsize) / ds);
    L.radial.assign(n + 1, 0.0);
    L.radial[0] = minsize;
    const double step = L.scaling_r2s * (1.0 / minsize - 1.0 / maxsize) / n;
    for (long long i = n - 1; i >= 0; --i) L.radial[n - i] = L.scaling_r2s * maxsize / (L.scaling_r2s + maxsize * i * step);
    L.nrad = n;
}

// relevant boxes of `L` within the even-aligned 6x6 block around m, minus the 3x3 (Level.h:261-289)
void cousins_of(const TreeLevel& L, long long m, std::vector<int>& out) {
    out.clear();
    long long bx, by; box_of(m, bx, by);
    const long long ex = (bx / 2) * 2, ey = (by / 2) * 2;
    const long long x0 = std::max<long long>(ex - 2, 0), x1 = std::min<long long>(L.nside - 1, ex + 3);
    const long long y0 = std::max<long long>(ey - 2, 0), y1 = std::min<long long>(L.nside - 1, ey + 3);
    std::vector<std::pair<long long, int>> tmp;
    for (long long j = y0; j <= y1; ++j)
        for (long long i = x0; i <= x1; ++i)
            if (std::llabs(i - bx) > 1 || std::llabs(j - by) > 1) {
                const long long cm = morton_of(i, j);
                const int b = L.find_box(cm);
                if (b >= 0) tmp.push_back({cm, b});
            }
    std::sort(tmp.begin(), tmp.end());
    for (auto& t : tmp) out.push_back(t.second);
}
}  // namespace

// Cones of level l and the propagation plan of its parents.  `part` holds the wanted cones
// (box index << 32 | nonrel cone, each list sorted and unique) that the targets see; the cones
// needed by the parents' interpolation nodes are added here through the protobox routing table
// (BoxTree.h:299-428).  Fills T.L[l]'s cone lists and, for l > 2, appends the level's slot form
// of the propagation plan (PropSlots, entries in global parent-id order) and its CSR rows to
// T.pp_ptr / pp_nchild.  `seen` is the caller's scratch table, all -1 on entry and on return: it
// grows to the largest level's need once instead of being allocated and filled per level.
std::string finish_level(Tree& T, int l, std::vector<std::vector<unsigned long long>>& part, const std::vector<double>& ns,
                         const std::vector<double>& na, std::vector<int, NoInitAlloc<int>>& seen) {
    TreeLevel& L = T.L[l];
    LevelGeo G{&L, T.min_x, T.min_y};
    const int P = T.P, Ps = T.Ps;
    auto key = [](long long b, long long nonrel) { return ((unsigned long long)b << 32) | (unsigned long long)nonrel; };
    // cones needed by the parents' interpolation nodes, through the protobox routing
    // table (BoxTree.h:299-428): for each parent nonrel cone and child position, the
    // routing is computed once, from the first parent box (in cone order) that has it.
    // per route: its child cone segment for each of the P parent nodes at rn[r * P ...], and its
    // nu[r] distinct segments, ascending, at uq[r * P ...]
    struct Route { long long pnc; int pos; int first_pc; };
    std::vector<Route> routes;
    std::vector<int, NoInitAlloc<int>> rn, uq;   // cone segments fit an int (ntheta * nrad per box)
    std::vector<int> nu;
    std::vector<int> route_of;          // per (parent cone * 4 + pos): route index or -1
    std::vector<int> child_box;         // per (parent box * 4 + pos): child box index or -1
    const TreeLevel* Lpp = l > 2 ? &T.L[l - 1] : nullptr;
    if (Lpp) {
        const TreeLevel& Lp = *Lpp;
        LevelGeo Gp{&Lp, T.min_x, T.min_y};
        const size_t npar = Lp.cone_nonrel.size();
        // the children of each parent box: the child level's boxes are sorted, so a parent's
        // children follow one another
        child_box.assign(Lp.boxes.size() * 4, -1);
        parallel_for((long long)L.boxes.size(), [&](long long c0, long long c1) {
            for (long long c = c0; c < c1; ++c) {
                const int pb = Lp.find_box(L.boxes[c] / 4);
                if (pb >= 0) child_box[(size_t)pb * 4 + (size_t)(L.boxes[c] % 4)] = (int)c;
            }
        });
        route_of.assign(npar * 4, -1);
        // pnc * 4 + pos -> route, over the parent level's cone segment numbers
        long long maxnc = 0;
        for (long long nc : Lp.cone_nonrel) maxnc = std::max(maxnc, nc);
        const size_t need = (size_t)(maxnc + 1) * 4;
        if (seen.size() < need) {   // grown uninitialised, then filled with -1 in parallel
            const size_t old = seen.size();
            seen.resize(need);
            parallel_for((long long)(need - old), [&](long long a, long long b) {
                std::fill(seen.data() + old + a, seen.data() + old + b, -1);
            }, 1 << 16);
        }
        // routes numbered in (first parent cone, position) order, in four parallel passes:
        // (1) per (segment, position) the first parent cone that has it, an atomic minimum in
        // `seen`; (2) per chunk of parent cones, how many routes start there; (3) the routes of
        // each chunk from its offset, each marked in `seen` as -2 - route; (4) per parent cone and
        // position, its route.  Loads and stores of `seen` are atomic (relaxed): pass 3 reads
        // entries that other threads overwrite, and only compares them with its own cone.
        auto has = [&](size_t pc, int pos) { return child_box[(size_t)Lp.cone_box[pc] * 4 + pos] >= 0; };
        auto slot_of = [&](size_t pc, int pos) { return seen.data() + (size_t)(Lp.cone_nonrel[pc] * 4 + pos); };
        parallel_for((long long)npar, [&](long long p0, long long p1) {
            for (long long pc = p0; pc < p1; ++pc)
                for (int pos = 0; pos < 4; ++pos) {
                    if (!has(pc, pos)) continue;
                    int* sp = slot_of(pc, pos);
                    int cur = __atomic_load_n(sp, __ATOMIC_RELAXED);
                    while ((cur < 0 || cur > pc) &&
                           !__atomic_compare_exchange_n(sp, &cur, (int)pc, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                    }
                }
        });
        const long long nrc = std::max<long long>(1, std::min<long long>(8 * kMaxThreads, (long long)npar / 4096));
        std::vector<long long> rbase(nrc + 1, 0);
        auto chunk_range = [&](long long c, size_t& p0, size_t& p1) { p0 = npar * c / nrc; p1 = npar * (c + 1) / nrc; };
        parallel_for(nrc, [&](long long c0, long long c1) {
            for (long long c = c0; c < c1; ++c) {
                size_t p0, p1;
                chunk_range(c, p0, p1);
                long long n = 0;
                for (size_t pc = p0; pc < p1; ++pc)
                    for (int pos = 0; pos < 4; ++pos) n += has(pc, pos) && __atomic_load_n(slot_of(pc, pos), __ATOMIC_RELAXED) == (int)pc;
                rbase[c + 1] = n;
            }
        }, 1);
        for (long long c = 0; c < nrc; ++c) rbase[c + 1] += rbase[c];
        routes.resize((size_t)rbase[nrc]);
        parallel_for(nrc, [&](long long c0, long long c1) {
            for (long long c = c0; c < c1; ++c) {
                size_t p0, p1;
                chunk_range(c, p0, p1);
                long long id = rbase[c];
                for (size_t pc = p0; pc < p1; ++pc)
                    for (int pos = 0; pos < 4; ++pos) {
                        if (!has(pc, pos)) continue;
                        int* sp = slot_of(pc, pos);
                        if (__atomic_load_n(sp, __ATOMIC_RELAXED) != (int)pc) continue;
                        routes[id] = Route{Lp.cone_nonrel[pc], pos, (int)pc};
                        __atomic_store_n(sp, (int)(-2 - id), __ATOMIC_RELAXED);
                        ++id;
                    }
            }
        }, 1);
        parallel_for((long long)npar, [&](long long p0, long long p1) {
            for (long long pc = p0; pc < p1; ++pc)
                for (int pos = 0; pos < 4; ++pos)
                    if (has(pc, pos)) route_of[pc * 4 + pos] = -2 - *slot_of(pc, pos);
        });
        parallel_for((long long)routes.size(), [&](long long r0, long long r1) {
            for (long long r = r0; r < r1; ++r) seen[(size_t)(routes[r].pnc * 4 + routes[r].pos)] = -1;
        });
        rn.resize(routes.size() * P);
        uq.resize(routes.size() * P);
        nu.resize(routes.size());
        parallel_for((long long)routes.size(), [&](long long r0, long long r1) {
            // the parent nodes' radii and angles, once per route (cheb_to_cart's arithmetic)
            std::vector<double> rr(Ps), cs(T.Pang), sn(T.Pang);
            for (long long r = r0; r < r1; ++r) {
                const Route& R = routes[r];
                const long long pm = Lp.boxes[Lp.cone_box[R.first_pc]];
                int* nr = rn.data() + r * P;
                int* u = uq.data() + r * P;
                const long long pr = R.pnc % Lp.nrad, pt = R.pnc / Lp.nrad;
                const double da = kPiT / Lp.ntheta;
                double cx, cy;
                Gp.center(pm, cx, cy);
                for (int i = 0; i < Ps; ++i) rr[i] = Gp.cheb_to_radius(pr, ns[i]);
                for (int j = 0; j < T.Pang; ++j) {
                    const double th = (na[j] + 1.0) / 2.0 * da + da * pt;
                    cs[j] = std::cos(th);
                    sn[j] = std::sin(th);
                }
                long long h = -1;
                for (int it = 0; it < P; ++it) {
                    const double px = rr[it % Ps] * cs[it / Ps] + cx, py = rr[it % Ps] * sn[it / Ps] + cy;
                    nr[it] = (int)G.nonrel_of(pm * 4 + R.pos, px, py, h);
                }
                std::copy(nr, nr + P, u);
                std::sort(u, u + P);
                nu[r] = (int)(std::unique(u, u + P) - u);
            }
        });
        const long long nchunk = std::max<long long>(1, std::min<long long>(4 * kMaxThreads, (long long)npar / 256));
        const size_t base = part.size();
        part.resize(base + nchunk);
        parallel_for(nchunk, [&](long long c0, long long c1) {
            for (long long c = c0; c < c1; ++c) {
                const size_t p0 = npar * c / nchunk, p1 = npar * (c + 1) / nchunk;
                auto& w = part[base + c];
                for (size_t pc = p0; pc < p1; ++pc) {
                    for (int pos = 0; pos < 4; ++pos) {
                        const int r = route_of[pc * 4 + pos];
                        if (r < 0) continue;
                        const int cb = child_box[(size_t)Lp.cone_box[pc] * 4 + pos];
                        for (int j = 0; j < nu[r]; ++j) w.push_back(key(cb, uq[(size_t)r * P + j]));
                    }
                }
                sort_unique(w);
            }
        }, 1);
    }
    // merged cone list, sorted by box, then nonrel cone
    std::vector<unsigned long long> want = merge_unique(part);
    if (want.empty()) return "The number of cone segments on any level cannot be 0";
    L.cone_ptr.assign(L.boxes.size() + 1, 0);
    L.cone_box.resize(want.size()); L.cone_nonrel.resize(want.size());
    for (size_t q = 0; q < want.size(); ++q) {
        const int b = (int)(want[q] >> 32);
        L.cone_box[q] = b; L.cone_nonrel[q] = (long long)(want[q] & 0xFFFFFFFFull); L.cone_ptr[b + 1]++;
    }
    for (size_t b = 0; b < L.boxes.size(); ++b) L.cone_ptr[b + 1] += L.cone_ptr[b];
    L.cone_base = T.total_cones;
    T.total_cones += (int)L.cone_nonrel.size();
    if (!Lpp) return "";
    // propagation plan of this level in slot form: parents are the cones of level l-1, slots in
    // global parent-id order (levels are built upwards, so level l-1's id range is final)
    const TreeLevel& Lp = *Lpp;
    if (T.pp_ptr.empty()) T.pp_ptr.assign(1, 0);
    if ((long long)T.pp_ptr.size() - 1 != Lp.cone_base) return "internal: propagation plan out of order";
    const size_t npar = Lp.cone_nonrel.size();
    PropSlots S;
    S.level = l;
    S.entry_base = T.pp_total;
    S.route_nonrel = std::move(rn);
    long long done = T.pp_ptr.back();
    std::vector<long long> first(npar + 1, 0);   // per parent cone: its first slot
    for (size_t pc = 0; pc < npar; ++pc) {
        int nch = 0;
        for (int pos = 0; pos < 4; ++pos) nch += route_of[pc * 4 + pos] >= 0;
        first[pc + 1] = first[pc] + nch;
        done += (long long)nch * P;
        T.pp_nchild.push_back(nch);
        T.pp_ptr.push_back(done);
        T.prop_evals += (long long)nch * P;
    }
    const size_t nslot = (size_t)first[npar];
    S.slot_parent.resize(nslot); S.slot_child_box.resize(nslot); S.slot_pos.resize(nslot); S.slot_route.resize(nslot);
    parallel_for((long long)npar, [&](long long p0, long long p1) {
        for (long long pc = p0; pc < p1; ++pc) {
            long long q = first[pc];
            for (int pos = 0; pos < 4; ++pos) {
                const int r = route_of[pc * 4 + pos];
                if (r < 0) continue;
                S.slot_parent[q] = (int)pc;
                S.slot_child_box[q] = child_box[(size_t)Lp.cone_box[pc] * 4 + pos];
                S.slot_pos[q] = pos;
                S.slot_route[q] = r;
                ++q;
            }
        }
    }, 4096);
    T.pp_total = done;
    T.prop_slots.push_back(std::move(S));
    return "";
}

// relevant boxes of level l that a target in the (possibly virtual, outside the root box) box
// (bx, by) interpolates from: at level 2 every box not adjacent to it; deeper, the children of
// the boxes adjacent to its parent box that are not adjacent to it.  For a target inside the
// root box this is the cousin list above; with the adjacent leaf boxes (the direct near
// field) every source is counted once.
void target_list(const TreeLevel& L, int l, long long bx, long long by, std::vector<int>& out) {
    out.clear();
    std::vector<std::pair<long long, int>> tmp;
    auto consider = [&](long long i, long long j) {
        if (i < 0 || j < 0 || i >= L.nside || j >= L.nside) return;
        if (std::llabs(i - bx) <= 1 && std::llabs(j - by) <= 1) return;
        const long long cm = morton_of(i, j);
        const int b = L.find_box(cm);
        if (b >= 0) tmp.push_back({cm, b});
    };
    if (l == 2) {
        for (long long j = 0; j < L.nside; ++j)
            for (long long i = 0; i < L.nside; ++i) consider(i, j);
    } else {
        const long long px = bx >> 1, py = by >> 1;   // arithmetic shift: floor for negative boxes
        for (long long j = 2 * (py - 1); j <= 2 * (py + 1) + 1; ++j)
            for (long long i = 2 * (px - 1); i <= 2 * (px + 1) + 1; ++i) consider(i, j);
    }
    std::sort(tmp.begin(), tmp.end());
    for (auto& t : tmp) out.push_back(t.second);
}
// ---------------------------------------------------------------- build
std::string build_tree_boxes(const std::vector<double>& x, const std::vector<double>& y, int nlevels, double k,
                             int Ps, int Pang, Tree& T) {
    if (nlevels < 3) return "IFGF accelerator requires at least 3 levels.";
    if (nlevels > 24) return "nlevels too large";
    T = Tree();
    T.nlevels = nlevels; T.k = k; T.Ps = Ps; T.Pang = Pang; T.P = Ps * Pang; T.N = (long long)x.size();
    const long long N = T.N;
    const int D = nlevels - 1;
    tree_root_box(x, y, T.min_x, T.min_y, T.boxsize0);
    // Morton sort at the leaf level (stable), BoxTree.h:73-106
    std::vector<long long> code(N);
    const double leaf_size = T.boxsize0 / (double)(1LL << D);
    for (long long i = 0; i < N; ++i) {
        code[i] = point_morton(x[i], y[i], T.min_x, T.min_y, leaf_size, D);
        if (code[i] < 0) return "The 2D box index cannot be < 0 or larger than the number of boxes";
    }
    T.sorting.resize(N);
    std::iota(T.sorting.begin(), T.sorting.end(), 0LL);
    std::stable_sort(T.sorting.begin(), T.sorting.end(), [&](long long a, long long b) { return code[a] < code[b]; });
    T.inverse.resize(N);
    T.xs.resize(N); T.ys.resize(N);
    std::vector<long long>& scode = T.codes;
    scode.resize(N);
    for (long long i = 0; i < N; ++i) {
        T.inverse[T.sorting[i]] = i;
        T.xs[i] = x[T.sorting[i]]; T.ys[i] = y[T.sorting[i]]; scode[i] = code[T.sorting[i]];
    }
    // levels, relevant boxes (BoxTree.h:111-174, 205-231)
    T.L.resize(nlevels);
    for (int l = 1; l < nlevels; ++l) {
        TreeLevel& L = T.L[l];
        L.level = l; L.nside = 1LL << l; L.boxsize = T.boxsize0 / (double)(1LL << l);
        init_cones(L, k);
    }
    {
        TreeLevel& LD = T.L[D];
        for (long long i = 0; i < N; ++i) {
            if (i == 0 || scode[i] != scode[i - 1]) {
                LD.boxes.push_back(scode[i]);
                T.leaf_start.push_back((int)i);
                T.leaf_count.push_back(0);
            }
            T.leaf_count.back()++;
            T.point_leaf.push_back((int)LD.boxes.size() - 1);
        }
        for (int l = D - 1; l >= 2; --l) {
            std::vector<long long>& b = T.L[l].boxes;
            for (long long m : T.L[l + 1].boxes) b.push_back(m / 4);
            b.erase(std::unique(b.begin(), b.end()), b.end());   // parents of a sorted list stay sorted
        }
    }
    // leaf neighbours (Level.h:378-404)
    {
        const TreeLevel& LD = T.L[D];
        T.nbr_ptr.assign(LD.boxes.size() + 1, 0);
        for (size_t b = 0; b < LD.boxes.size(); ++b) {
            long long bx, by; box_of(LD.boxes[b], bx, by);
            std::vector<std::pair<long long, int>> nb;
            for (long long j = std::max<long long>(0, by - 1); j <= std::min<long long>(LD.nside - 1, by + 1); ++j)
                for (long long i = std::max<long long>(0, bx - 1); i <= std::min<long long>(LD.nside - 1, bx + 1); ++i) {
                    const long long m = morton_of(i, j);
                    const int q = LD.find_box(m);
                    if (q >= 0) nb.push_back({m, q});
                }
            std::sort(nb.begin(), nb.end());
            for (auto& e : nb) T.nbr_box.push_back(e.second);
            T.nbr_ptr[b + 1] = (int)T.nbr_box.size();
            long long nsrc = 0;
            for (auto& e : nb) nsrc += T.leaf_count[e.second];
            T.near_pairs += nsrc * T.leaf_count[b];
        }
    }
    return "";
}

std::string build_tree_cones(Tree& T, const std::function<void(int level)>& level_done) {
    const long long N = T.N;
    const int nlevels = T.nlevels, D = nlevels - 1, Ps = T.Ps, Pang = T.Pang;
    const std::vector<long long>& scode = T.codes;
    // Chebyshev nodes of the cone interpolant (ascending, Chebyshev.h:10-24); GetInterpolationPoint
    std::vector<double> ns(Ps), na(Pang);
    for (int i = 0; i < Ps; ++i) ns[Ps - 1 - i] = std::cos(kPiT * (2.0 * i + 1.0) / (2.0 * Ps));
    for (int i = 0; i < Pang; ++i) na[Pang - 1 - i] = std::cos(kPiT * (2.0 * i + 1.0) / (2.0 * Pang));
    const int P = T.P;

    std::vector<int, NoInitAlloc<int>> seen;   // finish_level's route table
    // relevant cones, level by level (BoxTree.h:553-583).  A wanted cone is the key
    // (box index << 32 | nonrel cone); each level's keys are collected per thread, then sorted
    // and deduplicated, which gives the cones in (box, nonrel) order.
    for (int l = 2; l < nlevels; ++l) {
        TreeLevel& L = T.L[l];
        LevelGeo G{&L, T.min_x, T.min_y};
        const int shift = 2 * (D - l);
        auto key = [](long long b, long long nonrel) { return ((unsigned long long)b << 32) | (unsigned long long)nonrel; };
        std::vector<std::vector<unsigned long long>> part;
        // cones seen by the cousins' points (BoxTree.h:235-277)
        {
            const long long nchunk = std::max<long long>(1, std::min<long long>(4 * kMaxThreads, N / 1024));
            part.resize(nchunk);
            parallel_for(nchunk, [&](long long c0, long long c1) {
                std::vector<int> cs;
                std::vector<long long> hr;   // per cousin: the last target's radial interval
                for (long long c = c0; c < c1; ++c) {
                    const long long i0 = N * c / nchunk, i1 = N * (c + 1) / nchunk;
                    long long old = -1;
                    auto& w = part[c];
                    for (long long i = i0; i < i1; ++i) {
                        const long long m = scode[i] >> shift;
                        if (m != old) { cousins_of(L, m, cs); old = m; hr.assign(cs.size(), -1); }
                        for (size_t j = 0; j < cs.size(); ++j)
                            w.push_back(key(cs[j], G.nonrel_of(L.boxes[cs[j]], T.xs[i], T.ys[i], hr[j])));
                    }
                    sort_unique(w);
                }
            }, 1);
        }
        std::string msg = finish_level(T, l, part, ns, na, seen);
        if (!msg.empty()) return msg;
        if (level_done) level_done(l);
    }
    // leaf-level cones have no children: close the propagation CSR for them
    if (T.pp_ptr.empty()) T.pp_ptr.assign(1, 0);
    while ((long long)T.pp_ptr.size() - 1 < T.total_cones) { T.pp_ptr.push_back(T.pp_total); T.pp_nchild.push_back(0); }
    for (size_t c = 0; c < T.L[D].cone_nonrel.size(); ++c) T.leaf_evals += (long long)P * T.leaf_count[T.L[D].cone_box[c]];
    return "";
}

std::string build_tree_interp(Tree& T) {
    const long long N = T.N;
    const int nlevels = T.nlevels, D = nlevels - 1;
    const double k = T.k;
    const std::vector<long long>& scode = T.codes;
    // interpolation plan (BoxTree.h:876-937): per sorted target, all levels, all cousins.  A
    // first pass counts each target's terms (its boxes' cousin counts), a second fills them in
    // place.
    T.ip_ptr.assign(N + 1, 0);
    {
        std::vector<std::vector<int>> ncous(nlevels);   // per level and box: cousin count
        for (int l = 2; l <= D; ++l) {
            const TreeLevel& L = T.L[l];
            ncous[l].assign(L.boxes.size(), 0);
            parallel_for((long long)L.boxes.size(), [&](long long b0, long long b1) {
                std::vector<int> cs;
                for (long long b = b0; b < b1; ++b) { cousins_of(L, L.boxes[b], cs); ncous[l][b] = (int)cs.size(); }
            }, 256);
        }
        std::vector<int> cnt(N, 0);
        parallel_for(N, [&](long long i0, long long i1) {
            for (int l = D; l >= 2; --l) {
                const TreeLevel& L = T.L[l];
                const int shift = 2 * (D - l);
                for (long long i = i0; i < i1; ++i) cnt[i] += ncous[l][L.find_box(scode[i] >> shift)];
            }
        });
        for (long long i = 0; i < N; ++i) T.ip_ptr[i + 1] = T.ip_ptr[i] + cnt[i];
        T.ip.resize(T.ip_ptr[N]);
        std::vector<char> bad(N, 0);
        parallel_for(N, [&](long long i0, long long i1) {
            std::vector<int> cs, hc;          // per cousin: the last target's cone
            std::vector<long long> hr;        // and radial interval
            std::vector<int> o(i1 - i0);
            for (long long i = i0; i < i1; ++i) o[i - i0] = T.ip_ptr[i];
            for (int l = D; l >= 2; --l) {   // the reference interpolates level D first (BoxTree.h:1049-1061)
                const TreeLevel& L = T.L[l];
                LevelGeo G{&L, T.min_x, T.min_y};
                const int shift = 2 * (D - l);
                long long old = -1;
                for (long long i = i0; i < i1; ++i) {
                    const long long m = scode[i] >> shift;
                    if (m != old) { cousins_of(L, m, cs); old = m; hr.assign(cs.size(), -1); hc.assign(cs.size(), -1); }
                    for (size_t j = 0; j < cs.size(); ++j) {
                        const int c = cs[j];
                        double lx = T.xs[i], ly = T.ys[i];
                        const long long nonrel = G.cart_to_cheb_cone(L.boxes[c], lx, ly, hr[j]);
                        const int cc = hc[j] >= 0 && L.cone_nonrel[hc[j]] == nonrel ? hc[j] : L.find_cone(c, nonrel);
                        hc[j] = cc;
                        if (cc < 0) { bad[i] = 1; T.ip[o[i - i0]++] = InterpEntry{0, l, 0.0, 0.0, 0.0, 0.0}; continue; }
                        const double r = G.cheb_to_radius(nonrel % L.nrad, lx);
                        const double sr = std::sqrt(r);
                        T.ip[o[i - i0]++] = InterpEntry{L.cone_base + cc, l, lx, ly, std::cos(k * r) / sr, std::sin(k * r) / sr};
                    }
                }
            }
        });
        for (long long i = 0; i < N; ++i) if (bad[i]) return "internal: interpolation cone missing";
        T.interp_evals = T.ip_ptr[N];
    }
    return "";
}

std::string build_tree(const std::vector<double>& x, const std::vector<double>& y, int nlevels, double k,
                       int Ps, int Pang, Tree& T) {
    std::string msg = build_tree_boxes(x, y, nlevels, k, Ps, Pang, T);
    if (msg.empty()) msg = build_tree_cones(T);
    if (msg.empty()) msg = build_tree_interp(T);
    return msg;
}

}  // namespace ifgf

namespace ifgf {

// ---------------------------------------------------------------- off-surface targets
std::string build_target_tree(const Tree& S, const std::vector<double>& tx, const std::vector<double>& ty, Tree& E) {
    if (tx.size() != ty.size()) return "target coordinate arrays differ in length";
    const int nlevels = S.nlevels, D = nlevels - 1;
    E = Tree();
    E.nlevels = nlevels; E.k = S.k; E.Ps = S.Ps; E.Pang = S.Pang; E.P = S.P; E.N = S.N;
    E.min_x = S.min_x; E.min_y = S.min_y; E.boxsize0 = S.boxsize0;
    E.leaf_start = S.leaf_start; E.leaf_count = S.leaf_count;
    const long long M = (long long)tx.size();
    // cone segments out to the farthest target: a box centre is within R of any target, and a
    // parent's interpolation node is within the parent's reach plus half a child diagonal of
    // the child's centre, hence the growth with the level
    const double cx0 = S.min_x + 0.5 * S.boxsize0, cy0 = S.min_y + 0.5 * S.boxsize0;
    double R = std::sqrt(2.0) * S.boxsize0;
    for (long long t = 0; t < M; ++t)
        R = std::max(R, std::hypot(tx[t] - cx0, ty[t] - cy0) + std::sqrt(2.0) / 2.0 * S.boxsize0);
    E.L.resize(nlevels);
    for (int l = 1; l < nlevels; ++l) {
        TreeLevel& L = E.L[l];
        L.level = l; L.nside = 1LL << l; L.boxsize = S.L[l].boxsize;
        L.boxes = S.L[l].boxes;
        const double reach = (R + std::sqrt(2.0) * S.boxsize0 * (1.0 - std::ldexp(1.0, -l))) * (1.0 + 1e-10);
        init_cones(L, E.k, reach);
    }
    // virtual leaf boxes of the targets (may lie outside [0, 2^D))
    const double bsD = E.L[D].boxsize;
    std::vector<long long> tbx(M), tby(M);
    for (long long t = 0; t < M; ++t) {
        tbx[t] = (long long)std::floor((tx[t] - E.min_x) / bsD);
        tby[t] = (long long)std::floor((ty[t] - E.min_y) / bsD);
    }
    std::vector<double> ns(E.Ps), na(E.Pang);
    for (int i = 0; i < E.Ps; ++i) ns[E.Ps - 1 - i] = std::cos(kPiT * (2.0 * i + 1.0) / (2.0 * E.Ps));
    for (int i = 0; i < E.Pang; ++i) na[E.Pang - 1 - i] = std::cos(kPiT * (2.0 * i + 1.0) / (2.0 * E.Pang));
    const int P = E.P;
    std::vector<int, NoInitAlloc<int>> seen;   // finish_level's route table
    for (int l = 2; l < nlevels; ++l) {
        TreeLevel& L = E.L[l];
        LevelGeo G{&L, E.min_x, E.min_y};
        const int sh = D - l;
        const long long nchunk = std::max<long long>(1, std::min<long long>(4 * kMaxThreads, M / 256));
        std::vector<std::vector<unsigned long long>> part(nchunk);
        parallel_for(nchunk, [&](long long c0, long long c1) {
            std::vector<int> cs;
            for (long long c = c0; c < c1; ++c) {
                auto& w = part[c];
                for (long long t = M * c / nchunk; t < M * (c + 1) / nchunk; ++t) {
                    target_list(L, l, tbx[t] >> sh, tby[t] >> sh, cs);
                    for (int cb : cs)
                        w.push_back(((unsigned long long)cb << 32) | (unsigned long long)G.nonrel_of(L.boxes[cb], tx[t], ty[t]));
                }
                sort_unique(w);
            }
        }, 1);
        // a level whose targets see no box still needs the cones its parents route to
        bool any = false;
        for (auto& w : part) any = any || !w.empty();
        if (!any && l == 2) part.assign(1, std::vector<unsigned long long>{});
        std::string msg = finish_level(E, l, part, ns, na, seen);
        if (!msg.empty() && msg != "The number of cone segments on any level cannot be 0") return msg;
        if (!msg.empty()) {   // no cone at this level: empty lists, nothing below needs it either
            TreeLevel& Le = E.L[l];
            Le.cone_ptr.assign(Le.boxes.size() + 1, 0);
            Le.cone_box.clear(); Le.cone_nonrel.clear();
            Le.cone_base = E.total_cones;
            if (l > 2) {
                const TreeLevel& Lp = E.L[l - 1];
                if (E.pp_ptr.empty()) E.pp_ptr.assign(1, 0);
                for (size_t pc = 0; pc < Lp.cone_nonrel.size(); ++pc) { E.pp_nchild.push_back(0); E.pp_ptr.push_back(E.pp_ptr.back()); }
            }
        }
    }
    if (E.pp_ptr.empty()) E.pp_ptr.assign(1, 0);
    while ((long long)E.pp_ptr.size() - 1 < E.total_cones) { E.pp_ptr.push_back(E.pp_total); E.pp_nchild.push_back(0); }
    for (size_t c = 0; c < E.L[D].cone_nonrel.size(); ++c) E.leaf_evals += (long long)P * E.leaf_count[E.L[D].cone_box[c]];
    // per target: interpolation entries, level D first (BoxTree.h:1049-1061), and the
    // adjacent leaf boxes of the direct near field
    std::vector<std::vector<InterpEntry>> per(M);
    std::vector<std::vector<int>> nb(M);
    std::vector<char> bad(M, 0);
    parallel_for(M, [&](long long t0, long long t1) {
        std::vector<int> cs;
        for (long long t = t0; t < t1; ++t) {
            for (int l = D; l >= 2; --l) {
                const TreeLevel& L = E.L[l];
                LevelGeo G{&L, E.min_x, E.min_y};
                target_list(L, l, tbx[t] >> (D - l), tby[t] >> (D - l), cs);
                for (int c : cs) {
                    double lx = tx[t], ly = ty[t];
                    const long long nonrel = G.cart_to_cheb_cone(L.boxes[c], lx, ly);
                    const int cc = L.find_cone(c, nonrel);
                    if (cc < 0) { bad[t] = 1; continue; }
                    const double r = G.cheb_to_radius(nonrel % L.nrad, lx);
                    const double sr = std::sqrt(r);
                    per[t].push_back(InterpEntry{L.cone_base + cc, l, lx, ly, std::cos(E.k * r) / sr, std::sin(E.k * r) / sr});
                }
            }
            const TreeLevel& LD = E.L[D];
            std::vector<std::pair<long long, int>> tmp;
            for (long long j = tby[t] - 1; j <= tby[t] + 1; ++j)
                for (long long i = tbx[t] - 1; i <= tbx[t] + 1; ++i) {
                    if (i < 0 || j < 0 || i >= LD.nside || j >= LD.nside) continue;
                    const long long m = morton_of(i, j);
                    const int q = LD.find_box(m);
                    if (q >= 0) tmp.push_back({m, q});
                }
            std::sort(tmp.begin(), tmp.end());
            for (auto& e : tmp) nb[t].push_back(e.second);
        }
    });
    for (long long t = 0; t < M; ++t) if (bad[t]) return "internal: target interpolation cone missing";
    E.ip_ptr.assign(M + 1, 0);
    E.nbr_ptr.assign(M + 1, 0);
    for (long long t = 0; t < M; ++t) {
        E.ip_ptr[t + 1] = E.ip_ptr[t] + (int)per[t].size();
        E.nbr_ptr[t + 1] = E.nbr_ptr[t] + (int)nb[t].size();
        for (int q : nb[t]) E.near_pairs += E.leaf_count[q];
    }
    E.ip.reserve(E.ip_ptr[M]);
    E.nbr_box.reserve(E.nbr_ptr[M]);
    for (long long t = 0; t < M; ++t) {
        E.ip.insert(E.ip.end(), per[t].begin(), per[t].end());
        E.nbr_box.insert(E.nbr_box.end(), nb[t].begin(), nb[t].end());
    }
    E.interp_evals = E.ip_ptr[M];
    return "";
}

}  // namespace ifgf
