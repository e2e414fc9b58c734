// tree.hpp -- host build of the IFGF box tree, flattened for the device.
//
// Reproduces the tree of IFGF_Source/BoxTree.h + Level.h (Morton sort, relevant boxes,
// cone segments, cousin/neighbour rules, protobox routing) and turns it into plain arrays:
//   * points in Morton order (BoxTree.h:73-106), leaf boxes as contiguous point ranges;
//   * all relevant cones of all levels numbered globally (one coefficient buffer);
//   * an interpolation plan: per target point, its (cone, s, theta, e^{ikr}/sqrt r) entries
//     over all levels and cousins (BoxTree.h:876-937);
//   * a propagation plan: per parent cone, per child and interpolation node, the child cone,
//     its Chebyshev coordinates and the factor ratio (BoxTree.h:767-868), kept here in the
//     compact slot form (PropSlots) whose entries the device computes;
//   * per leaf box, the neighbour ranges of the near field (BoxTree.h:614-683).
#pragma once

#include <vector>
#include <string>
#include <cstdint>
#include <complex>
#include <functional>
#include <memory>
#include <utility>

namespace ifgf {

struct TreeLevel {
    int level = 0;
    double boxsize = 0.0;
    long long nside = 0;
    double scaling_r2s = 0.0;
    long long ntheta = 0, nrad = 0;
    std::vector<double> radial;            // nrad + 1 radial interval ends (Level.h:131-140)
    std::vector<long long> boxes;          // relevant boxes, ascending Morton codes
    std::vector<int> cone_ptr;             // per box: its cones [cone_ptr[b], cone_ptr[b+1])
    std::vector<long long> cone_nonrel;    // per cone (local numbering)
    std::vector<int> cone_box;             // per cone: box index
    int cone_base = 0;                     // global id of this level's first cone

    int find_box(long long morton) const;
    int find_cone(int box, long long nonrel) const;   // local cone id or -1
};

struct InterpEntry {   // one (target, level, cousin) term of the interpolation
    int cone;          // global cone id
    int pad;
    double s, th;      // Chebyshev coordinates in the cousin's cone
    double fr, fi;     // e^{ikr}/sqrt(r)
};

struct PropEntry {     // one (parent cone, child, node) term of the propagation
    int child_cone;    // global cone id at the child level
    int pad;
    double s, th;      // Chebyshev coordinates of the parent node in the child cone
    double wr, wi;     // e^{ik r_child}/sqrt(r_child) / (e^{ik r_parent}/sqrt(r_parent))
};

// The propagation plan of one level pair (parents at level l - 1, children at level l), in
// the compact form the host builds: the entries themselves (PropEntry, one per slot and node)
// are computed on the device from it (plan_device.cu).  A slot is one (parent cone, child box)
// pair; slots are in parent-cone order, then child position, so slot q's entries are
// pp[entry_base + q * P + node].  route_nonrel holds, per route (a parent cone segment and a
// child position, BoxTree.h:299-428), the child's cone segment of each of the P parent nodes.
// an allocator whose value-less construct leaves the element uninitialised, so that resizing a
// large table that a parallel loop fills anyway costs no serial zero fill
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = NoInitAlloc<U>; };
    NoInitAlloc() = default;
    template <class U> NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <class U> void construct(U* p) noexcept { ::new ((void*)p) U; }
    template <class U, class... A> void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};

struct PropSlots {
    int level = 0;                        // child level l
    long long entry_base = 0;             // global index of the first entry
    std::vector<int> slot_parent;         // parent cone, local index at level l - 1
    std::vector<int> slot_child_box;      // child box index at level l
    std::vector<int> slot_pos;            // child position 0..3 (child Morton = parent * 4 + pos)
    std::vector<int> slot_route;          // route index
    std::vector<int, NoInitAlloc<int>> route_nonrel;   // per route, P child cone segments in node order
};

struct Tree {
    int nlevels = 0, Ps = 5, Pang = 5, P = 25;
    long long N = 0;
    double k = 0.0;
    double min_x = 0, min_y = 0, boxsize0 = 0;
    std::vector<long long> sorting, inverse;   // sorted position -> original index, and back
    std::vector<double> xs, ys;                // Morton-sorted coordinates
    std::vector<long long> codes;              // their leaf-level Morton codes
    std::vector<TreeLevel> L;                  // index = level; 0 and 1 unused
    // leaf boxes (level D = nlevels-1)
    std::vector<int> leaf_start, leaf_count, point_leaf;
    std::vector<int> nbr_ptr, nbr_box;         // per leaf box: neighbour leaf boxes (<= 9)
    int total_cones = 0;
    // interpolation plan (CSR over sorted target points)
    std::vector<int> ip_ptr;
    std::vector<InterpEntry> ip;
    // propagation plan: for each level l in [3, D] the parent cones are those of level l-1;
    // CSR over parent global cone ids: pp_ptr[c] .. pp_ptr[c+1], grouped by child then node.
    // The entries are built on the device from prop_slots (pp_total of them).
    std::vector<long long> pp_ptr;
    std::vector<PropSlots> prop_slots;
    long long pp_total = 0;
    std::vector<int> pp_nchild;                // per parent cone: number of relevant children
    long long prop_evals = 0, interp_evals = 0, leaf_evals = 0, near_pairs = 0;
};

// Build the tree for the given points (original order).  Returns "" or an error message.
std::string build_tree(const std::vector<double>& x, const std::vector<double>& y, int nlevels, double k,
                       int Ps, int Pang, Tree& T);
// build_tree in its three stages, for a caller that starts device work between them: the boxes
// (Morton sort, relevant boxes, leaf neighbours), then the cones of every level with the
// propagation plan's slot form, then the interpolation plan.  Each returns "" or an error
// message and needs the stages before it.  build_tree_cones calls level_done(l) once level l's
// cones and, for l > 2, its propagation slots (T.prop_slots.back()) are final.
std::string build_tree_boxes(const std::vector<double>& x, const std::vector<double>& y, int nlevels, double k,
                             int Ps, int Pang, Tree& T);
std::string build_tree_cones(Tree& T, const std::function<void(int level)>& level_done = nullptr);
std::string build_tree_interp(Tree& T);

// Evaluation plan for off-surface targets (the accelerated form of ForwardMap::propagate_unacc,
// ForwardMap.tpp:701-727).  E keeps the source boxes of S (sources, leaf ranges, Morton order)
// and gets the cones and propagation plan the targets need, with cone segments reaching the
// farthest target.  Per target, in input order: interpolation entries (E.ip_ptr / E.ip) and
// the adjacent leaf boxes of the direct near field (E.nbr_ptr / E.nbr_box).
std::string build_target_tree(const Tree& S, const std::vector<double>& tx, const std::vector<double>& ty, Tree& E);

// Morton code of (x, y) at `level` for a root box [min_x, min_x + size] (Level.h:145-161);
// returns -1 when the point is outside.
long long point_morton(double x, double y, double min_x, double min_y, double boxsize, int level);
void tree_root_box(const std::vector<double>& x, const std::vector<double>& y, double& min_x, double& min_y, double& size);

}  // namespace ifgf
