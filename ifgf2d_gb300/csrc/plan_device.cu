// plan_device.cu -- the IFGF propagation plan built on the device.
//
// The plan holds, for every parent cone segment, child box and parent interpolation node, the
// child cone that node falls in, the node's Chebyshev coordinates in that cone and the ratio of
// the factored kernel e^{ikr}/sqrt(r) between the child and parent centres (BoxTree.h:767-868,
// Level.h:347-437).  The host keeps the structure -- which cones exist, the protobox routes
// (BoxTree.h:299-428), one slot per (parent cone, child box) -- and the device computes the
// entries, one thread per (slot, node), writing the FP64 plan and its complex64 copy.  That
// moves the bulk of the set-up arithmetic (tens of millions of entries at N = 131072, each with
// trigonometric and square-root evaluations) off the host, and the entries never cross the bus.
//
// The geometry follows the host restatement in tree.cpp step for step; this translation unit
// is compiled without FMA contraction so the arithmetic rounds as the host's does, and only
// the device's cos / sin / atan may differ from the host's by an ulp.
#include "context.hpp"
#include <memory>

namespace ifgf {
namespace {

constexpr double kPiD = 3.14159265358979323846;

// one tree level, as the plan kernel reads it
struct LevelDesc {
    const long long* boxes;        // relevant boxes (Morton codes, ascending)
    const int* cone_box;           // per cone: box index
    const long long* cone_nonrel;  // per cone: cone segment (nonrel)
    const int* cone_ptr;           // per box: first cone
    const double* radial;          // nrad + 1 radial interval ends
    double boxsize, scaling;
    long long nrad, ntheta;
    int cone_base;
};
struct ChebNodes { double s[8], a[8]; };

__device__ __forceinline__ unsigned long long gather_bits(unsigned long long x) {
    x &= 0x5555555555555555ull;
    x = (x ^ (x >> 1)) & 0x3333333333333333ull;
    x = (x ^ (x >> 2)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x ^ (x >> 4)) & 0x00FF00FF00FF00FFull;
    x = (x ^ (x >> 8)) & 0x0000FFFF0000FFFFull;
    x = (x ^ (x >> 16)) & 0xFFFFFFFFull;
    return x;
}
__device__ __forceinline__ void center(const LevelDesc& L, double min_x, double min_y, long long m, double& cx, double& cy) {
    const long long bx = (long long)gather_bits((unsigned long long)m), by = (long long)gather_bits((unsigned long long)m >> 1);
    cx = min_x + bx * L.boxsize + 0.5 * L.boxsize;
    cy = min_y + by * L.boxsize + 0.5 * L.boxsize;
}
// polar angle in [0, 2 pi) (PolarCoordinates.h:8-27)
__device__ double atan_0_2pi(double y, double x) {
    if (x > 0 && y >= 0) return atan(y / x);
    if (x > 0 && y < 0) return atan(y / x) + 2.0 * kPiD;
    if (x < 0 && y > 0) return atan(y / x) + kPiD;
    if (x < 0 && y == 0) return kPiD;
    if (x < 0 && y < 0) return atan(y / x) + kPiD;
    if (x == 0 && y > 0) return kPiD / 2;
    if (x == 0 && y < 0) return 3.0 * kPiD / 2;
    return 0;
}
__device__ __forceinline__ double cheb_to_radius(const LevelDesc& L, long long pr, double s) {   // Level.h:347-356
    const double rmin = L.scaling / L.radial[pr + 1];
    const double dr = L.scaling / L.radial[pr] - rmin;
    return L.scaling / ((s + 1.0) / 2.0 * dr + rmin);
}
__device__ __forceinline__ double radius_to_cheb(const LevelDesc& L, long long pr, double r) {   // Level.h:413-422
    const double rmin = L.scaling / L.radial[pr + 1];
    const double dr = L.scaling / L.radial[pr] - rmin;
    return (L.scaling / r - rmin) / dr * 2.0 - 1.0;
}

// one thread per (slot, parent node): the plan entry of that node in the slot's child box
__global__ void k_prop_plan(LevelDesc Lp, LevelDesc Lc, double min_x, double min_y, double k, int Ps, ChebNodes cn, int P,
                            const int* __restrict__ slot_parent, const int* __restrict__ slot_child_box,
                            const int* __restrict__ slot_pos, const int* __restrict__ slot_route,
                            const int* __restrict__ route_nonrel, long long nslots, PropE<double>* __restrict__ out64,
                            PropE<float>* __restrict__ out32, int* __restrict__ err) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nslots * P) return;
    const long long q = idx / P;
    const int it = (int)(idx - q * P);
    const int pc = slot_parent[q], cb = slot_child_box[q];
    const long long pm = Lp.boxes[Lp.cone_box[pc]], pnc = Lp.cone_nonrel[pc];
    const long long cm = pm * 4 + slot_pos[q];
    const long long nonrel = route_nonrel[(long long)slot_route[q] * P + it];
    // the parent node in Cartesian coordinates (Level.h:358-375)
    const long long ppr = pnc % Lp.nrad, ppt = pnc / Lp.nrad;
    const double pda = kPiD / Lp.ntheta;
    const double rp = cheb_to_radius(Lp, ppr, cn.s[it % Ps]);
    const double th = (cn.a[it / Ps] + 1.0) / 2.0 * pda + pda * ppt;
    double pcx, pcy;
    center(Lp, min_x, min_y, pm, pcx, pcy);
    double x = rp * cos(th) + pcx, y = rp * sin(th) + pcy;
    // its Chebyshev coordinates in the child's cone segment `nonrel` (Level.h:424-437)
    double ccx, ccy;
    center(Lc, min_x, min_y, cm, ccx, ccy);
    x -= ccx;
    y -= ccy;
    double r = sqrt(x * x + y * y), a = 0.0;
    if (r == 0.0) r = 0.0; else a = atan_0_2pi(y, x);
    const long long cpr = nonrel % Lc.nrad, cpt = nonrel / Lc.nrad;
    const double cda = kPiD / Lc.ntheta;
    const double ls = radius_to_cheb(Lc, cpr, r);
    const double lt = (a - cda * cpt) / cda * 2.0 - 1.0;
    const double rc = cheb_to_radius(Lc, cpr, ls);
    // the child cone's index: binary search in the child box's sorted cone segments
    int lo = Lc.cone_ptr[cb], hi = Lc.cone_ptr[cb + 1];
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (Lc.cone_nonrel[mid] < nonrel) lo = mid + 1; else hi = mid;
    }
    const long long e = idx;
    if (lo >= Lc.cone_ptr[cb + 1] || Lc.cone_nonrel[lo] != nonrel) {
        atomicExch(err, 1);
        out64[e] = PropE<double>{0, it, 0.0, 0.0, 0.0, 0.0};
        if (out32) out32[e] = PropE<float>{0, 0.f, 0.f, 0.f, 0.f};
        return;
    }
    // e^{ik rc}/sqrt(rc) / (e^{ik rp}/sqrt(rp))
    double sc, cc, sp, cp;
    sincos(k * rc, &sc, &cc);
    sincos(k * rp, &sp, &cp);
    const double ic = 1.0 / sqrt(rc), ip = 1.0 / sqrt(rp);
    const double fr = cc * ic, fi = sc * ic, gr = cp * ip, gi = sp * ip;
    const double den = gr * gr + gi * gi;
    const double wr = (fr * gr + fi * gi) / den, wi = (fi * gr - fr * gi) / den;
    const int child = Lc.cone_base + lo;
    out64[e] = PropE<double>{child, it, ls, lt, wr, wi};
    if (out32) out32[e] = PropE<float>{child, (float)ls, (float)lt, (float)wr, (float)wi};
}

// one thread per (leaf cone, node): the node's position and 1 / (e^{ikr}/sqrt(r)) at its radius
// (BoxTree.h:714-745)
__global__ void k_leaf_nodes(LevelDesc L, double min_x, double min_y, double k, int Ps, ChebNodes cn, int P, long long ncones,
                             LeafNode* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ncones * P) return;
    const long long c = idx / P;
    const int it = (int)(idx - c * P);
    const long long m = L.boxes[L.cone_box[c]], nonrel = L.cone_nonrel[c];
    const long long pr = nonrel % L.nrad, pt = nonrel / L.nrad;
    const double da = kPiD / L.ntheta;
    const double r = cheb_to_radius(L, pr, cn.s[it % Ps]);
    const double th = (cn.a[it / Ps] + 1.0) / 2.0 * da + da * pt;
    double cx, cy;
    center(L, min_x, min_y, m, cx, cy);
    double sk, ck;
    sincos(k * r, &sk, &ck);
    const double sr = sqrt(r);   // 1 / (e^{ikr} / sqrt(r)) = sqrt(r) e^{-ikr}
    out[idx] = LeafNode{r * cos(th) + cx, r * sin(th) + cy, ck * sr, -sk * sr};
}

// a parent's terms sorted by child cone (stable), with the parent node (entry index mod P)
// recorded: one warp per parent cone, each lane ranking its entries against the parent's
// child-cone list in shared memory
constexpr int kSortWarps = 8;
template <typename R>
__global__ void __launch_bounds__(kSortWarps * 32) k_sort_plan(const long long* __restrict__ pp_ptr, int ncones,
                                                               const PropE<double>* __restrict__ pp, int P,
                                                               PropB<R>* __restrict__ out) {
    __shared__ int cc[kSortWarps][4 * kMaxP];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pc = blockIdx.x * kSortWarps + warp;
    if (pc >= ncones) return;
    const long long e0 = pp_ptr[pc];
    const int ne = (int)(pp_ptr[pc + 1] - e0);
    for (int i = lane; i < ne; i += 32) cc[warp][i] = pp[e0 + i].child_cone;
    __syncwarp();
    for (int i = lane; i < ne; i += 32) {
        const int c = cc[warp][i];
        int rank = 0;
        for (int j = 0; j < ne; ++j) {
            const int d = cc[warp][j];
            rank += (d < c) || (d == c && j < i);
        }
        const PropE<double> E = pp[e0 + i];
        out[e0 + rank] = PropB<R>{E.child_cone, i % P, (R)E.s, (R)E.th, (R)E.wr, (R)E.wi};
    }
}

__global__ void k_interp_to_c64(const InterpE<double>* __restrict__ in, long long n, InterpE<float>* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const InterpE<double> e = in[i];
    out[i] = InterpE<float>{e.cone, (float)e.s, (float)e.th, (float)e.fr, (float)e.fi};
}

// device copies of one level's arrays, kept alive until the plan kernels ran
struct LevelBufs {
    DBuf<long long> boxes, cone_nonrel;
    DBuf<int> cone_box, cone_ptr;
    DBuf<double> radial;
};
cudaError_t upload_level(const TreeLevel& L, int cone_base, LevelBufs& B, LevelDesc& d) {
    cudaError_t e;
    if ((e = B.boxes.upload(L.boxes)) != cudaSuccess) return e;
    if ((e = B.cone_nonrel.upload(L.cone_nonrel)) != cudaSuccess) return e;
    if ((e = B.cone_box.upload(L.cone_box)) != cudaSuccess) return e;
    if ((e = B.cone_ptr.upload(L.cone_ptr)) != cudaSuccess) return e;
    if ((e = B.radial.upload(L.radial)) != cudaSuccess) return e;
    d = LevelDesc{B.boxes.p, B.cone_box.p, B.cone_nonrel.p, B.cone_ptr.p, B.radial.p, L.boxsize, L.scaling_r2s, L.nrad,
                  L.ntheta, cone_base};
    return cudaSuccess;
}

}  // namespace

cudaError_t build_prop_plan(const Tree& T, PropE<double>* pp64, PropE<float>* pp32, int* err, cudaStream_t s,
                            const int* level_cone_base, const long long* level_entry_base) {
    if (T.Ps > 8 || T.Pang > 8) return cudaErrorInvalidValue;
    ChebNodes cn{};
    // Chebyshev nodes of the cone interpolant, ascending (Chebyshev.h:10-24), as the host tree has them
    for (int i = 0; i < T.Ps; ++i) cn.s[T.Ps - 1 - i] = std::cos(kPiD * (2.0 * i + 1.0) / (2.0 * T.Ps));
    for (int i = 0; i < T.Pang; ++i) cn.a[T.Pang - 1 - i] = std::cos(kPiD * (2.0 * i + 1.0) / (2.0 * T.Pang));
    // every input buffer lives until the kernels ran.  All levels are uploaded before the first
    // launch: a copy from pageable host memory queued behind a running kernel holds the host
    // until the kernel ends.
    std::vector<LevelBufs> lb(T.nlevels);
    std::vector<LevelDesc> ld(T.nlevels);
    std::vector<char> up(T.nlevels, 0);
    const size_t ns = T.prop_slots.size();
    std::vector<DBuf<int>> sp(ns), scb(ns), spos(ns), sr(ns);
    std::vector<DBuf<int>> rn(ns);
    cudaError_t e = cudaSuccess;
    for (size_t q = 0; q < ns && e == cudaSuccess; ++q) {
        const PropSlots& S = T.prop_slots[q];
        if (S.slot_parent.empty()) continue;
        for (int l : {S.level - 1, S.level})
            if (!up[l] && e == cudaSuccess) {
                e = upload_level(T.L[l], level_cone_base ? level_cone_base[l] : T.L[l].cone_base, lb[l], ld[l]);
                up[l] = 1;
            }
        if (e == cudaSuccess) e = sp[q].upload(S.slot_parent);
        if (e == cudaSuccess) e = scb[q].upload(S.slot_child_box);
        if (e == cudaSuccess) e = spos[q].upload(S.slot_pos);
        if (e == cudaSuccess) e = sr[q].upload(S.slot_route);
        if (e == cudaSuccess) e = rn[q].upload(S.route_nonrel.data(), S.route_nonrel.size());
    }
    for (size_t q = 0; q < ns && e == cudaSuccess; ++q) {
        const PropSlots& S = T.prop_slots[q];
        const long long nslots = (long long)S.slot_parent.size();
        if (nslots == 0) continue;
        const long long n = nslots * T.P;
        const long long eb = level_entry_base ? level_entry_base[S.level] : S.entry_base;
        k_prop_plan<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(ld[S.level - 1], ld[S.level], T.min_x, T.min_y, T.k, T.Ps, cn, T.P,
                                                                 sp[q].p, scb[q].p, spos[q].p, sr[q].p, rn[q].p, nslots,
                                                                 pp64 + eb, pp32 ? pp32 + eb : nullptr, err);
        e = cudaGetLastError();
    }
    // stream-ordered buffers are freed in stream order after the kernels; plain ones need the
    // kernels finished first
    if (alloc_stream() == s && e == cudaSuccess) return cudaSuccess;
    const cudaError_t es = cudaStreamSynchronize(s);
    return e != cudaSuccess ? e : es;
}

struct PropPlanByLevel::Impl {
    struct Level {
        long long entry_base = 0, n = 0;
        DBuf<int> sp, scb, spos, sr, rn;
        DBuf<PropE<double>> o64;
        DBuf<PropE<float>> o32;
    };
    cudaStream_t st = nullptr;
    cudaEvent_t ready = nullptr, done = nullptr;
    cudaError_t status = cudaSuccess;
    std::vector<std::unique_ptr<LevelBufs>> lb;
    std::vector<LevelDesc> ld;
    std::vector<char> up;
    std::vector<std::unique_ptr<Level>> lv;
    DBuf<int> err;
    ChebNodes cn{};
    ~Impl() {
        lv.clear();   // stream-ordered frees on st, after its copies
        lb.clear();
        err.release();
        if (ready) cudaEventDestroy(ready);
        if (done) cudaEventDestroy(done);
        if (st) cudaStreamDestroy(st);   // released once its queued work is done
    }
};

PropPlanByLevel::PropPlanByLevel() : d(new Impl) {
    d->status = cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking);
    if (d->status == cudaSuccess) d->status = cudaEventCreateWithFlags(&d->ready, cudaEventDisableTiming);
    if (d->status == cudaSuccess) d->status = cudaEventCreateWithFlags(&d->done, cudaEventDisableTiming);
}
PropPlanByLevel::~PropPlanByLevel() { delete d; }

void PropPlanByLevel::add(const Tree& T, int l) {
    Impl& I = *d;
    if (I.status != cudaSuccess) return;
    if (T.Ps > 8 || T.Pang > 8 || T.prop_slots.empty() || T.prop_slots.back().level != l) { I.status = cudaErrorInvalidValue; return; }
    AllocStream guard(I.st);
    cudaError_t e = cudaSuccess;
    if (I.lb.empty()) {
        for (int q = 0; q < T.nlevels; ++q) I.lb.emplace_back(new LevelBufs);
        I.ld.resize(T.nlevels); I.up.assign(T.nlevels, 0);
        for (int i = 0; i < T.Ps; ++i) I.cn.s[T.Ps - 1 - i] = std::cos(kPiD * (2.0 * i + 1.0) / (2.0 * T.Ps));
        for (int i = 0; i < T.Pang; ++i) I.cn.a[T.Pang - 1 - i] = std::cos(kPiD * (2.0 * i + 1.0) / (2.0 * T.Pang));
        e = I.err.alloc(1);
        if (e == cudaSuccess) e = cudaMemsetAsync(I.err.p, 0, sizeof(int), I.st);
    }
    // the levels' arrays are final once their cones exist: level l - 1 was uploaded with the
    // previous level (as its child level), level l now
    for (int q : {l - 1, l})
        if (!I.up[q] && e == cudaSuccess) {
            e = upload_level(T.L[q], T.L[q].cone_base, *I.lb[q], I.ld[q]);
            I.up[q] = 1;
        }
    const PropSlots& S = T.prop_slots.back();
    std::unique_ptr<Impl::Level> vp(new Impl::Level);
    Impl::Level& v = *vp;
    v.entry_base = S.entry_base;
    v.n = (long long)S.slot_parent.size() * T.P;
    if (v.n > 0 && e == cudaSuccess) {
        if (e == cudaSuccess) e = v.sp.upload(S.slot_parent);
        if (e == cudaSuccess) e = v.scb.upload(S.slot_child_box);
        if (e == cudaSuccess) e = v.spos.upload(S.slot_pos);
        if (e == cudaSuccess) e = v.sr.upload(S.slot_route);
        if (e == cudaSuccess) e = v.rn.upload(S.route_nonrel.data(), S.route_nonrel.size());
        if (e == cudaSuccess) e = v.o64.alloc((size_t)v.n);
        if (e == cudaSuccess) e = v.o32.alloc((size_t)v.n);
        if (e == cudaSuccess) {
            k_prop_plan<<<(unsigned)((v.n + 255) / 256), 256, 0, I.st>>>(I.ld[l - 1], I.ld[l], T.min_x, T.min_y, T.k, T.Ps, I.cn, T.P,
                                                                         v.sp.p, v.scb.p, v.spos.p, v.sr.p, v.rn.p,
                                                                         (long long)S.slot_parent.size(), v.o64.p, v.o32.p, I.err.p);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) { I.status = e; return; }
    I.lv.push_back(std::move(vp));
}

cudaError_t PropPlanByLevel::gather(PropE<double>* pp64, PropE<float>* pp32, int* err, cudaStream_t s) {
    Impl& I = *d;
    if (I.status != cudaSuccess) return I.status;
    AllocStream guard(I.st);
    cudaError_t e = cudaEventRecord(I.ready, s);   // the plan's allocation on s
    if (e == cudaSuccess) e = cudaStreamWaitEvent(I.st, I.ready, 0);
    for (const auto& vp : I.lv) {
        const Impl::Level& v = *vp;
        if (v.n == 0 || e != cudaSuccess) continue;
        e = cudaMemcpyAsync(pp64 + v.entry_base, v.o64.p, sizeof(PropE<double>) * (size_t)v.n, cudaMemcpyDeviceToDevice, I.st);
        if (e == cudaSuccess && pp32)
            e = cudaMemcpyAsync(pp32 + v.entry_base, v.o32.p, sizeof(PropE<float>) * (size_t)v.n, cudaMemcpyDeviceToDevice, I.st);
    }
    if (e == cudaSuccess && I.err.p) e = cudaMemcpyAsync(err, I.err.p, sizeof(int), cudaMemcpyDeviceToDevice, I.st);
    if (e == cudaSuccess) e = cudaEventRecord(I.done, I.st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, I.done, 0);
    I.lv.clear();   // the level buffers are freed on st after the copies
    return e;
}

cudaError_t build_leaf_nodes(const Tree& T, LeafNode* out, cudaStream_t s) {
    if (T.Ps > 8 || T.Pang > 8) return cudaErrorInvalidValue;
    const TreeLevel& L = T.L[T.nlevels - 1];
    const long long nc = (long long)L.cone_nonrel.size();
    if (nc == 0) return cudaSuccess;
    ChebNodes cn{};
    for (int i = 0; i < T.Ps; ++i) cn.s[T.Ps - 1 - i] = std::cos(kPiD * (2.0 * i + 1.0) / (2.0 * T.Ps));
    for (int i = 0; i < T.Pang; ++i) cn.a[T.Pang - 1 - i] = std::cos(kPiD * (2.0 * i + 1.0) / (2.0 * T.Pang));
    LevelBufs lb;
    LevelDesc d;
    cudaError_t e = upload_level(L, L.cone_base, lb, d);
    if (e != cudaSuccess) return e;
    const long long n = nc * T.P;
    k_leaf_nodes<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, T.min_x, T.min_y, T.k, T.Ps, cn, T.P, nc, out);
    e = cudaGetLastError();
    if (alloc_stream() == s && e == cudaSuccess) return cudaSuccess;   // stream-ordered inputs: freed after the kernel
    const cudaError_t es = cudaStreamSynchronize(s);
    return e != cudaSuccess ? e : es;
}

template <typename R>
void launch_sort_plan(const long long* pp_ptr, int ncones, const PropE<double>* pp, int P, PropB<R>* out, cudaStream_t s) {
    if (ncones <= 0) return;
    k_sort_plan<R><<<(ncones + kSortWarps - 1) / kSortWarps, kSortWarps * 32, 0, s>>>(pp_ptr, ncones, pp, P, out);
}
template void launch_sort_plan<double>(const long long*, int, const PropE<double>*, int, PropB<double>*, cudaStream_t);
template void launch_sort_plan<float>(const long long*, int, const PropE<double>*, int, PropB<float>*, cudaStream_t);

void launch_interp_to_c64(const InterpE<double>* in, long long n, InterpE<float>* out, cudaStream_t s) {
    if (n <= 0) return;
    k_interp_to_c64<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, n, out);
}

}  // namespace ifgf
