// ifgf_device.cuh -- device helpers shared by the single-vector and the batched IFGF apply:
// complex multiply-add in the arithmetic type, warp sums, the cone interpolant evaluation and
// the compile-time dispatch over the supported (Ps, Pang).
#pragma once
#include "ifgf2d_kernels.cuh"

namespace ifgf {

__device__ __forceinline__ double rfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return fmaf(a, b, c); }

template <typename R>
__device__ __forceinline__ void cmac(V2<R>& acc, V2<R> a, V2<R> b) {
    acc.x = rfma(a.x, b.x, rfma(-a.y, b.y, acc.x));
    acc.y = rfma(a.x, b.y, rfma(a.y, b.x, acc.y));
}
template <typename R>
__device__ __forceinline__ R warp_sum_r(R v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// T_0..T_{n-1} at x (Chebyshev.h:38-68)
template <typename R, int NT>
__device__ __forceinline__ void cheb_row(R x, R* T) {
    T[0] = R(1);
    if (NT > 1) T[1] = x;
#pragma unroll
    for (int i = 2; i < NT; ++i) T[i] = R(2) * x * T[i - 1] - T[i - 2];
}
// sum_a T_a(th) sum_q T_q(s) c[a*PS + q] (Interpolator.h:55-77, evaluated separably) with the
// Chebyshev rows given (shared by several right-hand sides).  T_0 = 1, so each inner sum starts
// from its q = 0 coefficient and the outer sum from its a = 0 term: the same sums in the same
// order as multiplying by T_0, with 2 PA + 2 fewer multiply-adds (the FP64 kernels are bound by
// them); only the sign of an exact zero can differ.
template <typename R, int PS, int PA>
__device__ __forceinline__ V2<R> interp_eval_tt(const V2<R>* __restrict__ c, const R* Ts, const R* Tt) {
    V2<R> r;
#pragma unroll
    for (int a = 0; a < PA; ++a) {
        V2<R> u = c[a * PS];
#pragma unroll
        for (int q = 1; q < PS; ++q) {
            const V2<R> v = c[a * PS + q];
            u.x = rfma(Ts[q], v.x, u.x); u.y = rfma(Ts[q], v.y, u.y);
        }
        if (a == 0) {
            r = u;
        } else {
            r.x = rfma(Tt[a], u.x, r.x); r.y = rfma(Tt[a], u.y, r.y);
        }
    }
    return r;
}
template <typename R, int PS, int PA>
__device__ __forceinline__ V2<R> interp_eval(const V2<R>* __restrict__ c, R s, R th) {
    R Ts[PS], Tt[PA];
    cheb_row<R, PS>(s, Ts);
    cheb_row<R, PA>(th, Tt);
    return interp_eval_tt<R, PS, PA>(c, Ts, Tt);
}

#define IFGF_DISPATCH_P(PS_, PA_, ...)                                              \
    if (PS_ == 5 && PA_ == 5) { constexpr int PS = 5, PA = 5; __VA_ARGS__; }        \
    else if (PS_ == 5 && PA_ == 7) { constexpr int PS = 5, PA = 7; __VA_ARGS__; }   \
    else if (PS_ == 3 && PA_ == 5) { constexpr int PS = 3, PA = 5; __VA_ARGS__; }   \
    else if (PS_ == 3 && PA_ == 3) { constexpr int PS = 3, PA = 3; __VA_ARGS__; }   \
    else if (PS_ == 7 && PA_ == 7) { constexpr int PS = 7, PA = 7; __VA_ARGS__; }   \
    else if (PS_ == 4 && PA_ == 4) { constexpr int PS = 4, PA = 4; __VA_ARGS__; }   \
    else if (PS_ == 6 && PA_ == 6) { constexpr int PS = 6, PA = 6; __VA_ARGS__; }

}  // namespace ifgf
