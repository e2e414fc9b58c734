"""CPU ORACLE — test infrastructure only.

ctypes front end of the C++ restatement of IFGF2D's forward map (oracle/*.hpp).
Only the tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module, always as the checker.  The product (``ifgf2d_gb300``) never imports it.

The geometry descriptors (``curve_circle`` ...) mirror Geometry/Curve.hpp:106-161.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

CURVE_CIRCLE, CURVE_KITE, CURVE_LINE, CURVE_STAR = 0, 1, 2, 3


def build(quiet: bool = True) -> str:
    """Compile the oracle shared library with the Makefile in this folder."""
    subprocess.run(["make", "-C", HERE], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        I64 = ctypes.POINTER(ctypes.c_longlong)
        I32 = ctypes.POINTER(ctypes.c_int)
        L.orc_hankel.argtypes = [ctypes.c_int, ctypes.c_longlong, D, D]
        L.orc_fm_create.restype = P
        L.orc_fm_create.argtypes = [ctypes.c_int, I32, I32, D, D, ctypes.c_int, I32, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.orc_fm_destroy.argtypes = [P]
        L.orc_fm_N.argtypes = [P]; L.orc_fm_N.restype = ctypes.c_longlong
        L.orc_fm_num_patches.argtypes = [P]; L.orc_fm_num_patches.restype = ctypes.c_longlong
        L.orc_fm_points.argtypes = [P, D, D, D, D]
        L.orc_fm_patch_info.argtypes = [P, D, I64]
        L.orc_fm_ns_lists.argtypes = [P, I64, D]
        L.orc_fm_point_weights.argtypes = [P, D, D]
        L.orc_fm_precompute.argtypes = [P, ctypes.c_double]
        L.orc_fm_precomp_matrix.argtypes = [P, ctypes.c_longlong, D]
        L.orc_fm_apply_unacc.argtypes = [P, D, D]
        L.orc_fm_apply_sing.argtypes = [P, D, D]
        L.orc_fm_setup_ifgf.argtypes = [P, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_fm_setup_ifgf.restype = ctypes.c_int
        L.orc_fm_last_error.argtypes = [P]; L.orc_fm_last_error.restype = ctypes.c_char_p
        L.orc_fm_sorting.argtypes = [P, I64]
        L.orc_fm_work.argtypes = [P, I64]
        L.orc_fm_level_stats.argtypes = [P, I64, I64]
        L.orc_fm_apply_acc.argtypes = [P, D, D]
        L.orc_fm_ifgf_far.argtypes = [P, D, D]
        L.orc_fm_direct_excluded.argtypes = [P, D, D, ctypes.c_longlong, ctypes.c_longlong]
        L.orc_fm_solve.argtypes = [P, D, D, ctypes.c_int, ctypes.c_double, ctypes.c_longlong,
                                   ctypes.c_longlong, I64, D, I64, ctypes.c_int]
        L.orc_fm_solve.restype = ctypes.c_int
        L.orc_fm_propagate.argtypes = [P, ctypes.c_longlong, D, D, D, D]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i64(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))


def _i32(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def hankel1(order: int, x) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(2 * x.size)
    lib().orc_hankel(order, x.size, _d(x), _d(out))
    return out[0::2] + 1j * out[1::2]


# ---- curve descriptors: (type, closed, tlim1, tlim2, params[16]) --------------------
def curve_circle(cx=0.0, cy=0.0, r=1.0):
    return (CURVE_CIRCLE, True, 0.0, 2 * np.pi, [cx, cy, r])


def curve_kite(A=1.0, B=0.65, C=-0.65, D=1.5):
    return (CURVE_KITE, True, 0.0, 2 * np.pi, [A, B, C, D])


def curve_line(x1, y1, x2, y2):
    return (CURVE_LINE, False, -1.0, 1.0, [x1, y1, x2, y2])


def curve_star(a, b, cx=0.0, cy=0.0):
    a = list(a); b = list(b)
    assert len(a) == len(b) <= 6
    return (CURVE_STAR, True, 0.0, 2 * np.pi, [cx, cy, float(len(a))] + a + b)


def pack_curves(curves):
    n = len(curves)
    types = np.array([c[0] for c in curves], dtype=np.int32)
    closed = np.array([1 if c[1] else 0 for c in curves], dtype=np.int32)
    tl = np.array([[c[2], c[3]] for c in curves], dtype=np.float64).ravel()
    params = np.zeros((n, 16))
    for i, c in enumerate(curves):
        params[i, :len(c[4])] = c[4]
    return types, closed, tl, params.ravel()


def _cvec(v):
    v = np.ascontiguousarray(v, dtype=np.complex128)
    return v.view(np.float64)


class OracleForwardMap:
    """CPU restatement of ForwardMap<Np, SingleLayer, Ps, Pang> (ForwardMap/ForwardMap.hpp:49-177)."""

    def __init__(self, curves, Np, delta, wavelengths_per_patch, split_k, p=4.0,
                 patches_per_curve=0, junctions=(), formulation="single_layer", coupling=0.0):
        L = lib()
        types, closed, tl, params = pack_curves(curves)
        j = np.array(junctions, dtype=np.int32).ravel() if junctions else np.zeros(3, np.int32)
        self.h = L.orc_fm_create(len(curves), _i32(types), _i32(closed), _d(tl), _d(params),
                                 len(junctions), _i32(j), Np, delta, wavelengths_per_patch,
                                 split_k, p, patches_per_curve,
                                 {"single_layer": 0, "combined": 2}[formulation], coupling)
        self.Np = Np
        self.N = L.orc_fm_N(self.h)
        self.num_patches = L.orc_fm_num_patches(self.h)
        self.k = None

    def __del__(self):
        try:
            lib().orc_fm_destroy(self.h)
        except Exception:
            pass

    def points(self):
        n = self.N
        xs, ys, nx, ny = (np.empty(n) for _ in range(4))
        lib().orc_fm_points(self.h, _d(xs), _d(ys), _d(nx), _d(ny))
        return xs, ys, nx, ny

    def patch_info(self):
        t = np.empty(2 * self.num_patches)
        c = np.empty(self.num_patches, dtype=np.int64)
        lib().orc_fm_patch_info(self.h, _d(t), _i64(c))
        return t.reshape(-1, 2), c

    def near_singular(self):
        t12, cnt = self.patch_info()
        tot = int(cnt.sum())
        idx = np.empty(max(tot, 1), dtype=np.int64)
        tv = np.empty(max(tot, 1))
        lib().orc_fm_ns_lists(self.h, _i64(idx), _d(tv))
        return cnt, idx[:tot], tv[:tot]

    def point_weights(self):
        w = np.empty(self.N); e = np.empty(self.N)
        lib().orc_fm_point_weights(self.h, _d(w), _d(e))
        return w, e

    def precompute(self, k):
        self.k = k
        lib().orc_fm_precompute(self.h, k)

    def precomp_matrix(self, p):
        _, cnt = self.patch_info()
        out = np.empty(2 * self.Np * (self.Np + int(cnt[p])))
        lib().orc_fm_precomp_matrix(self.h, p, _d(out))
        return (out[0::2] + 1j * out[1::2]).reshape(self.Np + int(cnt[p]), self.Np).T

    def _vec_op(self, fn, x):
        xin = _cvec(x)
        out = np.empty(2 * self.N)
        fn(self.h, _d(xin), _d(out))
        return out[0::2] + 1j * out[1::2]

    def compute_Ax_unacc(self, x):
        return self._vec_op(lib().orc_fm_apply_unacc, x)

    def sing_near_sing(self, x):
        return self._vec_op(lib().orc_fm_apply_sing, x)

    def setup_ifgf(self, k, nlevels, Ps=5, Pang=5):
        rc = lib().orc_fm_setup_ifgf(self.h, k, nlevels, Ps, Pang)
        if rc != 0:
            msg = lib().orc_fm_last_error(self.h).decode()
            raise RuntimeError(f"oracle IFGF set-up failed ({rc}): {msg}")
        self.nlevels = nlevels

    def compute_Ax_acc(self, x):
        return self._vec_op(lib().orc_fm_apply_acc, x)

    def ifgf_far(self, intensities):
        return self._vec_op(lib().orc_fm_ifgf_far, intensities)

    def direct_excluded(self, intensities, rows=None):
        r0, r1 = (0, self.N) if rows is None else rows
        xin = _cvec(intensities)
        out = np.empty(2 * (r1 - r0))
        lib().orc_fm_direct_excluded(self.h, _d(xin), _d(out), r0, r1)
        return out[0::2] + 1j * out[1::2]

    def sorting(self):
        s = np.empty(self.N, dtype=np.int64)
        lib().orc_fm_sorting(self.h, _i64(s))
        return s

    def work(self):
        c = np.empty(6, dtype=np.int64)
        lib().orc_fm_work(self.h, _i64(c))
        keys = ["near_pairs", "leaf_evals", "prop_evals", "interp_evals", "cones", "cone_levels"]
        return dict(zip(keys, (int(v) for v in c)))

    def level_stats(self):
        b = np.zeros(self.nlevels, dtype=np.int64); c = np.zeros(self.nlevels, dtype=np.int64)
        lib().orc_fm_level_stats(self.h, _i64(b), _i64(c))
        return b, c

    def solve(self, rhs, accelerated, tol=1e-10, restart=300, maxit=300, exact_adjoint=False):
        """Householder GMRES (opGMRES.hpp:68-269); exact_adjoint selects the minimal-residual variant."""
        r = _cvec(rhs)
        x = np.empty(2 * self.N)
        it = np.zeros(1, dtype=np.int64); mv = np.zeros(1, dtype=np.int64); err = np.zeros(1)
        rc = lib().orc_fm_solve(self.h, _d(r), _d(x), 1 if accelerated else 0, tol, restart, maxit,
                                _i64(it), _d(err), _i64(mv), 1 if exact_adjoint else 0)
        return x[0::2] + 1j * x[1::2], dict(rc=rc, iters=int(it[0]), error=float(err[0]), matvecs=int(mv[0]))

    def propagate_unacc(self, xp, yp, density):
        xp = np.ascontiguousarray(xp, dtype=np.float64); yp = np.ascontiguousarray(yp, dtype=np.float64)
        d = _cvec(density)
        out = np.empty(2 * xp.size)
        lib().orc_fm_propagate(self.h, xp.size, _d(xp), _d(yp), _d(d), _d(out))
        return out[0::2] + 1j * out[1::2]


def mt19937_uniform(n: int, seed: int = 0) -> np.ndarray:
    """U[0,1) doubles from raw 32-bit mt19937(seed) words: u = w / 2^32.

    std::uniform_real_distribution output is implementation-defined, so the seeded
    densities of IFGF_Source/main.cpp:150-175 are regenerated from raw words.
    numpy's MT19937 is seeded with `_legacy_seeding`, which matches std::mt19937(seed).
    """
    bg = np.random.MT19937(0)
    bg._legacy_seeding(seed)
    words = np.random.Generator(bg).bit_generator.random_raw(n).astype(np.uint64)
    return (words & 0xFFFFFFFF).astype(np.float64) / 4294967296.0


def seeded_density(n: int, seed: int = 0) -> np.ndarray:
    u = mt19937_uniform(2 * n, seed)
    return u[0::2] + 1j * u[1::2]
