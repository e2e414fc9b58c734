"""ifgf2d_gb300 -- GB300-native forward map of IFGF2D (2D Helmholtz boundary integral operator).

Python mirror of the reference's C++ interface for the matvec that GMRES calls:

* ``ForwardMap``      -- ForwardMap<Np, SingleLayer, Ps, Pang> (ForwardMap/ForwardMap.hpp:49-177):
                         constructor (discretisation), ``compute_precomputations``,
                         ``precomps_and_setup``, ``compute_Ax_unacc`` / ``compute_Ax_acc``,
                         ``solve``, ``propagate_unacc`` and the public arrays ``xs_`` ... ``nys_``.
* ``LinearOperator``  -- ForwardMap/LinearOperator.hpp:27-58 (rows, cols, mapping, ``A * x``).
* curve constructors  -- Geometry/Curve.hpp:106-161 (``Circle``, ``Kite``, ``Line``) plus ``Star``.

All arithmetic runs in libifgf2d.so (C++ host + sm_103a CUDA kernels, include/ifgf2d.h).  The
reference throws std::logic_error / std::invalid_argument; these bindings raise the Python
equivalents (``RuntimeError`` subclasses below, ``ValueError`` for bad arguments).
"""
from __future__ import annotations

import ctypes
import math
import numpy as np

from . import _lib
from ._lib import APPLY_DIRECT, APPLY_IFGF, APPLY_IFGF_MIXED, PRECOND_NET, PRECOND_SPECTRAL

__all__ = ["ForwardMap", "LinearOperator", "Circle", "Kite", "Line", "Star", "Junction", "hankel1", "Group",
           "IFGF2DError", "NeighbourhoodError", "NoConvergence", "load_library"]


class IFGF2DError(RuntimeError):
    """Error status from libifgf2d (the reference throws std::logic_error)."""


class NeighbourhoodError(IFGF2DError):
    """A singular / near-singular point lies outside the leaf neighbourhood (BoxTree.h:1112-1153)."""


class NoConvergence(IFGF2DError):
    """GMRES stopped at max_iters before reaching the tolerance (Eigen NoConvergence)."""


def load_library():
    return _lib.load()


def _check(rc, ctx=None):
    if rc == 0:
        return
    msg = _lib.load().ifgf2d_last_error(ctx).decode() if ctx else ""
    name = _lib.STATUS.get(rc, str(rc))
    if rc == 1:
        raise ValueError(f"ifgf2d: {name}: {msg}")
    if rc == 3:
        raise NeighbourhoodError(f"ifgf2d: {name}: {msg}")
    raise IFGF2DError(f"ifgf2d: {name}: {msg}")


def seeded_density(n, seed=0):
    """Seeded benchmark density rho_j = u_{2j} + i u_{2j+1}, u = w / 2^32 from the raw words w
    of std::mt19937(seed) (the reference's benchmark densities, IFGF_Source/main.cpp:150-160,
    with an independent imaginary part).  numpy's MT19937 with legacy seeding is std::mt19937."""
    bg = np.random.MT19937(0)
    bg._legacy_seeding(seed)
    w = bg.random_raw(2 * n).astype(np.uint64) & 0xFFFFFFFF
    u = w.astype(np.float64) / 4294967296.0
    return u[0::2] + 1j * u[1::2]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _cview(x, n=None):
    x = np.ascontiguousarray(x, dtype=np.complex128)
    if n is not None and x.shape != (n,):
        raise ValueError(f"expected a vector of {n} complex values, got shape {x.shape}")
    return x


# ---------------------------------------------------------------- curves
def _curve(kind, closed, t1, t2, params):
    c = _lib.Curve()
    c.type, c.closed, c.tlim1, c.tlim2 = kind, 1 if closed else 0, float(t1), float(t2)
    for i, v in enumerate(params):
        c.params[i] = float(v)
    return c


def Circle(centerx=0.0, centery=0.0, radius=1.0):
    """Geometry/Curve.hpp:106-125 (parametrised on [0, 2 pi])."""
    return _curve(_lib.CURVE_CIRCLE, True, 0.0, 2 * math.pi, [centerx, centery, radius])


def Kite(A=1.0, B=0.65, C=-0.65, D=1.5):
    """Geometry/Curve.hpp:128-146: x = A cos t + B cos 2t + C, y = D sin t."""
    return _curve(_lib.CURVE_KITE, True, 0.0, 2 * math.pi, [A, B, C, D])


def Line(x1, y1, x2, y2):
    """Geometry/Curve.hpp:148-161: open segment on t in [-1, 1]."""
    return _curve(_lib.CURVE_LINE, False, -1.0, 1.0, [x1, y1, x2, y2])


def Star(a, b, centerx=0.0, centery=0.0):
    """Star-shaped curve r(t) = 1 + sum_m a_m cos mt + b_m sin mt (m <= 6; not in the reference)."""
    a = list(a); b = list(b)
    if len(a) != len(b) or len(a) > 6:
        raise ValueError("Star: a and b must have the same length <= 6")
    return _curve(_lib.CURVE_STAR, True, 0.0, 2 * math.pi, [centerx, centery, len(a)] + a + b)


def Junction(curve, touching_curve, t1_touches_t1):
    """Geometry/Curve.hpp:10-17 (with the owning curve index made explicit)."""
    j = _lib.Junction()
    j.curve, j.touching_curve, j.t1_touches_t1 = curve, touching_curve, 1 if t1_touches_t1 else 0
    return j


def hankel1(order: int, x) -> np.ndarray:
    """H_order^(1)(x) for real x > 0 on the GPU (device evaluator; replaces sp_bessel::hankelH1)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(2 * x.size)
    _check(_lib.load().ifgf2d_hankel(order, x.size, _dp(x), _dp(out)))
    return out[0::2] + 1j * out[1::2]


# ---------------------------------------------------------------- LinearOperator
class LinearOperator:
    """ForwardMap/LinearOperator.hpp:43-58: an operator defined by a mapping(x, out) callable."""

    def __init__(self, rows, cols, mapping):
        self._rows, self._cols, self.mapping_ = int(rows), int(cols), mapping

    def rows(self):
        return self._rows

    def cols(self):
        return self._cols

    def __mul__(self, x):
        out = np.empty(self._rows, dtype=np.complex128)
        self.mapping_(x, out)
        return out


# ---------------------------------------------------------------- ForwardMap
class ForwardMap:
    """ForwardMap<Np, SingleLayer, Ps, Pang> on one GB300.

    ForwardMap(delta, curves, curve_touch_tracker, wavelengths_per_patch, patch_split_wavenumber, p=4)
    with ``Np``, ``Ps``, ``Pang`` given as keyword arguments (template parameters in C++).
    ``patches_per_curve > 0`` selects an equal-parameter split instead of the arc-length rule.
    ``formulation="combined"`` selects the sound-soft combined field operator (1/2 I + K - i eta S)
    with eta = ``coupling`` (eta = k when coupling <= 0); the default is the reference's single layer.
    ``device_geometry=True`` computes the points, patch bounding boxes and near-singular points on
    the GPU (the patch limits stay on the host).
    """

    def __init__(self, delta, curves, curve_touch_tracker=(), wavelengths_per_patch=1.0,
                 patch_split_wavenumber=1.0, p=4.0, *, Np=10, Ps=5, Pang=5, patches_per_curve=0,
                 formulation="single_layer", coupling=0.0, device_geometry=False):
        L = _lib.load()
        curves = list(curves)
        if not curves:
            raise ValueError("ForwardMap needs at least one curve")
        carr = (_lib.Curve * len(curves))(*curves)
        jl = list(curve_touch_tracker)
        jarr = (_lib.Junction * max(len(jl), 1))(*jl) if jl else None
        forms = {"single_layer": _lib.SINGLE_LAYER, "combined": _lib.COMBINED}
        if formulation not in forms:
            raise ValueError(f"formulation must be one of {sorted(forms)}")
        opt = _lib.Options(Np, delta, wavelengths_per_patch, patch_split_wavenumber, p, patches_per_curve, Ps, Pang,
                           forms[formulation], float(coupling), 1 if device_geometry else 0)
        self.formulation = formulation
        h = ctypes.c_void_p()
        rc = L.ifgf2d_create(carr, len(curves), jarr, len(jl), ctypes.byref(opt), ctypes.byref(h))
        self._h = h.value
        if rc != 0:
            msg = L.ifgf2d_last_error(self._h).decode() if self._h else ""
            if self._h:
                L.ifgf2d_destroy(self._h)
                self._h = None
            if rc == 2:
                raise ValueError(f"ifgf2d_create: {msg}")
            _check(rc)
        self.Np, self.Ps, self.Pang = Np, Ps, Pang
        self.delta_, self.p_ = delta, p
        self.total_num_unknowns_ = int(L.ifgf2d_num_unknowns(self._h))
        self.num_patches_ = int(L.ifgf2d_num_patches(self._h))
        n = self.total_num_unknowns_
        self.xs_, self.ys_, self.nxs_, self.nys_ = (np.empty(n) for _ in range(4))
        _check(L.ifgf2d_get_points(self._h, _dp(self.xs_), _dp(self.ys_), _dp(self.nxs_), _dp(self.nys_)), self._h)
        self.GMRES_MAX_ITER_ = 300
        self.GMRES_TOLERANCE_ = 1e-10
        self.wavenumber = None
        self.nlevels = None

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            _lib.load().ifgf2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- geometry queries
    def patches(self):
        """(num_patches, 2) patch limits and the near-singular point count per patch."""
        t = np.empty(2 * self.num_patches_)
        c = np.empty(self.num_patches_, dtype=np.int64)
        _check(_lib.load().ifgf2d_get_patches(self._h, _dp(t), c.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))), self._h)
        return t.reshape(-1, 2), c

    def near_singular(self):
        """(counts per patch, concatenated point indices, concatenated Brent t values)."""
        _, cnt = self.patches()
        tot = int(cnt.sum())
        idx = np.empty(max(tot, 1), dtype=np.int64)
        t = np.empty(max(tot, 1))
        _check(_lib.load().ifgf2d_get_near_singular(self._h, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), _dp(t)), self._h)
        return cnt, idx[:tot], t[:tot]

    # -- set-up
    def compute_precomputations(self, wavenumber):
        """ForwardMap.tpp:391-423 (rectangular-polar weights, computed on the GPU)."""
        _check(_lib.load().ifgf2d_precompute(self._h, float(wavenumber)), self._h)
        self.wavenumber = float(wavenumber)
        self._setup_serial = getattr(self, "_setup_serial", 0) + 1   # invalidates evaluation plans

    def precomputations(self, patch):
        """Patch.hpp:55 precomputations_: Np x (Np + n_ns) complex matrix of one patch."""
        _, cnt = self.patches()
        ncol = self.Np + int(cnt[patch])
        out = np.empty(2 * self.Np * ncol)
        _check(_lib.load().ifgf2d_get_precomputations(self._h, int(patch), _dp(out)), self._h)
        return (out[0::2] + 1j * out[1::2]).reshape(ncol, self.Np).T

    def precomps_and_setup(self, wavenumber, nlevels=0):
        """ForwardMap.tpp:542-565; nlevels <= 0 picks the deepest tree that passes the neighbourhood check."""
        _check(_lib.load().ifgf2d_setup(self._h, float(wavenumber), int(nlevels)), self._h)
        self.wavenumber = float(wavenumber)
        self._setup_serial = getattr(self, "_setup_serial", 0) + 1   # invalidates evaluation plans
        self.nlevels = int(_lib.load().ifgf2d_get_nlevels(self._h))

    def prepare(self, wavenumber, nlevels=0):
        """The host part of precomps_and_setup (tree depth, tree, plans) with no GPU call, for
        a host thread that prepares contexts while the GPU serves others."""
        _check(_lib.load().ifgf2d_prepare(self._h, float(wavenumber), int(nlevels)), self._h)

    def get_tuning(self):
        """the context's launch-shape table (ifgf2d_get_tuning)"""
        L = _lib.load()
        c = np.zeros(int(L.ifgf2d_tuning_size()), dtype=np.int32)
        _check(L.ifgf2d_get_tuning(self._h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), self._h)
        return c

    def set_tuning(self, table):
        L = _lib.load()
        c = np.ascontiguousarray(table, dtype=np.int32)
        if c.size != int(L.ifgf2d_tuning_size()):
            raise ValueError(f"a tuning table has {int(L.ifgf2d_tuning_size())} entries, got {c.size}")
        _check(L.ifgf2d_set_tuning(self._h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), self._h)

    BATCH_TC_LEAF = 1
    BATCH_TC_PROPAGATION = 2
    BATCH_TC_LEAF_FP32 = 4
    BATCH_BULK_PROPAGATION = 8
    BATCH_GROUPED_INTERP = 16
    SINGLE_INTERP_BY_BOX_FP64 = 32
    SINGLE_INTERP_BY_BOX_C64 = 64

    _BATCH_BITS = 31

    @property
    def batch_tensor_cores(self):
        """bit mask of the batched complex64 kernel choices (BATCH_*: tcgen05 3xTF32 leaf and
        propagation, bulk-copy propagation, grouped interpolation).  They share the last entry
        of the tuning table with the single-vector choices (SINGLE_INTERP_BY_BOX_*), which this
        property leaves alone."""
        return int(self.get_tuning()[-1]) & self._BATCH_BITS

    @batch_tensor_cores.setter
    def batch_tensor_cores(self, mask):
        c = self.get_tuning()
        c[-1] = (int(c[-1]) & ~self._BATCH_BITS) | (int(mask) & self._BATCH_BITS)
        self.set_tuning(c)

    def autotune(self, reps=5, cache=True, cache_dir=None):
        """Pick the launch shapes of the leaf and per-level propagation kernels by timing them on
        this problem (ifgf2d_autotune).  With cache, the choice is stored on disk, keyed by the GPU
        and the problem signature, and reused without timing.  Returns the tuning table."""
        import json
        import os
        L = _lib.load()
        n = int(L.ifgf2d_tuning_size())
        c = np.zeros(n, dtype=np.int32)
        cp = c.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        key = path = None
        if cache:
            try:
                import torch
                dev = torch.cuda.get_device_name(torch.cuda.current_device())
            except Exception:
                dev = "gpu"
            wc = self.work_counts()
            # "v3": the variant set with the staged propagation and the interpolation by leaf box
            key = f"v3|{dev}|N={self.total_num_unknowns_}|k={self.wavenumber:.17g}|P={self.Ps}x{self.Pang}|" \
                  f"nl={self.nlevels}|cones={wc['cones']}|prop={wc['prop_evals']}"
            d = cache_dir or os.environ.get("IFGF2D_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "ifgf2d_gb300")
            path = os.path.join(d, "tuning.json")
            try:
                table = json.load(open(path))
            except Exception:
                table = {}
            if key in table and len(table[key]) == n:
                c[:] = table[key]
                _check(L.ifgf2d_set_tuning(self._h, cp), self._h)
                return c.copy()
        _check(L.ifgf2d_autotune(self._h, int(reps), cp), self._h)
        if cache:
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                try:
                    table = json.load(open(path))
                except Exception:
                    table = {}
                table[key] = [int(v) for v in c]
                with open(path, "w") as f:
                    json.dump(table, f, indent=0)
            except OSError:
                pass
        return c.copy()

    def getSorting(self):
        s = np.empty(self.total_num_unknowns_, dtype=np.int64)
        _check(_lib.load().ifgf2d_get_sorting(self._h, s.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))), self._h)
        return s

    def work_counts(self):
        c = np.zeros(8, dtype=np.int64)
        _check(_lib.load().ifgf2d_work_counts(self._h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))), self._h)
        keys = ["near_pairs", "leaf_evals", "prop_evals", "interp_evals", "cones", "nlevels", "sing_entries", "resident_bytes"]
        return dict(zip(keys, (int(v) for v in c)))

    # -- the matvec
    def _apply(self, x, mode):
        n = self.total_num_unknowns_
        xin = _cview(x, n)
        out = np.empty(n, dtype=np.complex128)
        _check(_lib.load().ifgf2d_apply(self._h, _dp(xin.view(np.float64)), _dp(out.view(np.float64)), mode), self._h)
        return out

    def compute_Ax_unacc(self, density, out=None, wavenumber=None):
        """ForwardMap.tpp:517-540: singular correction + direct O(N^2) far sum.

        The operator belongs to the wavenumber of the last precomputation; a ``wavenumber``
        other than that one raises ValueError (the reference would mix the two)."""
        if wavenumber is not None and float(wavenumber) != self.wavenumber:
            raise ValueError(f"compute_Ax_unacc: wavenumber {wavenumber} differs from the precomputed {self.wavenumber}")
        y = self._apply(density, APPLY_DIRECT)
        if out is not None:
            out[...] = y
        return y

    def compute_Ax_acc(self, density, out=None, mixed=False):
        """ForwardMap.tpp:609-655: singular correction + IFGF far sum (BoxTree::Solve).

        mixed=True evaluates the IFGF far field in complex64 (FP32 arithmetic on tables
        computed in FP64); the singular correction stays FP64.
        """
        y = self._apply(density, APPLY_IFGF_MIXED if mixed else APPLY_IFGF)
        if out is not None:
            out[...] = y
        return y

    def ifgf_far(self, intensities):
        """BoxTree::Solve on given intensities (IFGF_Source/BoxTree.h:1020-1071)."""
        n = self.total_num_unknowns_
        xin = _cview(intensities, n)
        out = np.empty(n, dtype=np.complex128)
        _check(_lib.load().ifgf2d_ifgf_far(self._h, _dp(xin.view(np.float64)), _dp(out.view(np.float64))), self._h)
        return out

    def apply_device(self, d_x, d_y, accelerated=True, mixed=False):
        """y = A x on device pointers (ints or objects with data_ptr(); N complex128 each).

        Work is queued on the context's stream (``stream()``); synchronise before reading y.
        """
        px = d_x.data_ptr() if hasattr(d_x, "data_ptr") else int(d_x)
        py = d_y.data_ptr() if hasattr(d_y, "data_ptr") else int(d_y)
        mode = (APPLY_IFGF_MIXED if mixed else APPLY_IFGF) if accelerated else APPLY_DIRECT
        _check(_lib.load().ifgf2d_apply_device(self._h, px, py, mode), self._h)

    def stream(self):
        return _lib.load().ifgf2d_stream(self._h)

    # -- many right-hand sides
    def _batch_in(self, X):
        n = self.total_num_unknowns_
        X = np.asarray(X, dtype=np.complex128)
        if X.ndim == 1:
            X = X[:, None]
        if X.shape[0] != n:
            raise ValueError(f"expected an ({n}, nrhs) matrix, got {X.shape}")
        return np.asfortranarray(X)

    def apply_batch(self, X, accelerated=True, mixed=False):
        """Y = A X for the columns of an (N, nrhs) matrix in one pass over the operator's tables
        (the reference applies LinearOperator::operator* once per column)."""
        Xf = self._batch_in(X)
        Y = np.empty_like(Xf, order="F")
        mode = (APPLY_IFGF_MIXED if mixed else APPLY_IFGF) if accelerated else APPLY_DIRECT
        _check(_lib.load().ifgf2d_apply_batch(self._h, _dp(Xf), _dp(Y), Xf.shape[1], mode),
               self._h)
        return Y

    def apply_batch_device(self, d_x, d_y, nrhs, accelerated=True, mixed=False):
        """Batched apply on device pointers: column-major N x nrhs complex128 matrices."""
        px = d_x.data_ptr() if hasattr(d_x, "data_ptr") else int(d_x)
        py = d_y.data_ptr() if hasattr(d_y, "data_ptr") else int(d_y)
        mode = (APPLY_IFGF_MIXED if mixed else APPLY_IFGF) if accelerated else APPLY_DIRECT
        _check(_lib.load().ifgf2d_apply_batch_device(self._h, px, py, int(nrhs), mode), self._h)

    def gmres_batch(self, B, accelerated=True, tol=None, restart=None, max_iters=None, raise_on_noconv=False, mixed=False,
                    precond=None):
        """GMRES for every column of an (N, nrhs) matrix, all columns in lock step on the batched
        operator; ``self.last_solve`` holds per-column iterations and errors.  precond="spectral":
        flexible GMRES with the spectral right preconditioner (IFGF operators only)."""
        if precond not in (None, "spectral"):
            raise ValueError("batched solves take precond=None or 'spectral'")
        Bf = self._batch_in(B)
        X = np.empty_like(Bf, order="F")
        nrhs = Bf.shape[1]
        it = np.zeros(nrhs, dtype=np.int32)
        err = np.zeros(nrhs, dtype=np.float64)
        tol = self.GMRES_TOLERANCE_ if tol is None else tol
        restart = self.GMRES_MAX_ITER_ if restart is None else restart
        max_iters = self.GMRES_MAX_ITER_ if max_iters is None else max_iters
        mode = (APPLY_IFGF_MIXED if mixed else APPLY_IFGF) if accelerated else APPLY_DIRECT
        if precond == "spectral":
            rc = _lib.load().ifgf2d_solve_batch_flexible(self._h, PRECOND_SPECTRAL, _dp(Bf), _dp(X), nrhs, mode, float(tol),
                                                         int(restart), int(max_iters),
                                                         it.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(err))
        else:
            rc = _lib.load().ifgf2d_solve_batch(self._h, _dp(Bf), _dp(X), nrhs, mode,
                                                float(tol), int(restart), int(max_iters),
                                                it.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(err))
        self.last_solve = dict(iters=it.tolist(), error=err.tolist(), converged=(rc == 0),
                               refinements=int(_lib.load().ifgf2d_last_refinements(self._h)) if mixed else 0)
        if rc == 8:
            if raise_on_noconv:
                raise NoConvergence(f"GMRES: iterations {it.tolist()}, estimated errors {err.tolist()}")
        else:
            _check(rc, self._h)
        return X

    # -- solver
    def solve(self, rhs, wavenumber, nlevels=0, accelerated=True, tol=None, restart=None, max_iters=None,
              raise_on_noconv=False, mixed=False):
        """ForwardMap.tpp:658-697: set-up, then GMRES (initial guess 0) on the device.

        Returns the density; ``self.last_solve`` holds iterations and the estimated error.
        """
        if accelerated:
            self.precomps_and_setup(wavenumber, nlevels)
        else:
            self.compute_precomputations(wavenumber)
        return self.gmres(rhs, accelerated, tol, restart, max_iters, raise_on_noconv, mixed)

    def gmres(self, rhs, accelerated=True, tol=None, restart=None, max_iters=None, raise_on_noconv=False, mixed=False):
        """Device GMRES; mixed=True: FP64 iterative refinement around complex64 inner solves
        (stop test on the FP64 relative residual)."""
        n = self.total_num_unknowns_
        b = _cview(rhs, n)
        x = np.empty(n, dtype=np.complex128)
        it = ctypes.c_int(0)
        err = ctypes.c_double(0.0)
        tol = self.GMRES_TOLERANCE_ if tol is None else tol
        restart = self.GMRES_MAX_ITER_ if restart is None else restart
        max_iters = self.GMRES_MAX_ITER_ if max_iters is None else max_iters
        rc = _lib.load().ifgf2d_solve(self._h, _dp(b.view(np.float64)), _dp(x.view(np.float64)),
                                      (APPLY_IFGF_MIXED if mixed else APPLY_IFGF) if accelerated else APPLY_DIRECT,
                                      float(tol), int(restart),
                                      int(max_iters), ctypes.byref(it), ctypes.byref(err))
        self.last_solve = dict(iters=it.value, error=err.value, converged=(rc == 0),
                               refinements=int(_lib.load().ifgf2d_last_refinements(self._h)) if (mixed and accelerated) else 0)
        if rc == 8:
            if raise_on_noconv:
                raise NoConvergence(f"GMRES: {it.value} iterations, estimated error {err.value:.3e}")
        else:
            _check(rc, self._h)
        return x

    def geometry_features(self):
        """(N, 4): curvature, unit tangent x, y and quadrature weight per point (patch order), the
        geometry the learned preconditioner reads"""
        g = np.empty((self.total_num_unknowns_, 4))
        _check(_lib.load().ifgf2d_get_geometry_features(self._h, _dp(g)), self._h)
        return g

    def solve_precond(self, net, rhs, accelerated=True, tol=None, restart=None, max_iters=None, mixed=False,
                      raise_on_noconv=False):
        """GMRES with the learned right preconditioner (flexible GMRES inside FP64 iterative
        refinement, plain GMRES after a stall); ``net`` is a learned.PreconditionerNet."""
        n = self.total_num_unknowns_
        b = _cview(rhs, n)
        x = np.empty(n, dtype=np.complex128)
        it = ctypes.c_int(0)
        err = ctypes.c_double(0.0)
        tol = self.GMRES_TOLERANCE_ if tol is None else tol
        restart = self.GMRES_MAX_ITER_ if restart is None else restart
        max_iters = self.GMRES_MAX_ITER_ if max_iters is None else max_iters
        mode = (APPLY_IFGF_MIXED if mixed else APPLY_IFGF) if accelerated else APPLY_DIRECT
        rc = _lib.load().ifgf2d_solve_precond(self._h, net.handle, _dp(b.view(np.float64)), _dp(x.view(np.float64)), mode,
                                              float(tol), int(restart), int(max_iters), ctypes.byref(it), ctypes.byref(err))
        self.last_solve = dict(iters=it.value, error=err.value, converged=(rc == 0))
        if rc == 8:
            if raise_on_noconv:
                raise NoConvergence(f"FGMRES: {it.value} iterations, error {err.value:.3e}")
        else:
            _check(rc, self._h)
        return x

    def solve_preconditioned(self, rhs, wavenumber, nlevels=0, tol=None, restart=None, max_iters=None, raise_on_noconv=False):
        """ForwardMap.solve in the chosen form (not in the reference): set-up, then complex64 inner
        solves inside FP64 iterative refinement with the spectral right preconditioner (flexible
        GMRES).  Combined formulation, closed curves; the same answer within the tolerance."""
        self.precomps_and_setup(wavenumber, nlevels)
        return self.solve_flexible(rhs, "spectral", tol=tol, restart=restart, max_iters=max_iters, mixed=True,
                                   raise_on_noconv=raise_on_noconv)

    def spectral_setup(self, scale=None):
        """Tables of the spectral right preconditioner (combined field, closed curves): the
        flat-boundary symbol's inverse along each curve, glancing damping eps = scale k^(1/3)
        (default IFGF2D_SPECTRAL_DEFAULT_SCALE).  After precompute."""
        _check(_lib.load().ifgf2d_spectral_setup(self._h, 0.0 if scale is None else float(scale)), self._h)

    def spectral_apply(self, r):
        """z = M r with the spectral preconditioner (host vectors)"""
        return self.spectral_symbol(r, "preconditioner")

    def spectral_symbol(self, r, which="preconditioner"):
        """z = Op(m) r along the curves with the spectral tables: m = the preconditioner's
        1/sigma ("preconditioner"), the flat symbol's magnitude |sigma| ("magnitude") or its
        inverse ("inverse_magnitude")"""
        kinds = {"preconditioner": 0, "magnitude": 1, "inverse_magnitude": 2}
        n = self.total_num_unknowns_
        rin = _cview(r, n)
        z = np.empty(n, dtype=np.complex128)
        _check(_lib.load().ifgf2d_spectral_symbol(self._h, kinds[which], _dp(rin.view(np.float64)), _dp(z.view(np.float64))),
               self._h)
        return z

    def solve_flexible(self, rhs, precond="spectral", net=None, accelerated=True, tol=None, restart=None, max_iters=None,
                       mixed=False, raise_on_noconv=False):
        """Flexible GMRES inside FP64 iterative refinement with a right preconditioner:
        ``precond`` "spectral", "net" (``net`` a learned.PreconditionerNet) or "spectral+net" (the
        network's correction on top of the spectral preconditioner)."""
        kinds = {"net": PRECOND_NET, "spectral": PRECOND_SPECTRAL, "spectral+net": PRECOND_NET | PRECOND_SPECTRAL}
        if precond not in kinds:
            raise ValueError(f"precond must be one of {sorted(kinds)}")
        n = self.total_num_unknowns_
        b = _cview(rhs, n)
        x = np.empty(n, dtype=np.complex128)
        it = ctypes.c_int(0)
        err = ctypes.c_double(0.0)
        tol = self.GMRES_TOLERANCE_ if tol is None else tol
        restart = self.GMRES_MAX_ITER_ if restart is None else restart
        max_iters = self.GMRES_MAX_ITER_ if max_iters is None else max_iters
        mode = (APPLY_IFGF_MIXED if mixed else APPLY_IFGF) if accelerated else APPLY_DIRECT
        rc = _lib.load().ifgf2d_solve_flexible(self._h, net.handle if net is not None else None, kinds[precond],
                                               _dp(b.view(np.float64)), _dp(x.view(np.float64)), mode, float(tol), int(restart),
                                               int(max_iters), ctypes.byref(it), ctypes.byref(err))
        self.last_solve = dict(iters=it.value, error=err.value, converged=(rc == 0),
                               refinements=int(_lib.load().ifgf2d_last_refinements(self._h)))
        if rc == 8:
            if raise_on_noconv:
                raise NoConvergence(f"FGMRES: {it.value} iterations, error {err.value:.3e}")
        else:
            _check(rc, self._h)
        return x

    def linear_operator(self, accelerated=True):
        """LinearOperator wrapping compute_Ax_acc / compute_Ax_unacc, as ForwardMap::solve builds it."""
        f = self.compute_Ax_acc if accelerated else self.compute_Ax_unacc
        return LinearOperator(self.total_num_unknowns_, self.total_num_unknowns_, lambda x, out: f(x, out))

    def propagate_acc(self, x_prop, y_prop, density):
        """The off-surface field of ``density`` at (x_prop, y_prop) with the IFGF: the accelerated
        counterpart of propagate_unacc (ForwardMap.tpp:701-727), within the IFGF tolerance of it.
        Needs precomps_and_setup; the evaluation plan is kept for repeated calls on the same
        points."""
        xp = np.ascontiguousarray(x_prop, dtype=np.float64).ravel()
        yp = np.ascontiguousarray(y_prop, dtype=np.float64).ravel()
        if xp.shape != yp.shape:
            raise ValueError("x_prop and y_prop must have the same length")
        L = _lib.load()
        key = (getattr(self, "_setup_serial", 0), xp.tobytes(), yp.tobytes())
        if getattr(self, "_eval_key", None) != key:
            _check(L.ifgf2d_eval_offsurface_setup(self._h, xp.size, _dp(xp), _dp(yp)), self._h)
            self._eval_key = key
        d = _cview(density, self.total_num_unknowns_)
        out = np.empty(xp.size, dtype=np.complex128)
        _check(L.ifgf2d_eval_offsurface(self._h, _dp(d.view(np.float64)), _dp(out.view(np.float64))), self._h)
        return out

    def propagate_acc_counts(self):
        c = np.zeros(4, dtype=np.int64)
        _check(_lib.load().ifgf2d_eval_offsurface_counts(self._h, c.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))), self._h)
        return dict(zip(["near_pairs", "leaf_evals", "prop_evals", "interp_evals"], (int(v) for v in c)))

    def propagate_unacc(self, x_prop, y_prop, density, wavenumber=None):
        """ForwardMap.tpp:701-727: direct evaluation of the layer potential off the surface."""
        if wavenumber is not None and self.wavenumber != float(wavenumber):
            self.compute_precomputations(wavenumber)
        xp = np.ascontiguousarray(x_prop, dtype=np.float64)
        yp = np.ascontiguousarray(y_prop, dtype=np.float64)
        if xp.shape != yp.shape:
            raise ValueError("x_prop and y_prop must have the same length")
        d = _cview(density, self.total_num_unknowns_)
        out = np.empty(xp.size, dtype=np.complex128)
        _check(_lib.load().ifgf2d_propagate(self._h, xp.size, _dp(xp), _dp(yp), _dp(d.view(np.float64)),
                                            _dp(out.view(np.float64))), self._h)
        return out


# ---------------------------------------------------------------- many obstacles
class Group:
    """Many obstacles as one block-diagonal operator (ifgf2d_group_*): the prepared ForwardMaps
    ``members`` (ForwardMap.prepare(k): each its own wavenumber and tree; the same Np, Ps, Pang
    and formulation) merged so that each phase of the set-up and of an apply is one launch over
    all of them.  Vectors hold every member's unknowns in member order; ``offsets`` gives each
    member's first unknown.  The members may be closed afterwards."""

    def __init__(self, members):
        L = _lib.load()
        members = list(members)
        if not members:
            raise ValueError("a group needs at least one member")
        arr = (ctypes.c_void_p * len(members))(*[m.handle for m in members])
        h = ctypes.c_void_p()
        rc = L.ifgf2d_group_create(arr, len(members), ctypes.byref(h))
        self._h = h.value
        if rc != 0:
            msg = L.ifgf2d_group_last_error(self._h).decode() if self._h else ""
            self.close()
            raise (ValueError if rc == 1 else IFGF2DError)(f"ifgf2d_group_create: {_lib.STATUS.get(rc, rc)}: {msg}")
        self.n = len(members)
        self.N = int(L.ifgf2d_group_num_unknowns(self._h))
        off = np.zeros(self.n + 1, dtype=np.int64)
        L.ifgf2d_group_offsets(self._h, off.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
        self.offsets = off

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().ifgf2d_group_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc == 0:
            return
        msg = _lib.load().ifgf2d_group_last_error(self._h).decode()
        raise (ValueError if rc == 1 else IFGF2DError)(f"ifgf2d group: {_lib.STATUS.get(rc, rc)}: {msg}")

    def split(self, v):
        """the per-member pieces of a group vector"""
        return [v[self.offsets[o]:self.offsets[o + 1]] for o in range(self.n)]

    def apply(self, x, mixed=False):
        xin = _cview(x, self.N)
        out = np.empty(self.N, dtype=np.complex128)
        self._check(_lib.load().ifgf2d_group_apply(self._h, _dp(xin.view(np.float64)), _dp(out.view(np.float64)),
                                                   APPLY_IFGF_MIXED if mixed else APPLY_IFGF))
        return out

    def solve(self, rhs, tol=1e-6, restart=300, max_iters=1000, mixed=True, precond=None):
        """GMRES for every member in lock step; ``self.last_solve`` holds per-member iterations and
        estimated errors (FP64 relative residuals with mixed=True).  precond="spectral": flexible
        GMRES with the spectral right preconditioner (each member at its own wavenumber)."""
        if precond not in (None, "spectral"):
            raise ValueError("group solves take precond=None or 'spectral'")
        b = _cview(rhs, self.N)
        x = np.empty(self.N, dtype=np.complex128)
        it = np.zeros(self.n, dtype=np.int32)
        err = np.zeros(self.n)
        mode = APPLY_IFGF_MIXED if mixed else APPLY_IFGF
        if precond == "spectral":
            rc = _lib.load().ifgf2d_group_solve_flexible(self._h, PRECOND_SPECTRAL, _dp(b.view(np.float64)),
                                                         _dp(x.view(np.float64)), mode, float(tol), int(restart), int(max_iters),
                                                         it.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(err))
        else:
            rc = _lib.load().ifgf2d_group_solve(self._h, _dp(b.view(np.float64)), _dp(x.view(np.float64)), mode, float(tol),
                                                int(restart), int(max_iters), it.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                _dp(err))
        self.last_solve = dict(iters=it.tolist(), error=err.tolist(), converged=(rc == 0))
        if rc != 8:
            self._check(rc)
        return x

