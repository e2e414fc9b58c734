"""The learned right preconditioner: network object, training data and training.

The network (a 1D convolution stack along the boundary, see include/ifgf2d.h and
csrc/precond_net.cuh) maps a residual r on a curve to M(r) = 2 r + sigma e^{i phi} (o_0 + i o_1)
(sigma the RMS of r, phi its canonical phase).  It is
trained on (residual, error) pairs harvested from the plain method's own solves: for a
problem A x = b with converged solution x*, a GMRES iterate x_j stopped after j iterations
gives r_j = b - A x_j and e_j = x* - x_j (A e_j = r_j), and the network learns
o ~ (e - 2 r) e^{-i phi} / sigma.  Training runs on the GPU with the library's own forward and backward kernels and
AdamW.  Solves use it through ForwardMap.solve_precond (flexible GMRES inside FP64 iterative
refinement, plain GMRES when it stalls).

Weights are stored as a flat binary: the 8-byte magic b"IFGFNET\\x02", the parameter count
(int64), the output weighting flag (int64; ifgf2d_net_set_output_weighting), then the FP32
parameters in the order of include/ifgf2d.h.  Files with the magic b"IFGFNET\\x01" have no flag
(unweighted).
"""
from __future__ import annotations

import ctypes
import math
import os
import struct

import numpy as np

from . import _lib

MAGIC = b"IFGFNET\x02"
MAGIC_V1 = b"IFGFNET\x01"
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "cfie_conv6x64.bin")
# the network trained as a correction of the spectral preconditioner (ForwardMap.solve_flexible
# with precond="spectral+net"): targets e - M_s r instead of e - 2 r
SPECTRAL_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "cfie_conv6x64_spectral.bin")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class NetError(RuntimeError):
    pass


def _pack(samples, with_e=True):
    lens = np.array([len(s[0]) for s in samples], dtype=np.int32)
    r = np.ascontiguousarray(np.concatenate([np.asarray(s[0], dtype=np.complex128) for s in samples]))
    e = np.ascontiguousarray(np.concatenate([np.asarray(s[1], dtype=np.complex128) for s in samples])) if with_e else None
    g = np.ascontiguousarray(np.concatenate([np.asarray(s[2], dtype=np.float64).reshape(-1, 4) for s in samples]))
    k = np.array([float(s[3]) for s in samples], dtype=np.float64)
    return lens, r, e, g, k


class PreconditionerNet:
    """The network on the current GPU.  Samples are tuples (r, e, geom, k): a residual and its
    error on one curve (patch order), the curve's geometry features (N x 4: curvature,
    tangent x, tangent y, quadrature weight; ForwardMap.geometry_features) and k."""

    def __init__(self, seed=0):
        L = _lib.load()
        h = ctypes.c_void_p()
        rc = L.ifgf2d_net_create(ctypes.c_ulonglong(seed), ctypes.byref(h))
        if rc != 0:
            raise NetError(f"ifgf2d_net_create failed ({rc})")
        self._h = h
        self.nparam = int(L.ifgf2d_net_num_params())

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                _lib.load().ifgf2d_net_destroy(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _check(self, rc):
        if rc != 0:
            raise NetError(f"ifgf2d net call failed ({rc}): {_lib.load().ifgf2d_net_last_error(self._h).decode()}")

    @property
    def params(self):
        p = np.empty(self.nparam, dtype=np.float32)
        self._check(_lib.load().ifgf2d_net_get_params(self._h, _fp(p)))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparam:
            raise ValueError(f"expected {self.nparam} parameters, got {p.size}")
        self._check(_lib.load().ifgf2d_net_set_params(self._h, _fp(p)))

    @property
    def weighted(self):
        """True when the output is the |sigma|-weighted correction of the spectral preconditioner"""
        return _lib.load().ifgf2d_net_output_weighting(self._h) == 1

    @weighted.setter
    def weighted(self, flag):
        self._check(_lib.load().ifgf2d_net_set_output_weighting(self._h, 1 if flag else 0))

    def save(self, path):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "wb") as f:
            f.write(MAGIC)
            f.write(struct.pack("<q", self.nparam))
            f.write(struct.pack("<q", 1 if self.weighted else 0))
            f.write(self.params.astype("<f4").tobytes())

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS):
        with open(path, "rb") as f:
            magic = f.read(8)
            if magic not in (MAGIC, MAGIC_V1):
                raise NetError(f"{path}: not a preconditioner weight file")
            (n,) = struct.unpack("<q", f.read(8))
            flags = struct.unpack("<q", f.read(8))[0] if magic == MAGIC else 0
            p = np.frombuffer(f.read(4 * n), dtype="<f4")
        net = cls()
        if n != net.nparam:
            raise NetError(f"{path}: {n} parameters, the network has {net.nparam}")
        net.params = p
        net.weighted = bool(flags & 1)
        return net

    def gradient(self, samples):
        lens, r, e, g, k = _pack(samples)
        loss = ctypes.c_double(0.0)
        grad = np.empty(self.nparam, dtype=np.float32)
        self._check(_lib.load().ifgf2d_net_gradient(self._h, len(samples), _ip(lens), _dp(r.view(np.float64)),
                                                    _dp(e.view(np.float64)), _dp(g), _dp(k), ctypes.byref(loss), _fp(grad)))
        return loss.value, grad

    def train_step(self, samples, lr=1e-3, weight_decay=1e-4):
        lens, r, e, g, k = _pack(samples)
        loss = ctypes.c_double(0.0)
        self._check(_lib.load().ifgf2d_net_train_step(self._h, len(samples), _ip(lens), _dp(r.view(np.float64)),
                                                      _dp(e.view(np.float64)), _dp(g), _dp(k), ctypes.c_float(lr),
                                                      ctypes.c_float(weight_decay), ctypes.byref(loss)))
        return loss.value

    def apply(self, samples):
        """M(r) per sample, and the raw two output channels (npoints x 2)"""
        lens, r, _, g, k = _pack([(s[0], None, s[2], s[3]) for s in samples], with_e=False)
        z = np.empty(r.size, dtype=np.complex128)
        o = np.empty(2 * r.size, dtype=np.float32)
        self._check(_lib.load().ifgf2d_net_apply(self._h, len(samples), _ip(lens), _dp(r.view(np.float64)), _dp(g), _dp(k),
                                                 _dp(z.view(np.float64)), _fp(o)))
        out, off = [], 0
        for n in lens:
            out.append(z[off:off + n])
            off += n
        return out, o.reshape(-1, 2)


# ---------------------------------------------------------------- training data
def harvest(fm, k, rhs, stops=(1, 2, 4, 8, 16, 32), tol=1e-9, base=None):
    """(r, e, geom, k) pairs from the plain FP64 IFGF GMRES of one problem: the converged
    solution x*, then GMRES stopped after j iterations for every j in `stops`.  base="spectral":
    the network is to correct the spectral preconditioner M_s, so the stored error is
    e - (M_s r - 2 r), whose target (e' - 2 r) is what M_s leaves of e.  base="spectral_weighted":
    the stored error is 2 r + Op(|sigma|)(e - M_s r), so that the loss measures what M_s leaves in
    the residual (A ~ Op(sigma) along the curve), and the network is applied through Op(1/|sigma|)."""
    xs = fm.gmres(rhs, accelerated=True, tol=tol, restart=300, max_iters=1000)
    geom = fm.geometry_features()
    if base in ("spectral", "spectral_weighted"):
        fm.spectral_setup()
    out = []
    for j in stops:
        xj = fm.gmres(rhs, accelerated=True, tol=1e-15, restart=max(j, 1), max_iters=j)
        r = rhs - fm.compute_Ax_acc(xj)
        if np.linalg.norm(r) <= 1e-12 * np.linalg.norm(rhs):
            break
        e = xs - xj
        if base == "spectral":
            e = e - (fm.spectral_apply(r) - 2.0 * r)
        elif base == "spectral_weighted":   # target Op(|sigma|) (e - M_s r): the residual-space error
            e = 2.0 * r + fm.spectral_symbol(e - fm.spectral_apply(r), "magnitude")
        out.append((r, e, geom, k))
    return out


def training_problems(n=160, seed=0, kmin=50.0, kmax=400.0, kite_every=4):
    """seeded star obstacles and kites with k ~ U(kmin, kmax), 10 points per wavelength"""
    from .scatterers import star_obstacles
    import ifgf2d_gb300 as G
    rng = np.random.default_rng(seed + 1000)
    obs = star_obstacles(n, seed=seed, kmin=kmin, kmax=kmax)
    probs = []
    for i, ob in enumerate(obs):
        if kite_every and i % kite_every == kite_every - 1:
            k = ob.k
            L = 9.3245   # the kite's perimeter
            npts = 16 * int(math.ceil(10 * k * L / (2 * np.pi) / 16))
            probs.append(("kite", G.Kite(), k, float(rng.uniform(0, 2 * np.pi)), npts))
        else:
            probs.append(("star", G.Star(ob.a, ob.b), ob.k, ob.angle, ob.npoints))
    return probs


def harvest_set(problems, stops=(1, 2, 4, 8, 16, 32), log=None, base=None):
    import ifgf2d_gb300 as G
    pairs = []
    for name, curve, k, ang, npts in problems:
        fm = G.ForwardMap(0.01, [curve], (), 1.0, k, Np=16, patches_per_curve=max(npts // 16, 4), formulation="combined")
        try:
            fm.precomps_and_setup(k, 0)
        except G.NeighbourhoodError:
            continue
        rhs = -np.exp(1j * k * (math.cos(ang) * fm.xs_ + math.sin(ang) * fm.ys_))
        pairs += harvest(fm, k, rhs, stops, base=base)
        if log:
            log(f"{name} k={k:.1f} N={fm.total_num_unknowns_}: {len(pairs)} pairs")
    return pairs


def train(net, pairs, steps=2000, batch_points=65536, lr=1e-3, lr_min=1e-5, weight_decay=1e-4, seed=0, val=None, log=None):
    """AdamW with a cosine learning rate; each step a random batch of pairs up to
    `batch_points` points.  Returns the loss history (and validation losses every 100 steps)."""
    rng = np.random.default_rng(seed)
    hist, vhist = [], []
    order = np.arange(len(pairs))
    for step in range(steps):
        rng.shuffle(order)
        batch, npts = [], 0
        for i in order:
            n = len(pairs[i][0])
            if batch and npts + n > batch_points:
                break
            batch.append(pairs[i])
            npts += n
        cur = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * step / max(steps, 1)))
        hist.append(net.train_step(batch, lr=cur, weight_decay=weight_decay))
        if val is not None and (step % 100 == 0 or step == steps - 1):
            vhist.append((step, net.gradient(val)[0]))
            if log:
                log(f"step {step}: train {hist[-1]:.4e} val {vhist[-1][1]:.4e} lr {cur:.2e}")
    return hist, vhist


def main(argv=None):
    """Train the network as shipped: python -m ifgf2d_gb300.learned --out PATH"""
    import argparse
    import time
    ap = argparse.ArgumentParser(description="harvest (residual, error) pairs from plain GMRES and train the network")
    ap.add_argument("--out", default=None)
    ap.add_argument("--base", choices=("none", "spectral", "spectral_weighted"), default="none",
                    help="spectral: train the correction of the spectral preconditioner; spectral_weighted: the same with "
                         "the |sigma|-weighted (residual-space) loss")
    ap.add_argument("--problems", type=int, default=160)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)
    t0 = time.perf_counter()
    base = None if args.base == "none" else args.base
    out = args.out or (SPECTRAL_WEIGHTS if base in ("spectral", "spectral_weighted") else DEFAULT_WEIGHTS)
    pairs = harvest_set(training_problems(args.problems, seed=args.seed), base=base)
    rng = np.random.default_rng(args.seed)
    idx = rng.permutation(len(pairs))
    nval = max(4, len(pairs) // 10)
    val, tr = [pairs[i] for i in idx[:nval]], [pairs[i] for i in idx[nval:]]
    print(f"{len(pairs)} pairs ({sum(len(p[0]) for p in pairs)} points) in {time.perf_counter() - t0:.1f} s", flush=True)
    net = PreconditionerNet(args.seed)
    t0 = time.perf_counter()
    train(net, tr, steps=args.steps, seed=args.seed, val=val, log=lambda m: print(m, flush=True))
    print(f"trained in {time.perf_counter() - t0:.1f} s", flush=True)
    net.weighted = base == "spectral_weighted"
    net.save(out)
    print("saved", out)


if __name__ == "__main__":
    main()
