"""Many independent obstacles, each solved to a tolerance on its own context.

The reference solves one obstacle per ForwardMap (ForwardMap.tpp:658-697).  Here the work of
an obstacle is split at the host/device line: a pool of host threads runs the host part
(discretisation, tree depth, tree and plans: ifgf2d_create + ifgf2d_prepare, no CUDA calls)
ahead of the device part (precomputation, device tables, GMRES, residual).  Set-up calls run
single-threaded inside (ifgf2d_set_host_threads(1)); the pool supplies the host parallelism.

* solve_obstacles: a few device threads each run one obstacle's device part at a time, on
  the obstacle's own context stream.
* solve_obstacles_grouped: the device threads take groups of obstacles, each merged into one
  block-diagonal operator (ifgf2d_group_*) whose set-up and applies are one launch per phase
  over the whole group, solved by GMRES per obstacle in lock step.

Obstacles below `direct_below` unknowns, and those whose points no tree depth keeps in the
leaf neighbourhood, use the direct operator, which needs no tree.

The seeded configuration of `star_obstacles` is the multi-obstacle benchmark: star curves
r(t) = 1 + sum_{m=1..5} a_m cos mt + b_m sin mt with a_m, b_m ~ U(-0.05, 0.05), k ~ U(10, 400),
N_i = 16 * ceil(10 k L / (2 pi) / 16) points (10 per wavelength, L the perimeter) and a plane
wave at an angle ~ U(0, 2 pi), drawn from numpy's default_rng(seed).
"""
from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Obstacle:
    a: np.ndarray                  # cosine coefficients a_1..a_M of the star radius
    b: np.ndarray                  # sine coefficients b_1..b_M
    k: float                       # wavenumber
    angle: float                   # incidence angle of the plane wave
    npoints: int                   # unknowns (a multiple of 16)
    result: dict = field(default_factory=dict)


def star_perimeter(a, b, nt=4000):
    t = np.linspace(0.0, 2 * np.pi, nt, endpoint=False)
    m = np.arange(1, len(a) + 1)
    r = 1.0 + (np.asarray(a)[None, :] * np.cos(m[None, :] * t[:, None]) + np.asarray(b)[None, :] * np.sin(m[None, :] * t[:, None])).sum(1)
    dr = (m[None, :] * (-np.asarray(a)[None, :] * np.sin(m[None, :] * t[:, None])
                        + np.asarray(b)[None, :] * np.cos(m[None, :] * t[:, None]))).sum(1)
    return float(np.sum(np.sqrt(r * r + dr * dr)) * (2 * np.pi / nt))


def star_obstacles(n=256, seed=0, kmin=10.0, kmax=400.0, modes=5, amp=0.05, ppw=10.0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        a = rng.uniform(-amp, amp, modes)
        b = rng.uniform(-amp, amp, modes)
        k = float(rng.uniform(kmin, kmax))
        ang = float(rng.uniform(0.0, 2 * np.pi))
        L = star_perimeter(a, b)
        npts = 16 * int(math.ceil(ppw * k * L / (2 * np.pi) / 16))
        out.append(Obstacle(a, b, k, ang, npts))
    return out


def _prepare_one(G, ob, direct_below):
    fm = G.ForwardMap(0.01, [G.Star(ob.a, ob.b)], (), 1.0, ob.k, Np=16, patches_per_curve=max(ob.npoints // 16, 4),
                      formulation="combined")
    accel = fm.total_num_unknowns_ >= direct_below
    if accel:
        try:
            fm.prepare(ob.k, 0)
        except G.NeighbourhoodError:
            accel = False
    return fm, accel


def _device_one(G, ob, fm, accel, tol, mixed, restart, max_iters):
    rhs = -np.exp(1j * ob.k * (math.cos(ob.angle) * fm.xs_ + math.sin(ob.angle) * fm.ys_))
    if accel:
        fm.precomps_and_setup(ob.k, 0)
    else:
        fm.compute_precomputations(ob.k)
    x = fm.gmres(rhs, accelerated=accel, tol=tol, restart=restart, max_iters=max_iters, mixed=mixed and accel)
    st = dict(fm.last_solve)
    y = fm.compute_Ax_acc(x) if accel else fm.compute_Ax_unacc(x)
    st["true_rel_residual"] = float(np.linalg.norm(y - rhs) / np.linalg.norm(rhs))
    st["accelerated"] = accel
    st["N"] = fm.total_num_unknowns_
    ob.result = st
    return x


def solve_obstacles(obstacles, tol=1e-6, workers=15, mixed=True, direct_below=0, restart=300, max_iters=1000,
                    keep_solutions=False, lookahead=None, device_threads=3):
    """Solve every obstacle (plane-wave scattering, combined field) to `tol`.  Returns the
    densities when keep_solutions, else None; each obstacle's `result` holds iterations,
    convergence, the true FP64 relative residual and the operator used.  workers = 0 runs
    everything on the calling thread.  device_threads > 1 runs the device part of that many
    obstacles at once (obstacle i on thread i mod device_threads), each on its own context
    stream; contexts allocate stream-ordered, so their set-up and tear-down do not stall one
    another."""
    import threading
    from . import _lib
    import ifgf2d_gb300 as G
    L = _lib.load()
    n = len(obstacles)
    xs = [None] * n
    if workers <= 0:
        for i, ob in enumerate(obstacles):
            fm, accel = _prepare_one(G, ob, direct_below)
            x = _device_one(G, ob, fm, accel, tol, mixed, restart, max_iters)
            del fm
            xs[i] = x if keep_solutions else None
        return xs if keep_solutions else None
    T = max(1, int(device_threads))
    ahead = max(lookahead or 2 * workers, T)
    slots = threading.Semaphore(ahead)          # host preparations submitted but not yet taken
    futs = [None] * n
    ready = [threading.Event() for _ in range(n)]
    stop = threading.Event()
    L.ifgf2d_set_host_threads(1)
    try:
        with ThreadPoolExecutor(workers) as ex, ThreadPoolExecutor(T) as dev:
            def submit_all():
                for i, ob in enumerate(obstacles):
                    while not slots.acquire(timeout=0.1):
                        if stop.is_set():
                            return
                    futs[i] = ex.submit(_prepare_one, G, ob, direct_below)
                    ready[i].set()

            def device_loop(t):
                try:
                    for i in range(t, n, T):
                        while not ready[i].wait(timeout=0.1):
                            if stop.is_set():
                                return
                        fm, accel = futs[i].result()
                        futs[i] = None
                        slots.release()
                        x = _device_one(G, obstacles[i], fm, accel, tol, mixed, restart, max_iters)
                        del fm
                        xs[i] = x if keep_solutions else None
                except BaseException:
                    stop.set()
                    raise

            sub = threading.Thread(target=submit_all, daemon=True)
            sub.start()
            try:
                for f in [dev.submit(device_loop, t) for t in range(T)]:
                    f.result()
            finally:
                stop.set()
                sub.join()
    finally:
        L.ifgf2d_set_host_threads(0)
    return xs if keep_solutions else None


def solve_obstacles_grouped(obstacles, tol=1e-6, workers=15, mixed=True, restart=300, max_iters=1000,
                            keep_solutions=False, chunk=16, device_threads=3, precond=None):
    """Solve the obstacles in groups (ifgf2d_group_*) of `chunk` obstacles (None: one group).
    The host part of each obstacle's set-up (discretisation, tree depth, tree and plans) runs on
    `workers` threads; `device_threads` threads take the groups in turn as their obstacles are
    prepared, each merging its group into one context with its own stream and running its device
    set-up and lock-step GMRES: each phase of a group's set-up and of every apply is one launch
    over all its obstacles, and several groups overlap on the GPU.  Obstacles whose points no tree
    depth keeps in the leaf neighbourhood use the direct operator, one at a time.  Each obstacle's
    `result` holds its iterations, convergence, true FP64 relative residual and operator; returns
    the densities when keep_solutions.  precond="spectral": the groups' GMRES is flexible, with the
    spectral right preconditioner."""
    from . import _lib
    import ifgf2d_gb300 as G
    L = _lib.load()
    n = len(obstacles)
    size = n if not chunk else max(1, int(chunk))
    xs = [None] * n
    direct = []
    futs = [None] * n

    def run_group(c0):
        idx = list(range(c0, min(n, c0 + size)))
        prepared = {i: futs[i].result() for i in idx}
        acc = [i for i in idx if prepared[i][1]]
        dlist = [(i, prepared[i][0]) for i in idx if not prepared[i][1]]
        if not acc:
            return dlist
        rhs_of = []
        for i in acc:
            ob, fm = obstacles[i], prepared[i][0]
            rhs_of.append(-np.exp(1j * ob.k * (math.cos(ob.angle) * fm.xs_ + math.sin(ob.angle) * fm.ys_)))
        grp = G.Group([prepared[i][0] for i in acc])
        for i in acc:                       # the group holds its own copy of everything
            prepared[i][0].close()
        rhs = np.concatenate(rhs_of)
        x = grp.solve(rhs, tol=tol, restart=restart, max_iters=max_iters, mixed=mixed, precond=precond)
        st = grp.last_solve
        res = grp.split(grp.apply(x) - rhs)
        parts = grp.split(x)
        for q, i in enumerate(acc):
            b = rhs_of[q]
            obstacles[i].result = {"iters": st["iters"][q], "error": st["error"][q], "converged": st["error"][q] < tol,
                                   "true_rel_residual": float(np.linalg.norm(res[q]) / np.linalg.norm(b)),
                                   "accelerated": True, "N": int(b.size), "grouped": True}
            if keep_solutions:
                xs[i] = parts[q].copy()
        grp.close()
        return dlist

    L.ifgf2d_set_host_threads(1)                # the pools supply the host parallelism
    try:
        with ThreadPoolExecutor(max(1, workers)) as ex, ThreadPoolExecutor(max(1, int(device_threads))) as dev:
            for i, ob in enumerate(obstacles):
                futs[i] = ex.submit(_prepare_one, G, ob, 0)
            for f in [dev.submit(run_group, c0) for c0 in range(0, n, size)]:
                direct += f.result()
    finally:
        L.ifgf2d_set_host_threads(0)
    for i, fm in direct:
        x = _device_one(G, obstacles[i], fm, False, tol, mixed, restart, max_iters)
        obstacles[i].result["grouped"] = False
        xs[i] = x if keep_solutions else None
        fm.close()
    return xs if keep_solutions else None
