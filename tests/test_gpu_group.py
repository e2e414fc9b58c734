"""Many obstacles as one block-diagonal operator (ifgf2d_group_*) -- needs a GPU.

A group merges prepared contexts of uneven sizes and wavenumbers; its apply must equal each
member's own apply on the member's unknowns, and its solve must reach every member's tolerance
with that member's own iteration count (GMRES per member, in lock step).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _members(lib, seed=3, n=10, kmax=150.0):
    from ifgf2d_gb300.scatterers import star_obstacles
    fms, kept = [], []
    for ob in star_obstacles(n, seed=seed, kmax=kmax):
        fm = lib.ForwardMap(0.01, [lib.Star(ob.a, ob.b)], (), 1.0, ob.k, Np=16, patches_per_curve=max(ob.npoints // 16, 4),
                            formulation="combined")
        try:
            fm.prepare(ob.k, 0)
        except lib.NeighbourhoodError:      # no tree depth keeps its singular points in the leaf neighbourhood
            continue
        fms.append(fm)
        kept.append(ob)
    assert len(fms) >= n - 2
    return kept, fms


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_gpu_group_apply_equals_members(lib, oracle):
    obs, fms = _members(lib)
    g = lib.Group(fms)
    assert g.N == sum(fm.total_num_unknowns_ for fm in fms)
    x = oracle.seeded_density(g.N)
    y64, y32 = g.apply(x), g.apply(x, mixed=True)
    for fm, ob, xs, a, b in zip(fms, obs, g.split(x), g.split(y64), g.split(y32)):
        fm.precomps_and_setup(ob.k, 0)
        assert rel(a, fm.compute_Ax_acc(xs)) < 1e-13
        assert rel(b, fm.compute_Ax_acc(xs, mixed=True)) < 1e-6


@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_group_solve_reaches_every_member(lib, mixed):
    obs, fms = _members(lib, seed=4)
    g = lib.Group(fms)
    rhs = np.concatenate([-np.exp(1j * ob.k * (np.cos(ob.angle) * fm.xs_ + np.sin(ob.angle) * fm.ys_))
                          for ob, fm in zip(obs, fms)])
    tol = 1e-6 if mixed else 1e-8
    x = g.solve(rhs, tol=tol, restart=300, max_iters=1000, mixed=mixed)
    assert g.last_solve["converged"]
    res = g.apply(x) - rhs
    for r, b in zip(g.split(res), g.split(rhs)):
        assert np.linalg.norm(r) / np.linalg.norm(b) < (tol if mixed else 10 * tol)
    # each member alone, the same solver
    for o, (fm, ob, xs, b) in enumerate(zip(fms, obs, g.split(x), g.split(rhs))):
        fm.precomps_and_setup(ob.k, 0)
        xo = fm.gmres(b, tol=tol, restart=300, max_iters=1000, mixed=mixed)
        assert abs(fm.last_solve["iters"] - g.last_solve["iters"][o]) <= 2, o
        assert rel(xs, xo) < (1e-5 if mixed else 1e-6)


@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_group_spectral_solve(lib, mixed):
    """Flexible GMRES with the spectral preconditioner over a group (each member's symbol at its
    own wavenumber): every member reaches its tolerance, with at most one iteration more than the
    unpreconditioned group solve and a fifth fewer over the group, and with the same solution."""
    obs, fms = _members(lib, seed=4)
    g = lib.Group(fms)
    rhs = np.concatenate([-np.exp(1j * ob.k * (np.cos(ob.angle) * fm.xs_ + np.sin(ob.angle) * fm.ys_))
                          for ob, fm in zip(obs, fms)])
    tol = 1e-6 if mixed else 1e-8
    x0 = g.solve(rhs, tol=tol, restart=300, max_iters=1000, mixed=mixed)
    it0 = np.array(g.last_solve["iters"])
    x1 = g.solve(rhs, tol=tol, restart=300, max_iters=1000, mixed=mixed, precond="spectral")
    it1 = np.array(g.last_solve["iters"])
    assert g.last_solve["converged"]
    res = g.apply(x1) - rhs
    for r, b in zip(g.split(res), g.split(rhs)):
        assert np.linalg.norm(r) / np.linalg.norm(b) < (tol if mixed else 10 * tol)
    assert np.all(it1 <= it0 + 1), (it0, it1)
    assert it1.sum() <= 0.8 * it0.sum(), (it0, it1)
    for a, b in zip(g.split(x1), g.split(x0)):
        assert rel(a, b) < (1e-5 if mixed else 1e-6)


def test_gpu_grouped_driver_matches_one_at_a_time(lib):
    """scatterers.solve_obstacles_grouped: groups of four obstacles on two device threads reach
    each obstacle's FP64 tolerance, and their solutions equal those of the one-at-a-time path."""
    from ifgf2d_gb300.scatterers import star_obstacles, solve_obstacles, solve_obstacles_grouped
    obs = star_obstacles(10, seed=5, kmax=150.0)
    xg = solve_obstacles_grouped(obs, tol=1e-8, workers=4, mixed=False, keep_solutions=True, chunk=4, device_threads=2)
    assert all(o.result["converged"] for o in obs)
    assert max(o.result["true_rel_residual"] for o in obs) < 1e-7
    ref = star_obstacles(10, seed=5, kmax=150.0)
    xr = solve_obstacles(ref, tol=1e-8, workers=0, mixed=False, keep_solutions=True)
    for a, b, o, r in zip(xg, xr, obs, ref):
        assert abs(o.result["iters"] - r.result["iters"]) <= 1
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-6


def test_gpu_group_of_one_equals_its_member(lib, oracle):
    """The degenerate group: one member's merged tables give that member's own apply and solve."""
    k = 150.0
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=128, formulation="combined")
    fm.prepare(k, 0)
    g = lib.Group([fm])
    assert g.N == fm.total_num_unknowns_ and list(g.offsets) == [0, g.N]
    x = oracle.seeded_density(g.N)
    fm.precomps_and_setup(k, 0)
    assert rel(g.apply(x), fm.compute_Ax_acc(x)) < 1e-13
    rhs = -np.exp(1j * k * fm.xs_)
    xg = g.solve(rhs, tol=1e-8, restart=300, max_iters=500, mixed=False)
    xm = fm.gmres(rhs, tol=1e-8, restart=300, max_iters=500)
    assert g.last_solve["converged"] and abs(g.last_solve["iters"][0] - fm.last_solve["iters"]) <= 1
    assert rel(xg, xm) < 1e-6
