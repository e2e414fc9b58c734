"""IFGF-accelerated off-surface field (ifgf2d_eval_offsurface) -- needs a GPU.

The reference evaluates off-surface fields directly (ForwardMap::propagate_unacc,
ForwardMap.tpp:701-727); the accelerated form must agree with that direct sum (pinned to the
oracle in test_gpu_parity.py) within the IFGF interpolation tolerance, here 1e-3 relative for
5 x 5 cones, for targets near the curve, inside and outside the tree's root box and far away.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _targets(fm, seed=0, n=4000, lo=-3.0, hi=3.0, gap=0.02):
    """uniform points in a square, minus those within `gap` of a discretisation point"""
    rng = np.random.default_rng(seed)
    p = rng.uniform(lo, hi, size=(n, 2))
    d = np.min(np.hypot(p[:, None, 0] - fm.xs_[None, :], p[:, None, 1] - fm.ys_[None, :]), axis=1)
    p = p[d > gap]
    return p[:, 0].copy(), p[:, 1].copy()


@pytest.mark.parametrize("form", ["single_layer", "combined"])
def test_gpu_offsurface_matches_direct(lib, oracle, form):
    k = 100.0
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=128, formulation=form)
    fm.precomps_and_setup(k, 0)
    d = oracle.seeded_density(fm.total_num_unknowns_)
    tx, ty = _targets(fm)
    u = fm.propagate_acc(tx, ty, d)
    ud = fm.propagate_unacc(tx, ty, d)
    assert rel(u, ud) < 1e-3
    # the plan is reused for a second density on the same points
    d2 = oracle.seeded_density(fm.total_num_unknowns_, seed=1)
    assert rel(fm.propagate_acc(tx, ty, d2), fm.propagate_unacc(tx, ty, d2)) < 1e-3
    # targets outside the root box, from just outside to far away
    th = np.linspace(0, 2 * np.pi, 97)[:-1]
    for R in (2.2, 5.0, 60.0, 2000.0):
        ox, oy = R * np.cos(th), R * np.sin(th)
        assert rel(fm.propagate_acc(ox, oy, d), fm.propagate_unacc(ox, oy, d)) < 1e-3, R


def test_gpu_offsurface_against_oracle(lib, oracle):
    k = 40.0
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=64)
    om = oracle.OracleForwardMap([oracle.curve_kite()], 16, 0.01, 1.0, k, patches_per_curve=64)
    fm.precomps_and_setup(k, 0)
    om.precompute(k)
    d = oracle.seeded_density(fm.total_num_unknowns_)
    tx, ty = _targets(fm, seed=3, n=600)
    assert rel(fm.propagate_acc(tx, ty, d), om.propagate_unacc(tx, ty, d)) < 1e-3


def test_gpu_offsurface_mie_circle(lib):
    """Combined field on the unit circle at k = 200 (N = 3200): the accelerated field at r = 2
    against the exact series for a sound-soft circle."""
    import scipy.special as sp
    k = 200.0
    fm = lib.ForwardMap(0.01, [lib.Circle()], (), 1.0, k, Np=16, patches_per_curve=200, formulation="combined")
    fm.precomps_and_setup(k, 0)
    x = fm.gmres(-np.exp(1j * k * fm.xs_), accelerated=True, tol=1e-10, restart=300, max_iters=1000)
    assert fm.last_solve["converged"]
    th = np.linspace(0, 2 * np.pi, 61)[:-1]
    r = 2.0 * np.ones_like(th)
    n = np.arange(-320, 321)
    c = -(1j ** n) * sp.jv(n, k) / sp.hankel1(n, k)
    ue = (c[None, :] * sp.hankel1(n[None, :], k * r[:, None]) * np.exp(1j * n[None, :] * th[:, None])).sum(1)
    u = fm.propagate_acc(r * np.cos(th), r * np.sin(th), x)
    assert np.abs(u - ue).max() / np.abs(ue).max() < 1e-3


def test_gpu_offsurface_edges(lib, oracle):
    k = 40.0
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=64)
    fm.precomps_and_setup(k, 0)
    d = oracle.seeded_density(fm.total_num_unknowns_)
    L = lib._lib.load()
    # no targets: a no-op
    assert fm.propagate_acc(np.zeros(0), np.zeros(0), d).size == 0
    # a target on a discretisation point: its own term is zero in both forms (r < 1e-14)
    tx, ty = np.array([fm.xs_[5], 0.3]), np.array([fm.ys_[5], 0.2])
    assert rel(fm.propagate_acc(tx, ty, d), fm.propagate_unacc(tx, ty, d)) < 1e-3
    # state and argument errors
    fm2 = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=64)
    fm2.compute_precomputations(k)
    with pytest.raises(lib.IFGF2DError):
        fm2.propagate_acc(tx, ty, d)
    assert L.ifgf2d_eval_offsurface_setup(fm.handle, -1, None, None) == 1
    bad = np.array([np.nan, 0.0])
    with pytest.raises(Exception):
        fm.propagate_acc(bad, bad, d)
