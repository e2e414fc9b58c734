"""The spectral right preconditioner (csrc/spectral_precond.cu) against its numpy oracle
(oracle/spectral_oracle.py), and the flexible GMRES that uses it.

The reference's GMRES is unpreconditioned (ForwardMap/ForwardMap.tpp:658-697); the
preconditioner only changes the iteration count, never the answer, so the solves are judged by
their FP64 true residual and against the unpreconditioned solution."""
import numpy as np
import pytest

from oracle.spectral_oracle import CURVE_KITE, CURVE_STAR, SpectralPreconditioner

pytestmark = pytest.mark.gpu

# the device runs the preconditioner in FP32 (tables, FFTs and sums)
TOL_APPLY = 2e-5

STAR_A, STAR_B = [0.03, -0.04, 0.02, 0.01, -0.02], [0.01, 0.02, -0.03, 0.04, 0.01]


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _pair(lib, oracle, shape, k, patches):
    if shape == "kite":
        curve, ocurve, ctype, params = lib.Kite(), oracle.curve_kite(), CURVE_KITE, [1.0, 0.65, -0.65, 1.5]
    else:
        curve, ocurve = lib.Star(STAR_A, STAR_B), oracle.curve_star(STAR_A, STAR_B)
        ctype, params = CURVE_STAR, [0.0, 0.0, 5.0] + STAR_A + STAR_B
    fm = lib.ForwardMap(0.01, [curve], (), 1.0, k, Np=16, patches_per_curve=patches, formulation="combined")
    om = oracle.OracleForwardMap([ocurve], 16, 0.01, 1.0, k, patches_per_curve=patches, formulation="combined", coupling=k)
    t12, _ = om.patch_info()
    fn = np.cos(np.pi * (2 * np.arange(16) + 1) / 32)
    tp = (t12[:, 0][:, None] + (fn[None, :] + 1) * 0.5 * (t12[:, 1] - t12[:, 0])[:, None]).ravel()
    return fm, (ctype, params, t12[:, 0], t12[:, 1], tp)


@pytest.mark.parametrize("shape,k,patches", [("kite", 100.0, 128), ("star", 60.0, 50), ("kite", 500.0, 512)])
def test_gpu_spectral_apply_matches_oracle(lib, oracle, shape, k, patches):
    """M r on the device equals the numpy restatement (its own arc-length tables and FFTs) on
    grids of 1024 (the star's 800 points), 2048 and 8192 points."""
    fm, cdesc = _pair(lib, oracle, shape, k, patches)
    fm.compute_precomputations(k)
    scale = 0.25
    fm.spectral_setup(scale)
    M = SpectralPreconditioner([cdesc], 16, k, eta=k, eps=scale * k ** (1 / 3))
    for seed in (0, 1):
        r = oracle.seeded_density(fm.total_num_unknowns_, seed=seed) - (0.5 + 0.5j)
        assert rel(fm.spectral_apply(r), M(r)) < TOL_APPLY
    # linear: M(a r1 + r2) = a M r1 + M r2
    r1 = oracle.seeded_density(fm.total_num_unknowns_, seed=2)
    r2 = oracle.seeded_density(fm.total_num_unknowns_, seed=3)
    a = 0.3 - 1.7j
    assert rel(fm.spectral_apply(a * r1 + r2), a * fm.spectral_apply(r1) + fm.spectral_apply(r2)) < TOL_APPLY


@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_spectral_solve_reaches_tolerance_in_fewer_iterations(lib, mixed):
    """Kite, k = 300: flexible GMRES with the spectral preconditioner reaches the FP64 tolerance
    with at most two thirds of plain GMRES's iterations, and the same solution."""
    k = 300.0
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=320, formulation="combined")
    fm.precomps_and_setup(k, 0)
    rhs = -np.exp(1j * k * fm.xs_)
    x0 = fm.gmres(rhs, tol=1e-6, mixed=mixed)
    it0 = fm.last_solve["iters"]
    x1 = fm.solve_flexible(rhs, precond="spectral", tol=1e-6, mixed=mixed)
    it1 = fm.last_solve["iters"]
    assert fm.last_solve["converged"]
    r = fm.compute_Ax_acc(x1) - rhs
    assert np.linalg.norm(r) / np.linalg.norm(rhs) < 1e-6
    assert it1 <= (2 * it0) // 3, (it0, it1)
    assert rel(x1, x0) < 1e-5


def test_gpu_spectral_rejects_what_it_does_not_cover(lib):
    """Single layer and open curves are refused with an argument error."""
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, 50.0, Np=16, patches_per_curve=64)
    fm.compute_precomputations(50.0)
    with pytest.raises(ValueError, match="combined"):
        fm.spectral_setup()
    fm = lib.ForwardMap(0.01, [lib.Line(0.0, 0.0, 1.0, 0.0)], (), 1.0, 50.0, Np=16, patches_per_curve=32,
                        formulation="combined")
    fm.compute_precomputations(50.0)
    with pytest.raises(ValueError, match="closed"):
        fm.spectral_setup()


@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_spectral_batch_solve(lib, mixed):
    """Eight incidence angles on the kite at k = 300 in one batched flexible solve: every column
    reaches the FP64 tolerance with at most two thirds of the unpreconditioned batch's iterations,
    and matches the single-vector spectral solve of that column."""
    k = 300.0
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=320, formulation="combined")
    fm.precomps_and_setup(k, 0)
    ang = np.linspace(0, 2 * np.pi, 8, endpoint=False)
    B = np.stack([-np.exp(1j * k * (np.cos(a) * fm.xs_ + np.sin(a) * fm.ys_)) for a in ang], axis=1)
    fm.gmres_batch(B, tol=1e-6, mixed=mixed)
    it0 = np.array(fm.last_solve["iters"])
    X = fm.gmres_batch(B, tol=1e-6, mixed=mixed, precond="spectral")
    it1 = np.array(fm.last_solve["iters"])
    assert fm.last_solve["converged"]
    assert np.all(it1 <= (2 * it0) // 3), (it0, it1)
    for c in (0, 5):
        r = fm.compute_Ax_acc(X[:, c]) - B[:, c]
        assert np.linalg.norm(r) / np.linalg.norm(B[:, c]) < 1e-6
        xs = fm.solve_flexible(B[:, c], "spectral", tol=1e-6, mixed=mixed)
        assert rel(X[:, c], xs) < 1e-5


def test_gpu_spectral_two_curves(lib, oracle):
    """Two obstacles in one operator (a kite and a circle beside it): each curve gets its own
    resampling grid and multiplier, all in the same four launches; the device M r equals the
    numpy restatement, and the flexible solve reaches the tolerance in fewer iterations."""
    k = 80.0
    kite, circ = lib.Kite(), lib.Circle(3.5, 0.0, 0.8)
    fm = lib.ForwardMap(0.01, [kite, circ], (), 1.0, k, Np=16, patches_per_curve=96, formulation="combined")
    om = oracle.OracleForwardMap([oracle.curve_kite(), oracle.curve_circle(3.5, 0.0, 0.8)], 16, 0.01, 1.0, k,
                                 patches_per_curve=96, formulation="combined", coupling=k)
    t12, _ = om.patch_info()
    fn = np.cos(np.pi * (2 * np.arange(16) + 1) / 32)
    tp = (t12[:, 0][:, None] + (fn[None, :] + 1) * 0.5 * (t12[:, 1] - t12[:, 0])[:, None]).ravel()
    P = t12.shape[0] // 2
    from oracle.spectral_oracle import CURVE_CIRCLE
    curves = [(CURVE_KITE, [1.0, 0.65, -0.65, 1.5], t12[:P, 0], t12[:P, 1], tp[:16 * P]),
              (CURVE_CIRCLE, [3.5, 0.0, 0.8], t12[P:, 0], t12[P:, 1], tp[16 * P:])]
    fm.precomps_and_setup(k, 0)
    fm.spectral_setup(0.25)
    M = SpectralPreconditioner(curves, 16, k, eta=k, eps=0.25 * k ** (1 / 3))
    r = oracle.seeded_density(fm.total_num_unknowns_, seed=4) - (0.5 + 0.5j)
    assert rel(fm.spectral_apply(r), M(r)) < TOL_APPLY
    rhs = -np.exp(1j * k * fm.xs_)
    fm.gmres(rhs, tol=1e-6)
    it0 = fm.last_solve["iters"]
    x = fm.solve_flexible(rhs, "spectral", tol=1e-6)
    assert fm.last_solve["converged"] and fm.last_solve["iters"] < it0
    assert np.linalg.norm(fm.compute_Ax_acc(x) - rhs) / np.linalg.norm(rhs) < 1e-6


def test_gpu_spectral_magnitude_symbols(lib, oracle):
    """The |sigma| and 1/|sigma| tables (the learned network's loss weighting) equal the numpy
    restatement, and on a smooth density one undoes the other."""
    k = 100.0
    fm, cdesc = _pair(lib, oracle, "kite", k, 128)
    fm.compute_precomputations(k)
    fm.spectral_setup(0.25)
    M = SpectralPreconditioner([cdesc], 16, k, eta=k, eps=0.25 * k ** (1 / 3))
    r = oracle.seeded_density(fm.total_num_unknowns_, seed=6) - (0.5 + 0.5j)
    for name, which in (("magnitude", 1), ("inverse_magnitude", 2)):
        assert rel(fm.spectral_symbol(r, name), M(r, which)) < TOL_APPLY
    t = cdesc[4]
    v = np.exp(3j * t) + 0.5 * np.cos(7 * t) + 0.2j * np.sin(20 * t)
    w = fm.spectral_symbol(fm.spectral_symbol(v, "magnitude"), "inverse_magnitude")
    assert rel(w, v) < 1e-4


def test_gpu_spectral_direct_config1(lib, oracle):
    """Config 1 (unit circle, k = 10, N = 200, direct operator, GMRES to 1e-10): flexible GMRES
    with the spectral preconditioner on the O(N^2) operator reaches the tolerance in fewer
    iterations than plain GMRES and matches the oracle's solution."""
    k = 10.0
    fm = lib.ForwardMap(0.01, [lib.Circle()], (), 1.0, k, Np=10, patches_per_curve=20, formulation="combined")
    fm.compute_precomputations(k)
    b = -np.exp(1j * k * fm.xs_)
    x0 = fm.gmres(b, accelerated=False, tol=1e-10)
    it0 = fm.last_solve["iters"]
    x1 = fm.solve_flexible(b, "spectral", accelerated=False, tol=1e-10)
    assert fm.last_solve["converged"] and fm.last_solve["iters"] < it0
    assert np.linalg.norm(fm.compute_Ax_unacc(x1) - b) / np.linalg.norm(b) < 1e-10
    assert rel(x1, x0) < 1e-8


def test_gpu_solve_preconditioned_wrapper(lib):
    """ForwardMap.solve_preconditioned: set-up and the chosen-form solve in one call."""
    k = 200.0
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=208, formulation="combined")
    b = -np.exp(1j * k * fm.xs_)
    x = fm.solve_preconditioned(b, k, tol=1e-6)
    assert fm.last_solve["converged"]
    assert np.linalg.norm(fm.compute_Ax_acc(x) - b) / np.linalg.norm(b) < 1e-6
