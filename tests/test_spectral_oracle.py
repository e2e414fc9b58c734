"""CPU pin of the spectral preconditioner's oracle (oracle/spectral_oracle.py).

On the unit circle the flat-boundary symbol's Fourier modes are the curve's own: a sampled
mode e^{i n t} must come back multiplied by 1/sigma(n), up to the resampling's interpolation
error, which grows with n as the uniform grid's points per wavelength fall."""
import numpy as np
import pytest

from oracle.spectral_oracle import CURVE_CIRCLE, CURVE_KITE, CurveTables, SpectralPreconditioner, curve_speed


def _circle(oracle, k, patches):
    om = oracle.OracleForwardMap([oracle.curve_circle()], 16, 0.01, 1.0, k, patches_per_curve=patches,
                                 formulation="combined", coupling=k)
    t12, _ = om.patch_info()
    fn = np.cos(np.pi * (2 * np.arange(16) + 1) / 32)
    tp = (t12[:, 0][:, None] + (fn[None, :] + 1) * 0.5 * (t12[:, 1] - t12[:, 0])[:, None]).ravel()
    return t12, tp


@pytest.mark.parametrize("n,tol", [(0, 1e-14), (5, 1e-13), (40, 1e-7), (51, 1e-6), (80, 1e-5), (120, 1e-4)])
def test_oracle_spectral_circle_modes(oracle, n, tol):
    k = 50.0
    t12, tp = _circle(oracle, k, 64)
    eps = 0.25 * k ** (1 / 3)
    M = SpectralPreconditioner([(CURVE_CIRCLE, [0.0, 0.0, 1.0], t12[:, 0], t12[:, 1], tp)], 16, k, eta=k, eps=eps)
    r = np.exp(1j * n * tp)
    ke = k + 1j * eps
    sig = 0.5 + k / (2 * np.sqrt(ke * ke - n * n + 0j))
    z = M(r)
    assert np.linalg.norm(z - r / sig) / np.linalg.norm(r / sig) < tol


def test_oracle_spectral_arc_length_of_the_kite(oracle):
    """The tables' curve length equals an independent fine trapezoid sum of |x'(t)|, and the
    uniform grid's back-interpolation reproduces smooth functions of arc length."""
    k = 100.0
    om = oracle.OracleForwardMap([oracle.curve_kite()], 16, 0.01, 1.0, k, patches_per_curve=128,
                                 formulation="combined", coupling=k)
    t12, _ = om.patch_info()
    fn = np.cos(np.pi * (2 * np.arange(16) + 1) / 32)
    tp = (t12[:, 0][:, None] + (fn[None, :] + 1) * 0.5 * (t12[:, 1] - t12[:, 0])[:, None]).ravel()
    sp = curve_speed(CURVE_KITE, [1.0, 0.65, -0.65, 1.5])
    tb = CurveTables(sp, t12[:, 0], t12[:, 1], tp, 16)
    t = np.linspace(0, 2 * np.pi, 200001)
    L = np.trapezoid(sp(t), t)
    assert abs(tb.L - L) < 1e-9 * L
    # a smooth periodic function of arc length, sampled on the grid, read back at the nodes
    f = lambda s: np.exp(1j * 2 * np.pi * 7 * s / tb.L)
    u = f(tb.L * np.arange(tb.nu) / tb.nu)
    assert np.max(np.abs(tb.back(u) - f(tb.s_nodes))) < 1e-9
    # and the forward resampling reads node values of the same function at the grid points
    g = tb.forward(f(tb.s_nodes))
    assert np.max(np.abs(g - u)) < 1e-9
