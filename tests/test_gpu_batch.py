"""Batched apply and solve (many right-hand sides, one operator) -- needs a GPU.

Each column of a batched result is checked against the single-vector path of the same
operator (which the parity tests pin to the oracle) and, for one column per case, against the
oracle itself.  Tolerances: FP64 batched apply within 1e-13 of the single apply (the same
terms, summed in another order); complex64 batched apply within 2e-6 of the FP64 apply, as the
single mixed apply; batched solves reach the FP64 tolerance per column.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _kite(lib, k, npatch, form="combined"):
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=npatch, formulation=form)
    fm.precomps_and_setup(k, 0)
    return fm


def _densities(oracle, n, nrhs):
    return np.stack([oracle.seeded_density(n, seed=s) for s in range(nrhs)], axis=1)


def _plane_waves(fm, k, nrhs):
    ang = 2 * np.pi * np.arange(nrhs) / nrhs
    return -np.exp(1j * k * (np.cos(ang)[None, :] * fm.xs_[:, None] + np.sin(ang)[None, :] * fm.ys_[:, None]))


@pytest.mark.parametrize("form,nrhs", [("combined", 5), ("combined", 70), ("single_layer", 33)])
def test_gpu_batch_apply_matches_single(lib, oracle, form, nrhs):
    k = 100.0
    fm = _kite(lib, k, 128, form)
    n = fm.total_num_unknowns_
    X = _densities(oracle, n, nrhs)
    Y = fm.apply_batch(X)
    Ym = fm.apply_batch(X, mixed=True)
    for r in range(nrhs):
        y = fm.compute_Ax_acc(X[:, r])
        assert rel(Y[:, r], y) < 1e-13, r
        assert rel(Ym[:, r], y) < 2e-6, r
    # one column against the oracle's own IFGF apply on the same tree
    ocurve = oracle.curve_kite()
    om = oracle.OracleForwardMap([ocurve], 16, 0.01, 1.0, k, patches_per_curve=128, formulation=form)
    om.precompute(k)
    om.setup_ifgf(k, fm.nlevels)
    c = nrhs // 2
    tol = 1e-6 if form == "combined" else 1e-11   # combined: the one-ulp sensitivity of its singular weights
    assert rel(Y[:, c], om.compute_Ax_acc(X[:, c])) < tol


@pytest.mark.parametrize("k,npatch,nrhs", [(100.0, 128, 64), (300.0, 384, 13), (40.0, 64, 1)])
def test_gpu_batch_tensor_core_kernels(lib, oracle, k, npatch, nrhs):
    """The batched complex64 kernels on the tcgen05 tensor cores (leaf cones in 3xTF32 and with
    three TF32 terms per operand, propagation in 3xTF32, leaf and propagation) against the FP32
    FMA kernels and the FP64 apply: every complex64 form within 2e-6 of FP64 and within 1.5e-6 of
    the FMA form (FP32-level agreement; a single TF32 product would give ~1e-3); repeated
    applies are bit-identical.  The FMA propagation with TMA-staged child coefficients is
    bit-identical to the one with global loads."""
    fm = _kite(lib, k, npatch)
    n = fm.total_num_unknowns_
    X = _densities(oracle, n, nrhs)
    Y = fm.apply_batch(X)
    fm.batch_tensor_cores = 0
    Yf = fm.apply_batch(X, mixed=True)
    # the FMA propagation with TMA-staged child coefficients does the same arithmetic in the same
    # order (B even; an odd batch falls back to the global-load kernel)
    fm.batch_tensor_cores = fm.BATCH_BULK_PROPAGATION
    assert np.array_equal(fm.apply_batch(X, mixed=True), Yf)
    for mask in (fm.BATCH_TC_LEAF, fm.BATCH_TC_LEAF_FP32, fm.BATCH_TC_PROPAGATION, fm.BATCH_TC_LEAF | fm.BATCH_TC_PROPAGATION,
                 fm.BATCH_GROUPED_INTERP, fm.BATCH_GROUPED_INTERP | fm.BATCH_TC_LEAF):
        fm.batch_tensor_cores = mask
        assert fm.batch_tensor_cores == mask
        Yt = fm.apply_batch(X, mixed=True)
        assert np.array_equal(fm.apply_batch(X, mixed=True), Yt)
        for r in range(nrhs):
            assert rel(Yt[:, r], Y[:, r]) < 2e-6, (mask, r)
            assert rel(Yf[:, r], Y[:, r]) < 2e-6, (mask, r)
            assert rel(Yt[:, r], Yf[:, r]) < 1.5e-6, (mask, r)


def test_gpu_batch_apply_direct_and_device(lib, oracle):
    import torch
    k = 40.0
    fm = _kite(lib, k, 64)
    n = fm.total_num_unknowns_
    X = _densities(oracle, n, 3)
    Yd = fm.apply_batch(X, accelerated=False)
    for r in range(3):
        assert np.array_equal(Yd[:, r], fm.compute_Ax_unacc(X[:, r]))
    # device entry point: column-major N x nrhs = a (nrhs, N) row-major tensor
    xt = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    yt = torch.empty_like(xt)
    fm.apply_batch_device(xt, yt, 3)
    torch.cuda.synchronize()
    Y = fm.apply_batch(X)
    assert np.array_equal(yt.cpu().numpy().T, Y)


def test_gpu_batch_apply_edge_cases(lib, oracle):
    k = 40.0
    fm = _kite(lib, k, 64)
    n = fm.total_num_unknowns_
    L = lib._lib.load()
    # nrhs = 0 is a no-op, negative is an argument error
    assert L.ifgf2d_apply_batch(fm.handle, None, None, 0, 1) == 0
    assert L.ifgf2d_apply_batch(fm.handle, None, None, -1, 1) == 1
    assert L.ifgf2d_apply_batch(fm.handle, None, None, 2, 1) == 1
    # a zero column stays zero and leaves the others untouched
    X = _densities(oracle, n, 4)
    X[:, 2] = 0
    Y = fm.apply_batch(X)
    assert np.all(Y[:, 2] == 0)
    assert rel(Y[:, 1], fm.compute_Ax_acc(X[:, 1])) < 1e-13
    # a single column through the batched path
    assert rel(fm.apply_batch(X[:, 0])[:, 0], fm.compute_Ax_acc(X[:, 0])) < 1e-13


def test_gpu_batch_solve_matches_single(lib):
    """Plane waves at 6 incidence angles: FP64 GMRES in lock step gives each column's own
    iterates (same Krylov space as the single solve)."""
    k = 100.0
    fm = _kite(lib, k, 128)
    B = _plane_waves(fm, k, 6)
    X = fm.gmres_batch(B, tol=1e-10, restart=300, max_iters=500)
    st = fm.last_solve
    assert st["converged"]
    for r in range(B.shape[1]):
        x = fm.gmres(B[:, r], tol=1e-10, restart=300, max_iters=500)
        assert abs(st["iters"][r] - fm.last_solve["iters"]) <= 1, r
        assert rel(X[:, r], x) < 1e-8, r
        assert rel(fm.compute_Ax_acc(X[:, r]), B[:, r]) < 1e-9, r


def test_gpu_batch_solve_restart_and_zero_column(lib):
    """Short restart cycles (the restart path) and a zero right-hand side in the batch."""
    k = 40.0
    fm = _kite(lib, k, 64)
    B = _plane_waves(fm, k, 4)
    B[:, 3] = 0
    X = fm.gmres_batch(B, tol=1e-9, restart=7, max_iters=600)
    st = fm.last_solve
    assert st["converged"]
    assert np.all(X[:, 3] == 0) and st["iters"][3] == 0
    for r in range(3):
        assert rel(fm.compute_Ax_acc(X[:, r]), B[:, r]) < 1e-8, r
        x = fm.gmres(B[:, r], tol=1e-9, restart=7, max_iters=600)
        assert rel(X[:, r], x) < 1e-6, r


def test_gpu_batch_mixed_solve_compacted_passes(lib):
    """Refinement passes that run on a subset of the columns (gathered into a compact batch):
    a zero column is converged from the start, and a tolerance below the complex64 operator's
    accuracy needs several FP64 passes.  Each other column reaches the FP64 tolerance and
    agrees with its own single-vector refinement solve."""
    k = 40.0
    fm = _kite(lib, k, 64)
    B = _plane_waves(fm, k, 5)
    B[:, 2] = 0
    X = fm.gmres_batch(B, tol=1e-9, restart=300, max_iters=2000, mixed=True)
    st = fm.last_solve
    assert st["converged"] and st["refinements"] >= 2
    assert np.all(X[:, 2] == 0) and st["iters"][2] == 0
    R = fm.apply_batch(X) - B
    for r in (0, 1, 3, 4):
        assert np.linalg.norm(R[:, r]) / np.linalg.norm(B[:, r]) < 1e-9, r
        x = fm.gmres(B[:, r], tol=1e-9, restart=300, max_iters=2000, mixed=True)
        assert fm.last_solve["refinements"] >= 2
        assert rel(X[:, r], x) < 1e-7, r


def test_gpu_batch_mixed_solve_reaches_fp64_tolerance(lib):
    """FP64 refinement around batched complex64 inner solves: every column's FP64 residual
    below 1e-6 (plane waves at 8 angles, kite k = 500, N = 8192)."""
    k = 500.0
    fm = _kite(lib, k, 512)
    B = _plane_waves(fm, k, 8)
    X = fm.gmres_batch(B, tol=1e-6, restart=300, max_iters=1000, mixed=True)
    assert fm.last_solve["converged"]
    R = fm.apply_batch(X) - B
    for r in range(B.shape[1]):
        assert np.linalg.norm(R[:, r]) / np.linalg.norm(B[:, r]) < 1e-6, r
