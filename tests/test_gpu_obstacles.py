"""Many independent obstacles (ifgf2d_gb300.scatterers) -- needs a GPU.

Every obstacle of the seeded star configuration reaches the FP64 tolerance through the
pipelined driver (host set-up on worker threads, device work on one or more device threads),
and the pipelined solutions equal those of a plain one-at-a-time run of the same code path.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("device_threads", [1, 3])
def test_gpu_obstacles_pipelined_match_sequential(lib, device_threads):
    """Pipelined (and, with device_threads > 1, several obstacles at once on their own streams)
    equals one at a time, bit for bit."""
    from ifgf2d_gb300.scatterers import star_obstacles, solve_obstacles
    obs = star_obstacles(12, seed=1, kmax=150.0)
    xs = solve_obstacles(obs, tol=1e-8, workers=4, mixed=False, keep_solutions=True, device_threads=device_threads)
    assert all(o.result["converged"] for o in obs)
    assert max(o.result["true_rel_residual"] for o in obs) < 1e-7
    ref = star_obstacles(12, seed=1, kmax=150.0)
    xr = solve_obstacles(ref, tol=1e-8, workers=0, mixed=False, keep_solutions=True)
    for a, b, o, r in zip(xs, xr, obs, ref):
        assert o.result["iters"] == r.result["iters"]
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()


def test_gpu_obstacles_mixed_reach_tolerance(lib):
    from ifgf2d_gb300.scatterers import star_obstacles, solve_obstacles
    obs = star_obstacles(16, seed=2)
    solve_obstacles(obs, tol=1e-6, workers=4, mixed=True, device_threads=2)
    assert all(o.result["converged"] for o in obs)
    assert max(o.result["true_rel_residual"] for o in obs) < 1e-6
    # the seeded configuration: N_i = 16 ceil(10 k L / 2 pi / 16)
    assert all(o.npoints % 16 == 0 and o.result["N"] == o.npoints for o in obs)
