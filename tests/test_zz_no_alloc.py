"""ifgf2d_apply_direct_noalloc: the direct forward map with no device allocation in the call.

Some callers cannot allocate device memory where they call the forward map (a host
application that owns the device memory budget, or a latency-critical loop that cannot take
cudaMalloc's implicit synchronisation).  This entry point keeps its scratch in a fixed array
inside the library; its output must equal the allocating path's, call after call, and the
device's free memory must not move across a call.  This file is collected last so that a
stop-at-first-failure run has already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the direct forward map's parity tolerance
IFGF2D_ERR_ARG = 1


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("geometry", ["circle_k10_n200", "kite_k100_n2048"])
def test_noalloc_direct_map_matches_allocating_path(lib, oracle, geometry):
    torch = pytest.importorskip("torch")
    if geometry == "circle_k10_n200":
        k, fm = 10.0, lib.ForwardMap(0.01, [lib.Circle()], (), 1.0, 10.0, Np=10, patches_per_curve=20)
    else:
        k, fm = 100.0, lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, 100.0, Np=16, patches_per_curve=128)
    fm.compute_precomputations(k)      # set-up resolves the scratch array and loads the kernels
    L = lib._lib.load()
    n = fm.total_num_unknowns_
    outs = []
    for seed in (0, 1):   # two calls in a row, different densities
        x = torch.from_numpy(oracle.seeded_density(n, seed=seed)).cuda()
        y_ref = torch.empty_like(x)
        y_new = torch.full_like(x, float("nan"))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = L.ifgf2d_apply_direct_noalloc(fm.handle, x.data_ptr(), y_new.data_ptr())
        assert rc == 0, L.ifgf2d_last_error(fm.handle).decode()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before, "the call changed the device's free memory"
        fm.apply_device(x, y_ref, accelerated=False)
        torch.cuda.synchronize()
        a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert _rel(a, b) < TOL
        outs.append(a)
    assert _rel(outs[0], outs[1]) > 1e-3   # the second call did not reuse the first result


def test_noalloc_rejects_sizes_beyond_its_maximum(lib):
    torch = pytest.importorskip("torch")
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, 500.0, Np=16, patches_per_curve=4097)
    assert fm.total_num_unknowns_ == 65552   # > IFGF2D_NOALLOC_MAX_N = 65536
    fm.compute_precomputations(500.0)
    L = lib._lib.load()
    x = torch.zeros(fm.total_num_unknowns_, dtype=torch.complex128, device="cuda")
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    rc = L.ifgf2d_apply_direct_noalloc(fm.handle, x.data_ptr(), y.data_ptr())
    assert rc == IFGF2D_ERR_ARG
    assert "IFGF2D_NOALLOC_MAX_N" in L.ifgf2d_last_error(fm.handle).decode()
