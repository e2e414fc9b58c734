"""The constructor's discretisation on the GPU (ForwardMap(..., device_geometry=True)) against
the host discretisation, which is bit-exact with the oracle (test_host_and_abi.py) -- needs a GPU.

ForwardMap.tpp:37-285: points, unit normals and quadrature factors per Fejer node
(Curve.hpp:97-102, Quadrature.hpp:151-173 on open curves), bounding boxes (Patch.tpp:36-64) and
the near-singular points found by Brent's minimiser (BrentsMethod.hpp:42-156).  The device's
sin / cos / pow differ from glibc's in the last bits, so positions agree to a few ulps; Brent's
step sequence can branch differently on such a difference, so the near-singular parameters
agree to its stopping tolerance (1e-6 relative), and the set of near-singular points must be
the same.  The operator built on either discretisation then agrees to the quadrature's accuracy.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RECT_LINES = [(0.5, -0.5, 0.5, 0.5), (0.5, 0.5, -0.5, 0.5), (-0.5, 0.5, -0.5, -0.5), (-0.5, -0.5, 0.5, -0.5)]
RECT_JUNCTIONS = [(0, 1, 0), (0, 3, 0), (1, 0, 0), (1, 2, 0), (2, 1, 0), (2, 3, 0), (3, 2, 0), (3, 0, 0)]

CASES = {
    "kite_k500_N8192": (lambda G: ([G.Kite()], ()), dict(delta=0.01, wl=1.0, k=500.0, Np=16, ppc=512)),
    "kite_k8000_N131072": (lambda G: ([G.Kite()], ()), dict(delta=0.01, wl=1.0, k=8000.0, Np=16, ppc=8192)),
    "kite_arclength_rule": (lambda G: ([G.Kite()], ()), dict(delta=0.01, wl=1.0, k=100.0, Np=16, ppc=0)),
    "circle": (lambda G: ([G.Circle()], ()), dict(delta=0.01, wl=0.5, k=10.0, Np=10, ppc=0)),
    "star": (lambda G: ([G.Star([0.03, -0.02, 0.01], [0.01, 0.04, -0.03])], ()), dict(delta=0.01, wl=1.0, k=50.0, Np=16, ppc=0)),
    "open_line": (lambda G: ([G.Line(-1, -0.2, 1, -0.2)], ()), dict(delta=0.1, wl=0.5, k=3.0, Np=20, ppc=0, p=6.0)),
    "rectangle_junctions": (lambda G: ([G.Line(*l) for l in RECT_LINES], [G.Junction(*j) for j in RECT_JUNCTIONS]),
                            dict(delta=0.01, wl=1.0, k=40.0, Np=10, ppc=0)),
}


def _pair(lib, name):
    make, a = CASES[name]
    out = []
    for dev in (False, True):
        curves, junc = make(lib)
        out.append(lib.ForwardMap(a["delta"], curves, junc, a["wl"], a["k"], a.get("p", 4.0), Np=a["Np"],
                                  patches_per_curve=a["ppc"], device_geometry=dev))
    return out[0], out[1], a


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_device_geometry_matches_host(lib, name):
    host, dev, a = _pair(lib, name)
    assert dev.total_num_unknowns_ == host.total_num_unknowns_ and dev.num_patches_ == host.num_patches_
    th, ch = host.patches()
    td, cd = dev.patches()
    assert np.array_equal(td, th)                       # the patch limits are the host's in both
    scale = max(np.abs(host.xs_).max(), np.abs(host.ys_).max())
    for a_, b_ in ((dev.xs_, host.xs_), (dev.ys_, host.ys_)):
        assert np.abs(a_ - b_).max() <= 1e-14 * scale
    for a_, b_ in ((dev.nxs_, host.nxs_), (dev.nys_, host.nys_)):
        assert np.abs(a_ - b_).max() <= 1e-14
    gh, gd = host.geometry_features(), dev.geometry_features()   # curvature, tangent, quadrature factor
    assert np.abs(gd[:, 3] - gh[:, 3]).max() <= 1e-13 * np.abs(gh[:, 3]).max()
    assert np.abs(gd[:, 0] - gh[:, 0]).max() <= 1e-11 * max(1.0, np.abs(gh[:, 0]).max())
    # the same near-singular points, parameters within Brent's tolerance
    assert np.array_equal(cd, ch)
    _, ih, tvh = host.near_singular()
    _, idv, tvd = dev.near_singular()
    assert np.array_equal(idv, ih)
    if tvh.size:
        assert np.abs(tvd - tvh).max() <= 1e-6 * max(1.0, np.abs(tvh).max())


@pytest.mark.parametrize("name", ["kite_k500_N8192", "open_line", "rectangle_junctions"])
def test_gpu_device_geometry_operator_matches_host(lib, oracle, name):
    """The direct forward map built on the device discretisation equals the host-built one to
    the rectangular-polar quadrature's accuracy."""
    host, dev, a = _pair(lib, name)
    k = a["k"]
    host.compute_precomputations(k)
    dev.compute_precomputations(k)
    d = oracle.seeded_density(host.total_num_unknowns_)
    yh, yd = host.compute_Ax_unacc(d), dev.compute_Ax_unacc(d)
    assert np.linalg.norm(yd - yh) / np.linalg.norm(yh) < 1e-9
