"""Host-side logic and the C ABI without a GPU (CPU only).

The discretisation (ForwardMap constructor) is host C++ inside libifgf2d.so; it must match
the oracle bit for bit.  The library must load and export every symbol of include/ifgf2d.h.
"""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(lib):
    from ifgf2d_gb300 import _lib
    header = open(os.path.join(ROOT, "include", "ifgf2d.h")).read()
    declared = set(re.findall(r"\b(ifgf2d_[a-z0-9_]+)\s*\(", header))
    assert declared == set(_lib.EXPORTS)
    L = ctypes.CDLL(_lib.library_path())
    for name in declared:
        assert hasattr(L, name), name


CASES = [
    ("circle", lambda G: G.Circle(), lambda O: O.curve_circle(), (10, 0.01, 0.5, 10.0, 4.0, 0)),
    ("circle20", lambda G: G.Circle(), lambda O: O.curve_circle(), (10, 0.01, 1.0, 10.0, 4.0, 20)),
    ("kite500", lambda G: G.Kite(), lambda O: O.curve_kite(), (16, 0.01, 1.0, 500.0, 4.0, 512)),
    ("kite_rule", lambda G: G.Kite(), lambda O: O.curve_kite(), (16, 0.01, 1.0, 100.0, 4.0, 0)),
    ("line", lambda G: G.Line(-1, -0.2, 1, -0.2), lambda O: O.curve_line(-1, -0.2, 1, -0.2), (20, 0.1, 0.5, 3.0, 6.0, 0)),
    ("star", lambda G: G.Star([0.03, -0.02, 0.01], [0.01, 0.04, -0.03]),
     lambda O: O.curve_star([0.03, -0.02, 0.01], [0.01, 0.04, -0.03]), (16, 0.01, 1.0, 50.0, 4.0, 0)),
]


@pytest.mark.parametrize("name,gc,oc,args", CASES, ids=[c[0] for c in CASES])
def test_discretisation_matches_oracle_bitwise(lib, oracle, name, gc, oc, args):
    Np, delta, wl, k, p, ppc = args
    fm = lib.ForwardMap(delta, [gc(lib)], (), wl, k, p, Np=Np, patches_per_curve=ppc)
    om = oracle.OracleForwardMap([oc(oracle)], Np, delta, wl, k, p, patches_per_curve=ppc)
    assert fm.total_num_unknowns_ == om.N and fm.num_patches_ == om.num_patches
    xs, ys, nx, ny = om.points()
    for a, b in ((fm.xs_, xs), (fm.ys_, ys), (fm.nxs_, nx), (fm.nys_, ny)):
        assert np.array_equal(a, b)
    t_g, c_g = fm.patches()
    t_o, c_o = om.patch_info()
    assert np.array_equal(t_g, t_o) and np.array_equal(c_g, c_o)
    _, i_g, tv_g = fm.near_singular()
    _, i_o, tv_o = om.near_singular()
    assert np.array_equal(i_g, i_o) and np.array_equal(tv_g, tv_o)


def test_bad_arguments_raise(lib):
    with pytest.raises(ValueError):
        lib.ForwardMap(0.01, [], (), 1.0, 10.0, Np=10)
    with pytest.raises(ValueError):
        lib.ForwardMap(-1.0, [lib.Circle()], (), 1.0, 10.0, Np=10)
    with pytest.raises(ValueError):
        lib.ForwardMap(0.01, [lib.Circle()], (), 1.0, 10.0, Np=1)
    with pytest.raises(ValueError):
        lib.Star([0.1] * 7, [0.0] * 7)


def test_apply_before_setup_is_a_state_error(lib):
    fm = lib.ForwardMap(0.01, [lib.Circle()], (), 1.0, 10.0, Np=10)
    with pytest.raises(lib.IFGF2DError):
        fm.compute_Ax_acc(np.ones(fm.total_num_unknowns_, complex))


def test_rectangle_junctions_discretise(lib, oracle):
    """make_rect (Geometry/Obstacles.cpp:6-23): four lines joined by junctions."""
    c1x, c1y, c2x, c2y = -0.5, 0.5, 0.5, -0.5
    lines = [(c2x, c2y, c2x, c1y), (c2x, c1y, c1x, c1y), (c1x, c1y, c1x, c2y), (c1x, c2y, c2x, c2y)]
    junc = [(0, 1, 0), (0, 3, 0), (1, 0, 0), (1, 2, 0), (2, 1, 0), (2, 3, 0), (3, 2, 0), (3, 0, 0)]
    fm = lib.ForwardMap(0.05, [lib.Line(*l) for l in lines], [lib.Junction(*j) for j in junc], 1.0, 5.0, 4.0, Np=10)
    om = oracle.OracleForwardMap([oracle.curve_line(*l) for l in lines], 10, 0.05, 1.0, 5.0, 4.0, junctions=junc)
    assert np.array_equal(fm.xs_, om.points()[0])
    _, i_g, _ = fm.near_singular()
    _, i_o, _ = om.near_singular()
    assert np.array_equal(i_g, i_o)


def test_star_obstacle_configuration():
    """The seeded multi-obstacle configuration: 256 stars, k in [10, 400], 10 points per
    wavelength rounded up to whole 16-point patches, reproducible from the seed."""
    from ifgf2d_gb300.scatterers import star_obstacles, star_perimeter
    a = star_obstacles(256)
    b = star_obstacles(256)
    assert len(a) == 256
    for o, p in zip(a, b):
        assert o.k == p.k and o.angle == p.angle and np.array_equal(o.a, p.a)
        assert 10.0 <= o.k <= 400.0 and np.all(np.abs(o.a) <= 0.05) and np.all(np.abs(o.b) <= 0.05)
        L = star_perimeter(o.a, o.b)
        assert o.npoints % 16 == 0 and o.npoints >= 10 * o.k * L / (2 * np.pi) > o.npoints - 16
    # the unperturbed star is the unit circle
    assert abs(star_perimeter(np.zeros(5), np.zeros(5)) - 2 * np.pi) < 1e-12


def test_prepare_builds_the_oracle_tree_without_a_gpu(lib, oracle):
    """ifgf2d_prepare is host-only: on a machine without a GPU it builds the tree, whose Morton
    sorting and work counts equal the oracle's (BoxTree.h:61-600, Level.h), with one set-up
    thread or all of them."""
    k = 40.0
    L = lib._lib.load()
    om = oracle.OracleForwardMap([oracle.curve_kite()], 16, 0.01, 1.0, k, patches_per_curve=64)
    seen = []
    for threads in (1, 0):
        assert L.ifgf2d_set_host_threads(threads) == 0
        fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=64)
        fm.prepare(k, 0)
        nl = int(L.ifgf2d_get_nlevels(fm.handle))
        om.setup_ifgf(k, nl)
        assert np.array_equal(fm.getSorting(), om.sorting())
        wc, ow = fm.work_counts(), om.work()
        for key in ("near_pairs", "leaf_evals", "prop_evals", "interp_evals", "cones"):
            assert wc[key] == ow[key], key
        seen.append((nl, fm.getSorting().tobytes(), tuple(sorted(wc.items()))))
        # the device tables do not exist yet: applies report the state, before any copy
        with pytest.raises(lib.IFGF2DError):
            fm.compute_Ax_acc(np.ones(fm.total_num_unknowns_, dtype=complex))
    assert seen[0] == seen[1]
    assert L.ifgf2d_set_host_threads(-1) == 1


@pytest.mark.parametrize("k,patches", [(500.0, 512), (2000.0, 2048), (8000.0, 8192)],
                         ids=["kite_k500_N8192", "kite_k2000_N32768", "kite_k8000_N131072"])
def test_prepare_tree_equals_oracle_at_full_size(lib, oracle, k, patches):
    """The benchmark kites at their full sizes (N = 8192, 32768, 131072; trees of depth 7, 8
    and 10): the host tree's depth choice, Morton sorting and per-apply work counts (near pairs,
    leaf-cone, propagation and interpolation evaluations, relevant cones) equal the oracle's
    BoxTree (BoxTree.h:61-600; cone counts per level from Level.h:88-142).  A cone or
    relevant-box rule that differs only at high k * box size shows here, without a GPU."""
    L = lib._lib.load()
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=patches)
    fm.prepare(k, 0)
    nl = int(L.ifgf2d_get_nlevels(fm.handle))
    om = oracle.OracleForwardMap([oracle.curve_kite()], 16, 0.01, 1.0, k, patches_per_curve=patches)
    om.setup_ifgf(k, nl)
    with pytest.raises(RuntimeError, match="neighborhood"):
        om.setup_ifgf(k, nl + 1)      # the depth is the deepest one the oracle accepts
    om.setup_ifgf(k, nl)
    assert np.array_equal(fm.getSorting(), om.sorting())
    wc, ow = fm.work_counts(), om.work()
    for key in ("near_pairs", "leaf_evals", "prop_evals", "interp_evals", "cones"):
        assert wc[key] == ow[key], key
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=64)
    assert L.ifgf2d_prepare(fm.handle, k, 2) == 4          # IFGF2D_ERR_NLEVELS, BoxTree.h:1117
    assert L.ifgf2d_prepare(fm.handle, -1.0, 0) == 1


def test_group_create_checks_its_members_before_any_gpu_work(lib):
    """ifgf2d_group_create rejects a NULL or empty member list, an unprepared member and members
    of different Np / Ps / Pang / formulation with a status and a message, before it touches the
    GPU, and the half-built group is destroyed cleanly."""
    L = lib._lib.load()
    h = ctypes.c_void_p()
    assert L.ifgf2d_group_create(None, 1, ctypes.byref(h)) == 1
    arr = (ctypes.c_void_p * 1)()
    assert L.ifgf2d_group_create(arr, 0, ctypes.byref(h)) == 1
    assert L.ifgf2d_group_create(arr, 1025, ctypes.byref(h)) == 1
    with pytest.raises(ValueError):
        lib.Group([])
    kite = lambda k, **kw: lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, **{"Np": 16, "patches_per_curve": 128,
                                                                           "formulation": "combined", **kw})
    a, b = kite(100.0), kite(150.0)
    with pytest.raises(lib.IFGF2DError, match="prepared"):
        lib.Group([a, b])                       # neither member prepared
    a.prepare(100.0, 0)
    c = kite(150.0, Np=10)
    c.prepare(150.0, 0)
    with pytest.raises(ValueError, match="Np"):
        lib.Group([a, c])                       # different Np
    d = kite(150.0, formulation="single_layer")
    d.prepare(150.0, 0)
    with pytest.raises(ValueError, match="formulation"):
        lib.Group([a, d])                       # different formulation


@pytest.mark.filterwarnings("ignore:This process .* is multi-threaded:DeprecationWarning")
def test_host_threads_after_fork(lib):
    """The host loops run on a pool of worker threads kept for the process.  A child forked
    after the pool started has none of its workers; its set-up must still run, on threads of its
    own, and give the same tree."""
    import os
    import signal
    import time
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, 300.0, Np=16, patches_per_curve=320)
    fm.prepare(300.0, 0)
    before = fm.getSorting()
    pid = os.fork()
    if pid == 0:   # child: a second set-up on the inherited pool state
        code = 1
        try:
            fm.prepare(300.0, 0)
            code = 0 if (fm.getSorting() == before).all() else 2
        finally:
            os._exit(code)
    deadline = time.time() + 120
    while True:
        done, status = os.waitpid(pid, os.WNOHANG)
        if done:
            break
        if time.time() > deadline:
            os.kill(pid, signal.SIGKILL)
            os.waitpid(pid, 0)
            raise AssertionError("the forked child's set-up did not finish")
        time.sleep(0.05)
    assert os.WIFEXITED(status) and os.WEXITSTATUS(status) == 0


def test_host_threads_concurrent_setups(lib):
    """Host set-ups from several threads at once: one runs its loops on the worker pool, the
    others find it busy and start threads of their own.  Every tree equals the one built alone."""
    from concurrent.futures import ThreadPoolExecutor
    ks = [150.0, 220.0, 300.0, 380.0, 260.0, 190.0]

    def build(k):
        fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, k, Np=16, patches_per_curve=int(1.024 * k) + 16)
        fm.prepare(k, 0)
        return fm.getSorting().tobytes(), tuple(sorted(fm.work_counts().items()))

    alone = [build(k) for k in ks]
    with ThreadPoolExecutor(len(ks)) as ex:
        together = list(ex.map(build, ks * 2))
    assert together == alone * 2
