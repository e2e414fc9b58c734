"""The C++ drop-in header (include/ifgf2d/ForwardMap.hpp): a program written against the
reference's ForwardMap interface compiles, links against libifgf2d.so (CPU test) and
reproduces the library's results (GPU test)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_check.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build")


def _build(lib):
    from ifgf2d_gb300 import build as b
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "dropin_check")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-L", b.OUT, "-lifgf2d",
           f"-Wl,-rpath,{b.OUT}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_dropin_header_compiles_and_links(lib):
    exe = _build(lib)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_dropin_program_matches_library(lib, tmp_path):
    exe = _build(lib)
    out = tmp_path / "y.bin"
    r = subprocess.run([exe, str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, dtype=np.uint8)
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, 100.0, 4.0, Np=16, patches_per_curve=64)
    fm.precomps_and_setup(100.0, 0)
    n = fm.total_num_unknowns_
    y = raw[:16 * 6 * n].view(np.complex128)
    meta = raw[16 * 6 * n:].view(np.float64)
    j = np.arange(n)
    x = np.cos(0.1 * j) + 1j * np.sin(0.2 * j)
    assert np.array_equal(y[:n], fm.compute_Ax_acc(x))
    assert np.array_equal(y[n:2 * n], fm.compute_Ax_unacc(x))
    # GMRES three ways on the combined-field operator: a user mapping under opGMRES (host
    # Arnoldi, GPU applies), the bound operator under opGMRES (ifgf2d_solve) and ForwardMap::solve
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, 100.0, 4.0, Np=16, patches_per_curve=64, formulation="combined")
    fm.precomps_and_setup(100.0, 0)
    b = -np.exp(1j * 100.0 * fm.xs_)
    x_user, x_dev, x_solve, x_pre = y[2 * n:3 * n], y[3 * n:4 * n], y[4 * n:5 * n], y[5 * n:6 * n]
    it_user, err_user, it_dev, err_dev, it_solve, err_solve, it_pre, err_pre = meta
    for xs, err in ((x_user, err_user), (x_dev, err_dev), (x_solve, err_solve)):
        assert err < 1e-8
        assert np.linalg.norm(fm.compute_Ax_acc(xs) - b) / np.linalg.norm(b) < 1e-7
    assert abs(it_user - it_dev) <= 1 and it_dev == it_solve
    assert np.linalg.norm(x_user - x_dev) / np.linalg.norm(x_dev) < 1e-6
    assert np.linalg.norm(x_dev - x_solve) / np.linalg.norm(x_solve) < 1e-10   # the same device solve, run twice
    # ForwardMap::solve_preconditioned (not in the reference): mixed precision, FP64 refinement
    # and the spectral preconditioner reach the same FP64 tolerance in fewer iterations
    assert err_pre < 1e-8 and it_pre < it_solve
    assert np.linalg.norm(fm.compute_Ax_acc(x_pre) - b) / np.linalg.norm(b) < 1e-7
    assert np.linalg.norm(x_pre - x_solve) / np.linalg.norm(x_solve) < 1e-6
