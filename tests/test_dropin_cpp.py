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
    y = np.fromfile(out, dtype=np.complex128)
    fm = lib.ForwardMap(0.01, [lib.Kite()], (), 1.0, 100.0, 4.0, Np=16, patches_per_curve=64)
    fm.precomps_and_setup(100.0, 0)
    j = np.arange(fm.total_num_unknowns_)
    x = np.cos(0.1 * j) + 1j * np.sin(0.2 * j)
    n = fm.total_num_unknowns_
    assert np.array_equal(y[:n], fm.compute_Ax_acc(x))
    assert np.array_equal(y[n:], fm.compute_Ax_unacc(x))
