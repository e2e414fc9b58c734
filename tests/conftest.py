"""pytest configuration: the `gpu` marker and import paths.

CPU tests (``-m "not gpu"``) check the oracle against golden vectors, the host-side
discretisation against the oracle and the C-ABI library's exports.  GPU tests (``-m gpu``)
are the parity tests proper: they call libifgf2d through the C ABI and compare with the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib():
    import ifgf2d_gb300 as G
    G.load_library()
    return G
