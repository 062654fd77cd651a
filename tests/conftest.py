"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on the CPU.

The session builds the product library and the oracle if they are missing (the
same step as __graft_entry__.build()), so a fresh checkout can run the suite.
"""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 machine)")


def _ensure_built():
    lib = os.path.join(ROOT, "sci-solver_eikonal_gb300", "libeikonal_gb300.so")
    orc = os.path.join(ROOT, "oracle", "liboracle.so")
    if not (os.path.exists(lib) and os.path.exists(orc)):
        import __graft_entry__
        __graft_entry__.build()


_ensure_built()


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def eik():
    return importlib.import_module("sci-solver_eikonal_gb300")


@pytest.fixture(scope="session")
def mg():
    return importlib.import_module("sci-solver_eikonal_gb300.meshgen")


@pytest.fixture(scope="session")
def O():
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(GOLDEN, "meshes.npz"))


@pytest.fixture(scope="session")
def ref_outputs():
    p = os.path.join(GOLDEN, "ref_gpu_outputs.npz")
    if not os.path.exists(p):
        pytest.skip("reference-kernel fixtures not generated")
    return np.load(p)


@pytest.fixture
def need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def relerr(got, want, floor=1e-6):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return np.abs(got - want) / np.maximum(np.abs(want), floor)


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))
