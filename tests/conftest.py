"""Shared fixtures.  `-m "not gpu"` runs everywhere; `-m gpu` needs a GB300."""
from __future__ import annotations

import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "giant-impact_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")

for _p in (ORACLE, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103) device")


def load_gi():
    if "gi" in sys.modules:
        return sys.modules["gi"]
    spec = importlib.util.spec_from_file_location("gi", os.path.join(PKG, "gi.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["gi"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def built():
    """Build (incrementally) libgi, the oracle and the reference kernels."""
    spec = importlib.util.spec_from_file_location("gi_build", os.path.join(PKG, "gi_build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b.build_all()


@pytest.fixture(scope="session")
def gi(built):
    return load_gi()


@pytest.fixture(scope="session")
def orc(built):
    import oracle
    return oracle


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def config1_params(gi):
    """Material of the 8,192-body settle workload: G = D = 1, mFe = 1, mSi = 0.4,
    KFe = 5, KSi = 1.5, KR 0.02 / 0.01, shell depth 0.002 / 0.001."""
    return gi.params_from_material(1.0, 1.0, 1.0, 0.4, 5.0, 1.5, 0.02, 0.01, 0.002, 0.001)


def reference_unit_params(gi):
    """The same material in the reference's normalisation (mSi = 1):
    mass / 0.4, K / 0.4^2 (time scaled by sqrt(0.4))."""
    mu = 0.4
    return gi.params_from_material(1.0, 1.0, 1.0 / mu, 1.0, 5.0 / mu**2, 1.5 / mu**2, 0.02, 0.01,
                                   0.002, 0.001)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
