"""Shared test set-up: import paths, the `gpu` marker, fixture helpers."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "landau-poisson-solver-2d_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the CUDA library")


GOLDEN_NAMES = ["ref_n8", "ref_n16", "ref_n24"]


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_case(g):
    from oracle.oracle import Case
    nx1, nx2, nv, n = [int(x) for x in g["case"]]
    lv, lx, nu, dt, a, k = [float(x) for x in g["case_f"]]
    return Case(nx1=nx1, nx2=nx2, nv=nv, n=n, lv=lv, lx=lx, nu=nu, dt=dt, a_amp=a, k_wave=k)


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if stale) and loads the CUDA library; raises when it cannot."""
    sys.path.insert(0, PKG)
    import build as pkg_build  # landau-poisson-solver-2d_gb300/build.py
    pkg_build.build()
    import lp_gb300
    lp_gb300.lib()
    return lp_gb300
