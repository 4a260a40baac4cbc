"""The C ABI library builds for sm_103a, loads without a GPU and exports every
function that include/lp_gb300.h declares; the Python binding covers them."""
from __future__ import annotations

import ctypes
import os
import re

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "lp_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:lp_status|const char \*|size_t|int)\s*\*?\s*(lp_\w+)\s*\(",
                                 src, re.M)))


def test_header_declares_entry_points():
    names = _declared()
    assert "lp_compute_q" in names and "lp_step" in names and len(names) >= 20


def test_library_exports_declared_symbols(gpu_lib):
    L = ctypes.CDLL(gpu_lib.LIB_PATH)
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(gpu_lib.EXPORTS) == _declared()


def test_create_without_device_reports_status(gpu_lib):
    # Invalid parameters are rejected before any device work.
    P = gpu_lib.Params(nx1=0, nx2=1, nv=4, n=8)
    try:
        gpu_lib.Context(P)
    except gpu_lib.LPError as e:
        assert e.status in (gpu_lib.ERR_INVALID, gpu_lib.ERR_NO_DEVICE)
    else:
        raise AssertionError("invalid parameters were accepted")
