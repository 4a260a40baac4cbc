"""The allocation-free projection lp_conserve_noalloc, called through the C
ABI with device buffers the caller owns, against lp_conserve (the existing
entry point) on two calls in a row.  Its scratch is a fixed device array in
the library, so this file is collected last: the test must hold both in a
fresh process and after every other test has used the library."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def test_conserve_noalloc_matches_conserve(gpu_lib):
    torch = pytest.importorskip("torch")
    lp = gpu_lib
    P = lp.Params(nx1=6, nx2=1, nv=6, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01)
    ctx = lp.Context(P)
    n3 = P.n ** 3
    c1, c2, cct = ctx.conservation_rows()
    dev = torch.device("cuda")
    c1_d = torch.from_numpy(np.ascontiguousarray(c1).ravel()).to(dev)
    c2_d = torch.from_numpy(np.ascontiguousarray(c2).ravel()).to(dev)
    cct_d = torch.from_numpy(np.ascontiguousarray(cct).ravel()).to(dev)
    L = lp.lib()
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(20261203)
    for ncell in (3, 5):  # two calls in a row, the second with more cells
        q = rng.standard_normal((ncell, n3)) + 1j * rng.standard_normal((ncell, n3))
        expected = np.stack([ctx.conserve(q[c]) for c in range(ncell)])
        qd = torch.from_numpy(np.ascontiguousarray(q).view(np.float64).ravel().copy()).to(dev)
        st = L.lp_conserve_noalloc(ctypes.c_void_p(qd.data_ptr()), ncell, n3,
                                   ctypes.c_void_p(c1_d.data_ptr()), ctypes.c_void_p(c2_d.data_ptr()),
                                   ctypes.c_void_p(cct_d.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert st == lp.OK
        torch.cuda.synchronize()
        got = qd.cpu().numpy().view(np.complex128).reshape(ncell, n3)
        assert rel(got, expected) < 1e-12
    # more cells than the fixed scratch holds are refused without touching the GPU
    st = L.lp_conserve_noalloc(ctypes.c_void_p(qd.data_ptr()), lp.NOALLOC_MAX_CELLS + 1, n3,
                               ctypes.c_void_p(c1_d.data_ptr()), ctypes.c_void_p(c2_d.data_ptr()),
                               ctypes.c_void_p(cct_d.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert st == lp.ERR_INVALID
    ctx.close()
