"""The allocation-free projection lp_conserve_noalloc, called through the C
ABI with device buffers the caller owns, against lp_conserve (the existing
entry point) on two calls in a row, at the largest cell count its fixed
scratch holds, at n = 32 (several strided passes per thread), and against the
reference's own conserveAllMoments outputs in the golden fixtures.  Its
scratch is a fixed device array in the library, so this file is collected
last: the tests must hold both in a fresh process and after every other test
has used the library."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, golden_case, load_golden, rel

pytestmark = pytest.mark.gpu


def _call(lp, torch, q, c1_d, c2_d, cct_d):
    """Projects the (ncell, n3) complex array q with lp_conserve_noalloc on the
    current stream and returns the result."""
    ncell, n3 = q.shape
    dev = torch.device("cuda")
    qd = torch.from_numpy(np.ascontiguousarray(q).view(np.float64).ravel().copy()).to(dev)
    stream = torch.cuda.current_stream()
    st = lp.lib().lp_conserve_noalloc(ctypes.c_void_p(qd.data_ptr()), ncell, n3,
                                      ctypes.c_void_p(c1_d.data_ptr()), ctypes.c_void_p(c2_d.data_ptr()),
                                      ctypes.c_void_p(cct_d.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert st == lp.OK
    torch.cuda.synchronize()
    return qd.cpu().numpy().view(np.complex128).reshape(ncell, n3)


def _rows(torch, ctx):
    c1, c2, cct = ctx.conservation_rows()
    dev = torch.device("cuda")
    return [torch.from_numpy(np.ascontiguousarray(x).ravel()).to(dev) for x in (c1, c2, cct)]


def test_conserve_noalloc_matches_conserve(gpu_lib):
    torch = pytest.importorskip("torch")
    lp = gpu_lib
    P = lp.Params(nx1=6, nx2=1, nv=6, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01)
    ctx = lp.Context(P)
    n3 = P.n ** 3
    c1_d, c2_d, cct_d = _rows(torch, ctx)
    rng = np.random.default_rng(20261203)
    for ncell in (3, 5):  # two calls in a row, the second with more cells
        q = rng.standard_normal((ncell, n3)) + 1j * rng.standard_normal((ncell, n3))
        expected = np.stack([ctx.conserve(q[c]) for c in range(ncell)])
        assert rel(_call(lp, torch, q, c1_d, c2_d, cct_d), expected) < 1e-12
    # more cells than the fixed scratch holds are refused without touching the GPU
    L = lp.lib()
    qd = torch.zeros(2 * n3, dtype=torch.float64, device="cuda")
    st = L.lp_conserve_noalloc(ctypes.c_void_p(qd.data_ptr()), lp.NOALLOC_MAX_CELLS + 1, n3,
                               ctypes.c_void_p(c1_d.data_ptr()), ctypes.c_void_p(c2_d.data_ptr()),
                               ctypes.c_void_p(cct_d.data_ptr()), None)
    assert st == lp.ERR_INVALID
    ctx.close()


def test_conserve_noalloc_max_cells_and_n32(gpu_lib):
    """ncell = LP_NOALLOC_MAX_CELLS (the last cell's partials and multipliers
    sit at the end of the fixed array) at n = 8, then n = 32 with a few cells
    (n3 = 32768: 2048 modes per chunk, eight strided passes per thread)."""
    torch = pytest.importorskip("torch")
    lp = gpu_lib
    rng = np.random.default_rng(20261204)
    for n, ncell in ((8, lp.NOALLOC_MAX_CELLS), (32, 3)):
        ctx = lp.Context(lp.Params(nx1=2, nx2=1, nv=4, n=n, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01))
        n3 = n ** 3
        c1_d, c2_d, cct_d = _rows(torch, ctx)
        q = rng.standard_normal((ncell, n3)) + 1j * rng.standard_normal((ncell, n3))
        got = _call(lp, torch, q, c1_d, c2_d, cct_d)
        for c in sorted({0, 1, ncell // 2, ncell - 2, ncell - 1}):
            assert rel(got[c], ctx.conserve(q[c])) < 1e-12, (n, c)
        if ncell > 3:
            # every cell: the projected arrays satisfy the five constraints
            c1, c2, _ = ctx.conservation_rows()
            t = np.stack([got.real @ c1[0], got.imag @ c2[1], got.imag @ c2[2], got.imag @ c2[3],
                          got.real @ c1[4]], axis=1)
            scale = np.abs(q).max() * np.abs(c1).max() * n3
            assert np.abs(t).max() / scale < 1e-13
        ctx.close()


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_conserve_noalloc_golden(gpu_lib, name):
    """Against conserveAllMoments of the reference's own build (the golden
    qhat -> qhat_cons pair), with the constraint rows of that case."""
    torch = pytest.importorskip("torch")
    lp = gpu_lib
    g = load_golden(name)
    c = golden_case(g)
    ctx = lp.Context(lp.Params(nx1=c.nx1, nx2=c.nx2, nv=c.nv, n=c.n, lv=c.lv, lx=c.lx, nu=c.nu, dt=c.dt,
                               a_amp=c.a_amp, k_wave=c.k_wave, fixes=0))
    c1_d, c2_d, cct_d = _rows(torch, ctx)
    q = np.stack([g["qhat"], g["qhat"]])  # two cells with the same modes
    got = _call(lp, torch, q, c1_d, c2_d, cct_d)
    for cell in range(2):
        assert rel(got[cell], g["qhat_cons"]) < 1e-12
    ctx.close()
