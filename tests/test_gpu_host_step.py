"""lp_collision_step_host (the collision step of a state in host memory, its
copies overlapped with the collisions) against lp_collision_step on the
resident state: the same kernels on the same cells -- bit for bit in one
chunk, within 1e-13 in 2 and 3 chunks (passes of fewer cells group the
per-block partial sums differently) -- FP64 and mixed, pageable and pinned
buffers, in place, several calls in flight (LP_HOST_ASYNC, the two staging
states alternating), and with cells that are not collided (the reference's
2-D mode, defect F3 left in) passing through."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel
from oracle.oracle import FIX_DEFAULT, FIX_F1

pytestmark = pytest.mark.gpu

KW = dict(nx1=80, nx2=1, nv=8, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)


def _pair(lp, precision, steps):
    """A state after `steps` advection steps and its collision step."""
    ref = lp.Context(lp.Params(**KW, fixes=FIX_DEFAULT, precision=precision))
    ref.set_init(1)
    for _ in range(steps):
        ref.advect_step()
    U0 = ref.get_state()
    ref.collision_step()
    return U0, ref.get_state()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_host_step_matches_resident_step(gpu_lib, precision):
    lp = gpu_lib
    U0, expected = _pair(lp, precision, 1)
    ctx = lp.Context(lp.Params(**KW, fixes=FIX_DEFAULT, precision=precision))
    for chunks in (1, 2, 3):
        out = np.zeros_like(U0)
        ctx.collision_step_host(U0, out, chunks)
        ctx.synchronize()
        if chunks == 1:
            assert np.array_equal(out, expected)
        else:
            assert rel(out, expected) < 1e-13, chunks
    torch = pytest.importorskip("torch")
    t_in = torch.from_numpy(U0.copy()).pin_memory()
    ctx.collision_step_host(t_in, t_in, 2)  # in place, pinned
    ctx.synchronize()
    assert rel(t_in.numpy(), expected) < 1e-13


def test_host_steps_in_flight(gpu_lib):
    """Five calls queued back to back with LP_HOST_ASYNC on two different
    inputs, each into its own pinned output: every output is the collision
    step of its own input."""
    torch = pytest.importorskip("torch")
    lp = gpu_lib
    Ua, Ea = _pair(lp, lp.PREC_MIXED, 1)
    Ub, Eb = _pair(lp, lp.PREC_MIXED, 2)
    ctx = lp.Context(lp.Params(**KW, fixes=FIX_DEFAULT, precision=lp.PREC_MIXED))
    ins = [torch.from_numpy(U.copy()).pin_memory() for U in (Ua, Ub)]
    outs = [torch.zeros(Ua.size, dtype=torch.float64).pin_memory() for _ in range(5)]
    for k in range(5):
        ctx.collision_step_host(ins[k % 2], outs[k], 1, asynchronous=(k < 4))
    ctx.synchronize()
    for k in range(5):
        assert np.array_equal(outs[k].numpy(), (Ea, Eb)[k % 2]), k


def test_host_step_passes_uncollided_cells(gpu_lib):
    lp = gpu_lib
    kw = dict(KW, nx1=3, nx2=3, nv=6, n=8)
    P = lp.Params(**kw, fixes=FIX_F1, precision=lp.PREC_FP64)  # F3 unfixed: only cells s < nx1 collide
    ref = lp.Context(P)
    ref.set_init(0)
    U0 = ref.get_state()
    ref.collision_step()
    ctx = lp.Context(P)
    out = np.zeros_like(U0)
    ctx.collision_step_host(U0, out, 1)
    ctx.synchronize()
    assert np.array_equal(out, ref.get_state())
    nrec = kw["nv"] ** 3 * 7
    assert np.array_equal(out[3 * nrec:], U0[3 * nrec:])
