"""Programmatic kernel-to-kernel edges in the step graphs.  With LP_PDL=1
(from the upstream kernel's programmatic port) or LP_PDL=2 (its
launch-completion port) in the environment at capture, every captured graph
(the collision step over all cells, the time step, the host-buffer collision
chunks, the batch step) is instantiated with each edge from one kernel to
the next made a programmatic dependency; every kernel waits on the device
for its predecessors before it reads anything.  The results are the same
bits as with the ordinary edges of the default, FP64 and mixed, 1-D and
2-D; the collision graph reports its programmatic edges."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import FIX_DEFAULT

pytestmark = pytest.mark.gpu

PORTS = ["1", "2"]


def _with_pdl(monkeypatch, pdl, fn):
    if pdl:
        monkeypatch.setenv("LP_PDL", pdl)
    else:
        monkeypatch.delenv("LP_PDL", raising=False)
    try:
        return fn()
    finally:
        monkeypatch.delenv("LP_PDL", raising=False)


def _params(lp, precision, **kw):
    base = dict(nx1=64, nx2=1, nv=8, n=24, lv=5.0, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
    base.update(kw)
    return lp.Params(**base, fixes=FIX_DEFAULT, precision=precision)


@pytest.mark.parametrize("port", PORTS)
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_collision_graph(gpu_lib, monkeypatch, precision, port):
    lp = gpu_lib

    def run():
        ctx = lp.Context(_params(lp, precision))
        ctx.set_init(0)
        for _ in range(3):
            ctx.collision_step()
        ctx.synchronize()
        return ctx.get_state(), ctx.collision_graph_kernels(), ctx.collision_graph_edges()

    u1, k1, e1 = _with_pdl(monkeypatch, port, run)
    u0, k0, e0 = _with_pdl(monkeypatch, None, run)
    assert np.array_equal(u1, u0)
    assert k1 == k0 > 0
    assert e0 == 0
    assert e1 > 0


@pytest.mark.parametrize("port", PORTS)
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_time_step_graph_2d(gpu_lib, monkeypatch, precision, port):
    lp = gpu_lib

    def run():
        ctx = lp.Context(_params(lp, precision, nx1=12, nx2=8, n=16))
        ctx.set_init(0)
        ctx.step(3)
        ctx.synchronize()
        return ctx.get_state()

    assert np.array_equal(_with_pdl(monkeypatch, port, run), _with_pdl(monkeypatch, None, run))


@pytest.mark.parametrize("port", PORTS)
def test_host_chunk_graphs(gpu_lib, monkeypatch, port):
    lp = gpu_lib
    P = _params(lp, 1, nx1=80, n=16)
    src = lp.Context(P)
    src.set_init(1)
    src.advect_step()
    U0 = src.get_state()

    def run():
        ctx = lp.Context(P)
        out = np.zeros_like(U0)
        ctx.collision_step_host(U0, out, 2)
        ctx.synchronize()
        return out

    assert np.array_equal(_with_pdl(monkeypatch, port, run), _with_pdl(monkeypatch, None, run))


@pytest.mark.parametrize("port", PORTS)
def test_batch_graph(gpu_lib, monkeypatch, port):
    lp = gpu_lib
    runs = [_params(lp, 1, nx1=8, n=8), _params(lp, 1, nx1=4, nx2=3, n=16, nu=0.1),
            _params(lp, 1, nx1=6, n=16, nu=0.02)]

    def run():
        b = lp.Batch(runs)
        for r in range(len(runs)):
            b.set_init(r, 1)
        b.step(2)
        return [b.get_state(r) for r in range(len(runs))]

    for a, c in zip(_with_pdl(monkeypatch, port, run), _with_pdl(monkeypatch, None, run)):
        assert np.array_equal(a, c)
