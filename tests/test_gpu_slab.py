"""The x1-slab contexts (lp_slab_* of the C ABI) on one GPU: every slab of
the grid in this process with the loopback exchange (no kernel waits on
another), stepped by the package's SlabSchedule, against one context over the
whole grid -- FP64 to 1e-12 in the state after two full steps (1-D, and a 2-D
grid in three uneven slabs), the mixed collisions within 1e-6 of FP64, and
each slab's initial state equal to its rows of the whole grid's."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel
from lp_slab import GpuSlab, LoopbackComm, SlabSchedule, slab_bounds
from oracle.oracle import FIX_DEFAULT

pytestmark = pytest.mark.gpu

CASE_1D = dict(nx1=8, nx2=1, nv=8, n=16, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
CASE_2D = dict(nx1=7, nx2=2, nv=6, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)


def _slabs(lp, kw, nslab, precision, U0=None):
    import torch
    P = lp.Params(**kw, fixes=FIX_DEFAULT, precision=precision)
    row = P.nx2 * P.nv ** 3 * 7
    stream = torch.cuda.Stream()  # one stream for every slab of this process
    slabs = []
    for r in range(nslab):
        i0, i1 = slab_bounds(P.nx1, nslab, r)
        s = GpuSlab(P, i0, i1, stream)
        if U0 is None:
            s.set_init(1)
        else:
            s.set_own_state(U0[i0 * row:i1 * row])
        slabs.append(s)
    return slabs


@pytest.mark.parametrize("kw,nslab", [(CASE_1D, 2), (CASE_2D, 3)], ids=["1d-2slabs", "2d-3slabs"])
def test_slabs_match_whole_grid(gpu_lib, kw, nslab):
    lp = gpu_lib
    pytest.importorskip("torch")
    ref = lp.Context(lp.Params(**kw, fixes=FIX_DEFAULT, precision=lp.PREC_FP64))
    ref.set_init(1)
    U0 = ref.get_state()
    slabs = _slabs(lp, kw, nslab, lp.PREC_FP64)
    assert np.array_equal(np.concatenate([s.own_state() for s in slabs]), U0)
    ref.step(2)
    SlabSchedule(slabs, LoopbackComm()).step(2)
    U = np.concatenate([s.own_state() for s in slabs])
    assert rel(U, ref.get_state()) < 1e-12
    # the field of the last stage solve is the whole grid's
    _, px, _ = slabs[0].ctx.global_fields()
    _, px_ref, _, _ = ref.last_fields()
    assert rel(px, px_ref) < 1e-12


def test_mixed_slabs_within_fp64(gpu_lib):
    lp = gpu_lib
    ref = lp.Context(lp.Params(**CASE_1D, fixes=FIX_DEFAULT, precision=lp.PREC_FP64))
    ref.set_init(1)
    U0 = ref.get_state()
    ref.step(2)
    slabs = _slabs(lp, CASE_1D, 2, lp.PREC_MIXED, U0)
    SlabSchedule(slabs, LoopbackComm()).step(2)
    U = np.concatenate([s.own_state() for s in slabs])
    assert rel(U, ref.get_state()) < 1e-6
