"""The x1-slab sharded time step of lp_slab.SlabSchedule on CPU ranks: gloo
processes (2 ranks, and 3 ranks with uneven slabs on a 2-D grid) and the
in-process loopback, each slab computed by the CPU oracle, against the
oracle's unsharded steps (defects F1-F3, F11, F12 fixed).  The sharded step
performs the same operations on every record and cell, so the states agree
to the last bit."""
from __future__ import annotations

import os
import socket
import tempfile

import numpy as np
import pytest

from lp_slab import DistComm, LoopbackComm, SlabSchedule, slab_bounds
from oracle.oracle import Case, FIX_DEFAULT, Oracle
from slab_oracle import OracleSlab

CASE_1D = dict(nx1=8, nx2=1, nv=6, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)
CASE_2D = dict(nx1=7, nx2=2, nv=4, n=8, lv=5.25, lx=4 * np.pi, nu=0.05, dt=0.01, a_amp=0.5, k_wave=0.5)


def _reference(case, nsteps):
    O = Oracle(case, fixes=FIX_DEFAULT)
    U0 = O.set_init(1)
    U = U0
    for _ in range(nsteps):
        U = O.step(U)
    return U0, U


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, case_kw, nsteps, out_dir):
    os.environ["OMP_NUM_THREADS"] = "2"
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    case = Case(**case_kw)
    i0, i1 = slab_bounds(case.nx1, world, rank)
    slab = OracleSlab(case, i0, i1)
    row = case.nx2 * case.nv ** 3 * 7
    U0 = Oracle(case, fixes=FIX_DEFAULT).set_init(1)
    slab.set_own_state(U0[i0 * row:i1 * row])
    SlabSchedule([slab], DistComm(case.nx1)).step(nsteps)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), slab.own_state())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,case_kw,nsteps", [(2, CASE_1D, 2), (3, CASE_2D, 1)], ids=["2ranks-1d", "3ranks-2d"])
def test_gloo_ranks_match_unsharded(world, case_kw, nsteps):
    import torch.multiprocessing as mp
    case = Case(**case_kw)
    _, U_ref = _reference(case, nsteps)
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_rank_main, args=(world, _free_port(), case_kw, nsteps, d), nprocs=world, join=True)
        U = np.concatenate([np.load(os.path.join(d, f"rank{r}.npy")) for r in range(world)])
    assert np.array_equal(U, U_ref), np.abs(U - U_ref).max()


def test_loopback_slabs_match_unsharded():
    case = Case(**CASE_1D)
    U0, U_ref = _reference(case, 2)
    row = case.nx2 * case.nv ** 3 * 7
    slabs = []
    for r in range(4):
        i0, i1 = slab_bounds(case.nx1, 4, r)
        s = OracleSlab(case, i0, i1)
        s.set_own_state(U0[i0 * row:i1 * row])
        slabs.append(s)
    SlabSchedule(slabs, LoopbackComm()).step(2)
    U = np.concatenate([s.own_state() for s in slabs])
    assert np.array_equal(U, U_ref), np.abs(U - U_ref).max()


def test_slab_bounds():
    assert [slab_bounds(8, 3, r) for r in range(3)] == [(0, 3), (3, 6), (6, 8)]
    assert [slab_bounds(64, 4, r) for r in range(4)] == [(0, 16), (16, 32), (32, 48), (48, 64)]
    with pytest.raises(ValueError):
        slab_bounds(2, 3, 0)
