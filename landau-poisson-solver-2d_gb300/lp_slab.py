"""Time steps of one run sharded over ranks in contiguous x1 slabs.

The reference distributes the spatial cells of one run over MPI ranks
(source/LP_ompi_1.cpp:164-178), collides each rank's cells (LP_ompi_1.cpp:504)
and then gathers the whole state on the root and broadcasts it back, every
step and in every RK3 stage (LP_ompi_1.cpp:518-567, advection_1.cpp:472-489).
Here each rank keeps only a slab of x1 rows, and a time step moves

- per SSP-RK3 stage, one halo row to each side (7 nv^3 nx2 doubles per face:
  the x1 upwind flux reads one row beyond the slab) by point-to-point
  send/recv;
- per SSP-RK3 stage, the three charge moments of every spatial cell by one
  all-gather, after which every rank solves the same small LDG Poisson
  system;
- nothing for the collisions, which are local to a spatial cell.

`SlabSchedule` is written against two small interfaces, so the same host
logic runs on GPUs and in tests:

- a slab: `rows(stage)` -> (first own row, last own row, left halo, right
  halo) as writable tensors of stage buffer `stage`; `charge(stage)` -> the
  own cells' charge moments (3 per cell); `fields(rt)` from the global
  charges; `advect_stage(stage)`; `collide()`.  `GpuSlab` is the C ABI's slab
  context (lp_slab_*), its tensors device views of the context's buffers;
- a communicator: `exchange(views)` fills the halos from the neighbours'
  edge rows (periodic in x1) and `allgather(rts)` returns the global charge
  vector in x1 order.  `DistComm` uses torch.distributed (NCCL for GPU
  tensors, gloo for CPU tensors) with one slab per rank; `LoopbackComm` holds
  every slab of the grid in one process (one GPU, or a test), where the
  exchanges are plain copies.
"""
from __future__ import annotations

import numpy as np


def slab_bounds(nx1, world, rank):
    """[i1_begin, i1_end) of rank `rank` when nx1 x1 rows are split into
    `world` contiguous slabs whose sizes differ by at most one."""
    base, extra = divmod(int(nx1), int(world))
    if base < 1:
        raise ValueError(f"{nx1} x1 rows cannot be split into {world} slabs")
    i0 = rank * base + min(rank, extra)
    return i0, i0 + base + (1 if rank < extra else 0)


class _DevView:
    """A device buffer of float64 values seen by torch without a copy."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False),
                                         "version": 3, "strides": None}


class GpuSlab:
    """One rank's slab on the current GPU (lp_slab_create): global x1 rows
    [i1_begin, i1_end) of the grid `params` (an lp_gb300.Params).  The
    context runs on `stream` (a torch.cuda.Stream; a new one if None), and
    SlabSchedule issues the exchanges' copies and collectives on the same
    stream, so they are ordered with the slab's kernels.  Slabs stepped in
    one process share one stream."""

    def __init__(self, params, i1_begin, i1_end, stream=None):
        import torch
        import lp_gb300 as lp
        self.torch = torch
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self.ctx = lp.SlabContext(params, i1_begin, i1_end)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.params = params
        self.nown = i1_end - i1_begin
        self.row = params.nx2 * params.nv ** 3 * 7  # doubles per x1 row
        n = (self.nown + 2) * self.row
        self.buf = [torch.as_tensor(_DevView(self.ctx.stage_device_ptr(s), n), device="cuda") for s in range(3)]
        self.rt = torch.zeros(3 * self.nown * params.nx2, dtype=torch.float64, device="cuda")

    def set_init(self, kind=1, u=2.0):
        self.ctx.set_init(kind, u)

    def set_own_state(self, U_own):
        """Own rows from the host (nown * nx2 * nv^3 * 7 doubles)."""
        with self.torch.cuda.stream(self.stream):
            self.buf[0][self.row:(self.nown + 1) * self.row].copy_(
                self.torch.from_numpy(np.ascontiguousarray(U_own, dtype=np.float64)))
        self.stream.synchronize()

    def own_state(self):
        self.stream.synchronize()
        with self.torch.cuda.stream(self.stream):
            out = self.buf[0][self.row:(self.nown + 1) * self.row].cpu().numpy()
        return out

    def rows(self, stage):
        b, r, m = self.buf[stage], self.row, self.nown
        return b[r:2 * r], b[m * r:(m + 1) * r], b[0:r], b[(m + 1) * r:(m + 2) * r]

    def charge(self, stage):
        self.ctx.charge(stage, self.rt.data_ptr())
        return self.rt

    def fields(self, rt_global):
        self.ctx.fields(rt_global.data_ptr())

    def advect_stage(self, stage):
        self.ctx.advect_stage(stage)

    def collide(self):
        nx2 = self.params.nx2
        if self.params.nu > 0:
            self.ctx.collision_step(nx2, (self.nown + 1) * nx2)


class LoopbackComm:
    """Every slab of the grid in this process, ordered by x1: the halo
    exchange and the all-gather are copies between them."""

    def exchange(self, views):
        n = len(views)
        for i, (_, _, lh, rh) in enumerate(views):
            lh.copy_(views[(i - 1) % n][1])
            rh.copy_(views[(i + 1) % n][0])

    def allgather(self, rts):
        import torch
        return torch.cat(list(rts))


class DistComm:
    """One slab per rank over torch.distributed (the default process group
    unless `group` is given); ranks hold the slabs in x1 order."""

    def __init__(self, nx1, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.sizes = [b - a for a, b in (slab_bounds(nx1, self.world, r) for r in range(self.world))]

    def _peer(self, r):
        return r if self.group is None else self.dist.get_global_rank(self.group, r)

    def exchange(self, views):
        (first, last, lh, rh), = views
        if self.world == 1:
            lh.copy_(last)
            rh.copy_(first)
            return
        left, right = self._peer((self.rank - 1) % self.world), self._peer((self.rank + 1) % self.world)
        d = self.dist
        # the first own row goes left (into that rank's right halo), the last
        # own row goes right; with two ranks both neighbours are the same rank
        # and the order of the operations pairs them as the tags do
        ops = [d.P2POp(d.isend, first.contiguous(), left, self.group, 0),
               d.P2POp(d.isend, last.contiguous(), right, self.group, 1),
               d.P2POp(d.irecv, rh, right, self.group, 0),
               d.P2POp(d.irecv, lh, left, self.group, 1)]
        for req in d.batch_isend_irecv(ops):
            req.wait()

    def allgather(self, rts):
        import torch
        (rt,) = rts
        ncell3 = rt.numel() // self.sizes[self.rank]  # 3 * nx2 values per x1 row
        per = max(self.sizes) * ncell3
        pad = torch.zeros(per, dtype=rt.dtype, device=rt.device)
        pad[:rt.numel()] = rt
        out = torch.empty(per * self.world, dtype=rt.dtype, device=rt.device)
        self.dist.all_gather_into_tensor(out, pad, group=self.group)
        return torch.cat([out[r * per:r * per + self.sizes[r] * ncell3] for r in range(self.world)])


class SlabSchedule:
    """Full time steps (SSP-RK3 advection with a Poisson solve per stage, then
    the collisions) of slabs that together cover the grid's x1 rows."""

    def __init__(self, slabs, comm):
        self.slabs = list(slabs)
        self.comm = comm

    def step(self, nsteps=1):
        stream = getattr(self.slabs[0], "stream", None)
        if stream is None:
            return self._step(nsteps)
        import torch
        with torch.cuda.stream(stream):
            self._step(nsteps)

    def _step(self, nsteps):
        for _ in range(nsteps):
            for stage in range(3):
                self.comm.exchange([s.rows(stage) for s in self.slabs])
                rt = self.comm.allgather([s.charge(stage) for s in self.slabs])
                for s in self.slabs:
                    s.fields(rt)
                    s.advect_stage(stage)
            for s in self.slabs:
                s.collide()
