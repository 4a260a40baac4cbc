"""A slab of a sharded run on the CPU oracle, with the interface of
lp_slab.GpuSlab, so the package's SlabSchedule can be checked on CPU ranks
(gloo) against the oracle's unsharded steps.  Test infrastructure only."""
from __future__ import annotations

import numpy as np

from oracle.oracle import Case, FIX_DEFAULT, Oracle


class OracleSlab:
    """Global x1 rows [i1_begin, i1_end) of `case` plus one halo row on each
    side: the flux, the charge sums and the collisions run on an oracle of
    the slab's geometry (with the whole grid's cell sizes), the Poisson solve
    on an oracle of the whole grid."""

    def __init__(self, case: Case, i1_begin, i1_end, fixes=FIX_DEFAULT):
        import torch
        self.case = case
        self.nown = i1_end - i1_begin
        self.i1_off = i1_begin - 1
        local = Case(**{**case.__dict__, "nx1": self.nown + 2})
        self.O = Oracle(local, fixes=fixes)
        self.O.set_cell_size(case.lx / case.nx1, case.lx / case.nx2)
        self.G = Oracle(case, fixes=fixes)
        self.nx2, self.nv3 = case.nx2, case.nv ** 3
        self.row = self.nx2 * self.nv3 * 7
        n = (self.nown + 2) * self.row
        self.buf = [np.zeros(n) for _ in range(3)]
        self.t = [torch.from_numpy(b) for b in self.buf]
        self.fl = None

    def set_own_state(self, U_own):
        self.buf[0][self.row:(self.nown + 1) * self.row] = U_own

    def own_state(self):
        return self.buf[0][self.row:(self.nown + 1) * self.row].copy()

    def rows(self, stage):
        b, r, m = self.t[stage], self.row, self.nown
        return b[r:2 * r], b[m * r:(m + 1) * r], b[0:r], b[(m + 1) * r:(m + 2) * r]

    def charge(self, stage):
        import torch
        return torch.from_numpy(self.O.charge(self.buf[stage], self.nx2, (self.nown + 1) * self.nx2))

    def fields(self, rt_global):
        _, _, _, fl = self.G.poisson_rt(rt_global.numpy())
        gnx1 = self.case.nx1
        idx = [((i1 + self.i1_off) % gnx1) * self.nx2 + i2 for i1 in range(self.nown + 2) for i2 in range(self.nx2)]
        self.fl = np.ascontiguousarray(fl[:, idx])

    def advect_stage(self, stage):
        out = self.buf[(stage + 1) % 3]
        self.O.rk3_stage(self.buf[0], self.buf[stage], self.fl, stage, out)

    def collide(self):
        if self.case.nu <= 0:
            return
        U = self.buf[0]
        rec = U.reshape(-1, self.nv3, 7)
        for s in range(self.nx2, (self.nown + 1) * self.nx2):
            f = self.O.nodes(U, s)
            du = self.O.rk4(f, self.O.conserve(self.O.compute_q(f)), rec[s].ravel()).reshape(self.nv3, 5)
            rec[s][:, [0, 3, 4, 5, 6]] = du
