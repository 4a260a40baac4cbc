"""ctypes bindings for the CPU oracle (liblp_oracle.so) and, where it was
built, the reference's own sources (oracle/_ref/libref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU arms of bench.py, never by the shipped library.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liblp_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
REF_LIN_SO = os.path.join(HERE, "_ref", "libref_lin.so")  # the FullandLinear build

FIX_F1, FIX_F2, FIX_F3, FIX_F11, FIX_F12 = 1, 2, 4, 8, 16
FIX_DEFAULT = FIX_F1 | FIX_F2 | FIX_F3 | FIX_F11 | FIX_F12

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_ip)
    raise TypeError(a.dtype)


def build_oracle(force: bool = False) -> str:
    """Compile oracle/lp_oracle.c into oracle/_build/liblp_oracle.so."""
    src = os.path.join(HERE, "lp_oracle.c")
    deps = [src, os.path.join(HERE, "lp_oracle.h"), os.path.join(HERE, "band_lu.h"),
            os.path.join(HERE, "dft3.h")]
    if not force and os.path.exists(ORACLE_SO) and all(
            os.path.getmtime(ORACLE_SO) >= os.path.getmtime(d) for d in deps):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    import subprocess
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", "-o", ORACLE_SO,
           src, "-lm"]
    subprocess.check_call(cmd)
    return ORACLE_SO


class _Params(ctypes.Structure):
    _fields_ = [("nx1", ctypes.c_int), ("nx2", ctypes.c_int), ("nv", ctypes.c_int),
                ("n", ctypes.c_int), ("lv", ctypes.c_double), ("lx", ctypes.c_double),
                ("nu", ctypes.c_double), ("dt", ctypes.c_double), ("a_amp", ctypes.c_double),
                ("k_wave", ctypes.c_double), ("fixes", ctypes.c_uint), ("linear_ei", ctypes.c_int)]


@dataclass
class Case:
    """One run configuration in the reference's variables."""
    nx1: int
    nx2: int
    nv: int
    n: int
    lv: float = 5.25
    lx: float = 4.0 * np.pi
    nu: float = 0.01
    dt: float = 0.01
    a_amp: float = 0.01
    k_wave: float = 0.5
    linear_ei: int = 0  # 1: the two-species variant (FullandLinear)

    @property
    def ncell(self):
        return self.nx1 * self.nx2

    @property
    def size(self):
        return self.ncell * self.nv ** 3


_olib = None


def _oracle_lib():
    global _olib
    if _olib is None:
        build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        L.lpo_create.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(ctypes.c_void_p)]
        L.lpo_create.restype = ctypes.c_int
        L.lpo_destroy.argtypes = [ctypes.c_void_p]
        L.lpo_weight.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.lpo_weight.restype = ctypes.c_double
        L.lpo_omega_tables.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        for name in ["lpo_grids", "lpo_cons", "lpo_fft3d", "lpo_fs", "lpo_compute_q",
                     "lpo_conserve", "lpo_intmodes", "lpo_rk4", "lpo_nodes", "lpo_set_init",
                     "lpo_poisson", "lpo_rk3", "lpo_collide", "lpo_step", "lpo_moments",
                     "lpo_band"]:
            getattr(L, name).restype = None
        L.lpo_collide.restype = ctypes.c_int
        L.lpo_entropy.restype = ctypes.c_double
        L.lpo_entropy.argtypes = [ctypes.c_void_p, _dp]
        L.lpo_marginal_x1v1.restype = None
        L.lpo_marginal_x1v1.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.lpo_intmodes.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 6 + [_dp]
        L.lpo_rk4.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, ctypes.c_int]
        L.lpo_nodes.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, _dp]
        L.lpo_set_init.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double]
        L.lpo_collide.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int]
        L.lpo_step.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int]
        L.lpo_band.argtypes = [ctypes.c_void_p, _ip, _dp, _ip]
        L.lpo_weight_lin.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.lpo_weight_lin.restype = ctypes.c_double
        for name in ["lpo_compute_q_lin", "lpo_conserve_lin", "lpo_cct_lin", "lpo_rk4_lin"]:
            getattr(L, name).restype = None
        L.lpo_compute_q_lin.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.lpo_conserve_lin.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.lpo_cct_lin.argtypes = [ctypes.c_void_p, _dp]
        L.lpo_rk4_lin.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, ctypes.c_int, _dp, ctypes.c_int]
        for name in ["lpo_charge", "lpo_poisson_rt", "lpo_rk3_stage", "lpo_set_cell_size"]:
            getattr(L, name).restype = None
        L.lpo_charge.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int, _dp]
        L.lpo_poisson_rt.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp]
        L.lpo_rk3_stage.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int, _dp]
        L.lpo_set_cell_size.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        _olib = L
    return _olib


class Oracle:
    """The CPU restatement for one case."""

    def __init__(self, case: Case, fixes: int = FIX_DEFAULT):
        self.case = case
        self.fixes = fixes
        self.L = _oracle_lib()
        p = _Params(case.nx1, case.nx2, case.nv, case.n, case.lv, case.lx, case.nu, case.dt,
                    case.a_amp, case.k_wave, fixes, int(case.linear_ei))
        h = ctypes.c_void_p()
        if self.L.lpo_create(ctypes.byref(p), ctypes.byref(h)) != 0:
            raise ValueError(f"oracle rejected case {case}")
        self.h = h
        self.n3 = case.n ** 3
        self.nv3 = case.nv ** 3

    def __del__(self):
        try:
            self.L.lpo_destroy(self.h)
        except Exception:
            pass

    def grids(self):
        n = self.case.n
        v, eta, wt, sc = (np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(14))
        self.L.lpo_grids(self.h, _p(v), _p(eta), _p(wt), _p(sc))
        return v, eta, wt, sc

    def cons(self):
        c1 = np.zeros(5 * self.n3); c2 = np.zeros(5 * self.n3); cct = np.zeros(25)
        self.L.lpo_cons(self.h, _p(c1), _p(c2), _p(cct))
        return c1.reshape(5, -1), c2.reshape(5, -1), cct.reshape(5, 5)

    def weight(self, xi, om):
        return self.L.lpo_weight(self.h, int(xi), int(om))

    def omega_tables(self):
        """ahat (n3), Shat (n3 x 6: 00, 01, 02, 11, 12, 22) and the |omega| == 0
        flags that weight() reads: W = (0 if flag else ahat) - d^T Shat d."""
        ah = np.zeros(self.n3); sh = np.zeros(6 * self.n3); rz = np.zeros(self.n3, np.uint8)
        self.L.lpo_omega_tables(self.h, _p(ah), _p(sh), rz.ctypes.data_as(ctypes.c_void_p))
        return ah, sh.reshape(-1, 6), rz.astype(bool)

    def fft3d(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        out = np.zeros_like(x)
        self.L.lpo_fft3d(self.h, _p(x.view(np.float64)), _p(out.view(np.float64)))
        return out

    def fs(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        out = np.zeros_like(x)
        self.L.lpo_fs(self.h, _p(x.view(np.float64)), _p(out.view(np.float64)))
        return out

    def compute_q(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        q = np.zeros(self.n3, np.complex128)
        self.L.lpo_compute_q(self.h, _p(f), _p(q.view(np.float64)))
        return q

    def conserve(self, q):
        q = np.array(q, dtype=np.complex128).reshape(-1)
        self.L.lpo_conserve(self.h, _p(q.view(np.float64)))
        return q

    def intmodes(self, k1, k2, k3, j1, j2, j3):
        out = np.zeros(10)
        self.L.lpo_intmodes(self.h, k1, k2, k3, j1, j2, j3, _p(out))
        return out

    def rk4(self, f, qhat, ucell, direct=False):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(qhat, dtype=np.complex128).reshape(-1)
        u = np.ascontiguousarray(ucell, dtype=np.float64).reshape(-1)
        du = np.zeros(self.nv3 * 5)
        self.L.lpo_rk4(self.h, _p(f), _p(q.view(np.float64)), _p(u), _p(du), int(direct))
        return du

    def nodes(self, U, cell):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        f = np.zeros(self.n3)
        self.L.lpo_nodes(self.h, _p(U), int(cell), _p(f))
        return f

    def set_init(self, kind=0, u=2.0):
        U = np.zeros(self.case.size * 7)
        self.L.lpo_set_init(self.h, _p(U), int(kind), float(u))
        return U

    def poisson(self, U):
        nc = self.case.ncell
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        potc, px, py = np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(3 * nc)
        fl = np.zeros(14 * nc)
        self.L.lpo_poisson(self.h, _p(U), _p(potc), _p(px), _p(py), _p(fl))
        return potc, px, py, fl.reshape(14, nc)

    def rk3(self, U):
        U = np.array(U, dtype=np.float64).reshape(-1)
        self.L.lpo_rk3(self.h, _p(U))
        return U

    def collide(self, U, direct=False):
        U = np.array(U, dtype=np.float64).reshape(-1)
        self.L.lpo_collide(self.h, _p(U), int(direct))
        return U

    def step(self, U, direct=False):
        U = np.array(U, dtype=np.float64).reshape(-1)
        self.L.lpo_step(self.h, _p(U), int(direct))
        return U

    # pieces of RK3 for slabs of a sharded run
    def charge(self, U, s0, s1):
        rt = np.zeros(3 * (s1 - s0))
        self.L.lpo_charge(self.h, _p(np.ascontiguousarray(U, dtype=np.float64).reshape(-1)), int(s0), int(s1),
                          _p(rt))
        return rt

    def poisson_rt(self, rt):
        nc = self.case.ncell
        potc, px, py, fl = np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(14 * nc)
        self.L.lpo_poisson_rt(self.h, _p(np.ascontiguousarray(rt, dtype=np.float64)), _p(potc), _p(px), _p(py),
                              _p(fl))
        return potc, px, py, fl.reshape(14, nc)

    def rk3_stage(self, U0, Us, fields14, stage, Uout):
        """Uout (a C-contiguous float64 array, written in place) =
        SSP-RK3 stage `stage` from U0, Us with the given field integrals."""
        self.L.lpo_rk3_stage(self.h, _p(U0), _p(Us), _p(np.ascontiguousarray(fields14, dtype=np.float64)),
                             int(stage), _p(Uout))

    def set_cell_size(self, dx, dy):
        self.L.lpo_set_cell_size(self.h, float(dx), float(dy))

    def moments(self, U, phix, phiy):
        out = np.zeros(6)
        self.L.lpo_moments(self.h, _p(np.ascontiguousarray(U, dtype=np.float64)),
                           _p(np.ascontiguousarray(phix)), _p(np.ascontiguousarray(phiy)),
                           _p(out))
        return out

    # two-species variant (FullandLinear)
    def weight_lin(self, xi, om):
        return self.L.lpo_weight_lin(self.h, int(xi), int(om))

    def compute_q_lin(self, f):
        q = np.zeros(self.n3, np.complex128)
        ql = np.zeros(self.n3, np.complex128)
        self.L.lpo_compute_q_lin(self.h, _p(np.ascontiguousarray(f, dtype=np.float64)),
                                 _p(q.view(np.float64)), _p(ql.view(np.float64)))
        return q, ql

    def conserve_lin(self, q, ql):
        q = np.array(q, dtype=np.complex128).reshape(-1)
        ql = np.array(ql, dtype=np.complex128).reshape(-1)
        self.L.lpo_conserve_lin(self.h, _p(q.view(np.float64)), _p(ql.view(np.float64)))
        return q, ql

    def cct_lin(self):
        out = np.zeros(4)
        self.L.lpo_cct_lin(self.h, _p(out))
        return out.reshape(2, 2)

    def rk4_lin(self, f, qhat, qlin, U, cell, direct=False):
        du = np.zeros(self.nv3 * 5)
        self.L.lpo_rk4_lin(self.h, _p(np.ascontiguousarray(f, dtype=np.float64)),
                           _p(np.ascontiguousarray(qhat, dtype=np.complex128).view(np.float64)),
                           _p(np.ascontiguousarray(qlin, dtype=np.complex128).view(np.float64)),
                           _p(np.ascontiguousarray(U, dtype=np.float64)), int(cell), _p(du), int(direct))
        return du

    def entropy(self, U):
        return float(self.L.lpo_entropy(self.h, _p(np.ascontiguousarray(U, dtype=np.float64))))

    def marginal_x1v1(self, U):
        out = np.zeros(self.case.nx1 * 4 * self.case.nv * 4)
        self.L.lpo_marginal_x1v1(self.h, _p(np.ascontiguousarray(U, dtype=np.float64)), _p(out))
        return out.reshape(self.case.nx1 * 4, self.case.nv * 4)

    def band(self):
        dims = np.zeros(4, np.int32)
        self.L.lpo_band(self.h, _p(dims), None, None)
        ndim, kl, ku, ldab = [int(x) for x in dims]
        ab = np.zeros(ldab * ndim)
        piv = np.zeros(ndim, np.int32)
        self.L.lpo_band(self.h, _p(dims), _p(ab), _p(piv))
        return dims, ab.reshape(ndim, ldab), piv


_rlibs = {}


def reference_available(linear: bool = False) -> bool:
    return os.path.exists(REF_LIN_SO if linear else REF_SO)


def _ref_lib(linear: bool = False):
    if linear not in _rlibs:
        L = ctypes.CDLL(REF_LIN_SO if linear else REF_SO)
        L.ref_setup.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 6 + [ctypes.c_int]
        L.ref_setup.restype = ctypes.c_int
        L.ref_ghat3.argtypes = [ctypes.c_double] * 6
        L.ref_ghat3.restype = ctypes.c_double
        L.ref_get_weights.restype = ctypes.c_int
        L.ref_get_weights.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
        L.ref_intmodes.argtypes = [ctypes.c_int] * 6 + [_dp]
        if linear:
            for name in ["ref_compute_q_lin", "ref_rk4_lin", "ref_get_weights_lin"]:
                getattr(L, name).restype = ctypes.c_int
            L.ref_compute_q_lin.argtypes = [_dp, _dp, _dp]
            L.ref_conserve_lin.argtypes = [_dp, _dp]
            L.ref_conserve_lin.restype = None
            L.ref_get_cct_lin.argtypes = [_dp]
            L.ref_get_cct_lin.restype = None
            L.ref_get_weights_lin.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
            L.ref_rk4_lin.argtypes = [_dp, ctypes.c_int, _dp, _dp, _dp, _dp]
        else:
            for name in ["ref_compute_q", "ref_rk4", "ref_collision_cells"]:
                getattr(L, name).restype = ctypes.c_int
            L.ref_rk4.argtypes = [_dp, ctypes.c_int, _dp, _dp, _dp]
            L.ref_collision_cells.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp]
        L.ref_get_band.argtypes = [_ip, _dp, _ip]
        L.ref_entropy.argtypes = [_dp]
        L.ref_entropy.restype = ctypes.c_double
        L.ref_marginal_x1v1.argtypes = [_dp, _dp]
        L.ref_marginal_x1v1.restype = None
        _rlibs[linear] = L
    return _rlibs[linear]


class Reference:
    """The reference's own routines (2-D geometry: nx1 = nx2 = nx)."""

    def __init__(self, case: Case, with_weights: bool = True):
        assert case.nx1 == case.nx2, "the reference runs only the square 2-D layout"
        self.case = case
        self.L = _ref_lib(bool(case.linear_ei))
        r = self.L.ref_setup(case.nx1, case.nv, case.n, case.lv, case.lx, case.nu, case.dt,
                             case.a_amp, case.k_wave, int(with_weights))
        if r != 0:
            raise ValueError(f"reference rejected case {case}")
        self.n3 = case.n ** 3
        self.nv3 = case.nv ** 3

    def grids(self):
        n = self.case.n
        v, eta, wt, sc = (np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(14))
        self.L.ref_get_grid(_p(v), _p(eta), _p(wt), _p(sc))
        return v, eta, wt, sc

    def cons(self):
        c1 = np.zeros(5 * self.n3); c2 = np.zeros(5 * self.n3); cct = np.zeros(25)
        self.L.ref_get_cons(_p(c1), _p(c2), _p(cct))
        return c1.reshape(5, -1), c2.reshape(5, -1), cct.reshape(5, 5)

    def weights(self, r0, r1):
        out = np.zeros((r1 - r0) * self.n3)
        assert self.L.ref_get_weights(r0, r1, _p(out)) == 0
        return out.reshape(r1 - r0, self.n3)

    def fft3d(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        out = np.zeros_like(x)
        self.L.ref_fft3d(_p(x.view(np.float64)), _p(out.view(np.float64)))
        return out

    def fs(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        out = np.zeros_like(x)
        self.L.ref_fs(_p(x.view(np.float64)), _p(out.view(np.float64)))
        return out

    def compute_q(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        q = np.zeros(self.n3, np.complex128)
        assert self.L.ref_compute_q(_p(f), _p(q.view(np.float64))) == 0
        return q

    def conserve(self, q):
        q = np.array(q, dtype=np.complex128).reshape(-1)
        self.L.ref_conserve(_p(q.view(np.float64)))
        return q

    def intmodes(self, k1, k2, k3, j1, j2, j3):
        out = np.zeros(10)
        self.L.ref_intmodes(k1, k2, k3, j1, j2, j3, _p(out))
        return out

    def rk4(self, f, cell, qhat, U):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(qhat, dtype=np.complex128).reshape(-1)
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        du = np.zeros(self.nv3 * 5)
        assert self.L.ref_rk4(_p(f), int(cell), _p(q.view(np.float64)), _p(U), _p(du)) == 0
        return du

    def set_init_spectral(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        f = np.zeros(self.case.nx1 * self.n3)
        self.L.ref_set_init_spectral(_p(U), _p(f))
        return f.reshape(self.case.nx1, self.n3)

    def set_init_ld(self):
        U = np.zeros(self.case.size * 7)
        self.L.ref_set_init_ld(_p(U))
        return U

    def pois2d(self, U):
        nc = self.case.ncell
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        potc, px, py = np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(3 * nc)
        fl = np.zeros(14 * nc)
        self.L.ref_pois2d(_p(U), _p(potc), _p(px), _p(py), _p(fl))
        return potc, px, py, fl.reshape(14, nc)

    def band(self):
        dims = np.zeros(4, np.int32)
        self.L.ref_get_band(_p(dims), None, None)
        ndim, kl, ku, ldab = [int(x) for x in dims]
        ab = np.zeros(ldab * ndim)
        piv = np.zeros(ndim, np.int32)
        self.L.ref_get_band(_p(dims), _p(ab), _p(piv))
        return dims, ab.reshape(ndim, ldab), piv

    def rk3(self, U):
        nc = self.case.ncell
        U = np.array(U, dtype=np.float64).reshape(-1)
        potc, px, py = np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(3 * nc)
        self.L.ref_rk3(_p(U), _p(potc), _p(px), _p(py))
        return U, potc, px, py

    def collision_cells(self, U, l0, l1):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        du = np.zeros((l1 - l0) * self.nv3 * 5)
        assert self.L.ref_collision_cells(_p(U), int(l0), int(l1), _p(du)) == 0
        return du

    # two-species variant (the FullandLinear build)
    def compute_q_lin(self, f):
        q = np.zeros(self.n3, np.complex128)
        ql = np.zeros(self.n3, np.complex128)
        assert self.L.ref_compute_q_lin(_p(np.ascontiguousarray(f, dtype=np.float64)),
                                        _p(q.view(np.float64)), _p(ql.view(np.float64))) == 0
        return q, ql

    def conserve_lin(self, q, ql):
        q = np.array(q, dtype=np.complex128).reshape(-1)
        ql = np.array(ql, dtype=np.complex128).reshape(-1)
        self.L.ref_conserve_lin(_p(q.view(np.float64)), _p(ql.view(np.float64)))
        return q, ql

    def cct_lin(self):
        out = np.zeros(4)
        self.L.ref_get_cct_lin(_p(out))
        return out.reshape(2, 2)

    def weights_lin(self, r0, r1):
        out = np.zeros((r1 - r0) * self.n3)
        assert self.L.ref_get_weights_lin(r0, r1, _p(out)) == 0
        return out.reshape(r1 - r0, self.n3)

    def rk4_lin(self, f, l, qhat, qlin, U):
        du = np.zeros(self.nv3 * 5)
        assert self.L.ref_rk4_lin(_p(np.ascontiguousarray(f, dtype=np.float64)), int(l),
                                  _p(np.ascontiguousarray(qhat, dtype=np.complex128).view(np.float64)),
                                  _p(np.ascontiguousarray(qlin, dtype=np.complex128).view(np.float64)),
                                  _p(np.ascontiguousarray(U, dtype=np.float64)), _p(du)) == 0
        return du

    def entropy(self, U):
        return float(self.L.ref_entropy(_p(np.ascontiguousarray(U, dtype=np.float64))))

    def marginal_x1v1(self, U):
        out = np.zeros(self.case.nx1 * 4 * self.case.nv * 4)
        self.L.ref_marginal_x1v1(_p(np.ascontiguousarray(U, dtype=np.float64)), _p(out))
        return out.reshape(self.case.nx1 * 4, self.case.nv * 4)

    def moments(self, U, phix, phiy):
        out = np.zeros(6)
        self.L.ref_moments(_p(np.ascontiguousarray(U, dtype=np.float64)),
                           _p(np.ascontiguousarray(phix)), _p(np.ascontiguousarray(phiy)),
                           _p(out))
        return out
