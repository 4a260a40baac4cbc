"""Python binding of the C ABI in include/lp_gb300.h (ctypes over
_build/liblp_gb300.so).  Every call goes to the GPU library; there is no
CPU fallback: a missing library or device raises.

    import lp_gb300 as lp
    ctx = lp.Context(lp.Params(nx1=64, nx2=1, nv=24, n=24, lv=6.0, lx=4*pi, nu=0.05,
                               dt=0.005, a_amp=0.5, k_wave=0.5))
    ctx.set_init(1)
    ctx.step(10)
    U = ctx.get_state()
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, replace

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "liblp_gb300.so")

OK, ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_NO_DEVICE, ERR_STATE = range(6)
FIX_F1, FIX_F2, FIX_F3, FIX_F11, FIX_F12 = 1, 2, 4, 8, 16
FIX_DEFAULT = FIX_F1 | FIX_F2 | FIX_F3 | FIX_F11 | FIX_F12
PREC_FP64, PREC_MIXED = 0, 1
HOST_ASYNC = 1

_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

EXPORTS = [
    "lp_ctx_create", "lp_ctx_destroy", "lp_set_stream", "lp_synchronize", "lp_last_error",
    "lp_device_bytes", "lp_set_state", "lp_get_state", "lp_state_device_ptr", "lp_set_init",
    "lp_fft3d", "lp_fs", "lp_compute_q", "lp_conserve", "lp_rk4_cell", "lp_nodes",
    "lp_weights_rows", "lp_conservation_rows", "lp_poisson", "lp_last_fields", "lp_advect_step",
    "lp_collision_step", "lp_collision_graph_kernels", "lp_collision_graph_edges", "lp_step", "lp_moments", "lp_time_kernel", "lp_measure_fp_peaks",
    "lp_conserve_noalloc",
    "lp_batch_create", "lp_batch_destroy", "lp_batch_set_stream", "lp_batch_synchronize",
    "lp_batch_last_error", "lp_batch_device_bytes", "lp_batch_set_state", "lp_batch_get_state",
    "lp_batch_set_init", "lp_batch_moments", "lp_batch_advect_step", "lp_batch_collision_step",
    "lp_batch_step", "lp_batch_classes", "lp_batch_class_info", "lp_batch_autotune",
    "lp_field_energy", "lp_collision_vjp", "lp_advect_vjp", "lp_step_vjp", "lp_field_energy_gradient",
    "lp_diagnostics", "lp_diagnostics_append", "lp_marginal_x1v1", "lp_state_append", "lp_state_restart",
    "lp_autotune", "lp_set_schedule", "lp_compute_q_lin", "lp_conserve_lin", "lp_rk4_cell_lin",
    "lp_slab_create", "lp_stage_device_ptr", "lp_slab_charge", "lp_slab_fields", "lp_slab_advect_stage",
    "lp_slab_fields_host", "lp_collision_step_host", "lp_set_adjoint_form", "lp_set_convolution_form",
    "lp_get_convolution_form",
]
NOALLOC_MAX_CELLS = 4096


class LPError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"lp status {status}: {msg}")
        self.status = status


class _Params(ctypes.Structure):
    _fields_ = [("nx1", ctypes.c_int), ("nx2", ctypes.c_int), ("nv", ctypes.c_int),
                ("n", ctypes.c_int), ("lv", ctypes.c_double), ("lx", ctypes.c_double),
                ("nu", ctypes.c_double), ("dt", ctypes.c_double), ("a_amp", ctypes.c_double),
                ("k_wave", ctypes.c_double), ("fixes", ctypes.c_uint), ("precision", ctypes.c_int),
                ("linear_ei", ctypes.c_int)]


@dataclass
class Params:
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
    fixes: int = FIX_DEFAULT
    precision: int = PREC_FP64
    linear_ei: int = 0

    @property
    def ncell(self):
        return self.nx1 * self.nx2

    @property
    def size(self):
        return self.ncell * self.nv ** 3

    def _c(self):
        return _Params(self.nx1, self.nx2, self.nv, self.n, self.lv, self.lx, self.nu, self.dt,
                       self.a_amp, self.k_wave, self.fixes, self.precision, self.linear_ei)


_lib = None


def lib():
    """Load liblp_gb300.so (raises FileNotFoundError when it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing; run the package build first")
        L = ctypes.CDLL(LIB_PATH)
        L.lp_ctx_create.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(_vp)]
        L.lp_last_error.restype = ctypes.c_char_p
        L.lp_last_error.argtypes = [_vp]
        L.lp_device_bytes.restype = ctypes.c_size_t
        L.lp_device_bytes.argtypes = [_vp]
        for name in ["lp_ctx_destroy", "lp_synchronize"]:
            getattr(L, name).argtypes = [_vp]
        L.lp_set_stream.argtypes = [_vp, _vp]
        L.lp_set_state.argtypes = [_vp, _dp, ctypes.c_size_t]
        L.lp_get_state.argtypes = [_vp, _dp, ctypes.c_size_t]
        L.lp_state_device_ptr.argtypes = [_vp, ctypes.POINTER(_dp)]
        L.lp_set_init.argtypes = [_vp, ctypes.c_int, ctypes.c_double]
        L.lp_fft3d.argtypes = [_vp, _dp, _dp]
        L.lp_fs.argtypes = [_vp, _dp, _dp]
        L.lp_compute_q.argtypes = [_vp, _dp, _dp]
        L.lp_conserve.argtypes = [_vp, _dp]
        L.lp_rk4_cell.argtypes = [_vp, _dp, ctypes.c_int, _dp, _dp]
        L.lp_nodes.argtypes = [_vp, _dp]
        L.lp_weights_rows.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _dp]
        L.lp_conservation_rows.argtypes = [_vp, _dp, _dp, _dp]
        L.lp_poisson.argtypes = [_vp, _dp, _dp, _dp, _dp]
        L.lp_last_fields.argtypes = [_vp, _dp, _dp, _dp, _dp]
        L.lp_advect_step.argtypes = [_vp]
        L.lp_collision_step.argtypes = [_vp, ctypes.c_int, ctypes.c_int]
        L.lp_collision_graph_kernels.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
        L.lp_collision_graph_edges.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
        L.lp_step.argtypes = [_vp, ctypes.c_int]
        L.lp_moments.argtypes = [_vp, _dp]
        L.lp_time_kernel.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _dp]
        L.lp_measure_fp_peaks.argtypes = [_dp, _dp]
        L.lp_conserve_noalloc.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp]
        L.lp_batch_create.argtypes = [ctypes.POINTER(_Params), ctypes.c_int, ctypes.POINTER(_vp)]
        for name in ["lp_batch_destroy", "lp_batch_synchronize", "lp_batch_advect_step",
                     "lp_batch_collision_step"]:
            getattr(L, name).argtypes = [_vp]
        L.lp_batch_set_stream.argtypes = [_vp, _vp]
        L.lp_batch_last_error.restype = ctypes.c_char_p
        L.lp_batch_last_error.argtypes = [_vp]
        L.lp_batch_device_bytes.restype = ctypes.c_size_t
        L.lp_batch_device_bytes.argtypes = [_vp]
        L.lp_batch_set_state.argtypes = [_vp, ctypes.c_int, _dp, ctypes.c_size_t]
        L.lp_batch_get_state.argtypes = [_vp, ctypes.c_int, _dp, ctypes.c_size_t]
        L.lp_batch_set_init.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.lp_batch_moments.argtypes = [_vp, ctypes.c_int, _dp]
        L.lp_batch_step.argtypes = [_vp, ctypes.c_int]
        L.lp_batch_classes.argtypes = [_vp]
        L.lp_batch_class_info.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _dp]
        L.lp_batch_autotune.argtypes = [_vp, ctypes.c_int, ctypes.c_char_p]
        L.lp_field_energy.argtypes = [_vp, _dp, _vp]
        L.lp_collision_vjp.argtypes = [_vp, _vp, _vp, _dp]
        L.lp_advect_vjp.argtypes = [_vp, _vp, _vp]
        L.lp_step_vjp.argtypes = [_vp, _vp, _vp, _dp]
        L.lp_field_energy_gradient.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _dp, _vp, _dp]
        L.lp_diagnostics.argtypes = [_vp, _dp]
        L.lp_compute_q_lin.argtypes = [_vp, _dp, _dp, _dp]
        L.lp_conserve_lin.argtypes = [_vp, _dp, _dp]
        L.lp_rk4_cell_lin.argtypes = [_vp, _dp, ctypes.c_int, _dp, _dp, _dp]
        L.lp_autotune.argtypes = [_vp, ctypes.c_int, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_int)]
        L.lp_set_schedule.argtypes = [_vp, ctypes.c_int, ctypes.c_int]
        L.lp_diagnostics_append.argtypes = [_vp, ctypes.c_char_p, ctypes.c_char_p]
        L.lp_marginal_x1v1.argtypes = [_vp, _dp]
        L.lp_state_append.argtypes = [_vp, ctypes.c_char_p]
        L.lp_state_restart.argtypes = [_vp, ctypes.c_char_p]
        L.lp_slab_create.argtypes = [ctypes.POINTER(_Params), ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)]
        L.lp_stage_device_ptr.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(_dp)]
        L.lp_slab_charge.argtypes = [_vp, ctypes.c_int, _vp]
        L.lp_slab_fields.argtypes = [_vp, _vp]
        L.lp_slab_advect_stage.argtypes = [_vp, ctypes.c_int]
        L.lp_slab_fields_host.argtypes = [_vp, _dp, _dp, _dp]
        L.lp_collision_step_host.argtypes = [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int]
        L.lp_set_adjoint_form.argtypes = [_vp, ctypes.c_int]
        L.lp_set_convolution_form.argtypes = [_vp, ctypes.c_int]
        L.lp_get_convolution_form.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
        for name in EXPORTS:
            f = getattr(L, name)
            if name not in ("lp_last_error", "lp_device_bytes", "lp_batch_last_error",
                            "lp_batch_device_bytes"):
                f.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def measure_fp_peaks():
    """(FP32, FP64) dense FMA throughput of the current device in TFLOP/s."""
    a, b = ctypes.c_double(), ctypes.c_double()
    st = lib().lp_measure_fp_peaks(ctypes.byref(a), ctypes.byref(b))
    if st != OK:
        raise LPError(st, "lp_measure_fp_peaks failed")
    return a.value, b.value


class Context:
    """One solver instance on the current CUDA device."""

    def __init__(self, params: Params, _slab=None):
        self.L = lib()
        h = _vp()
        if _slab is None:
            self.params = params
            st = self.L.lp_ctx_create(ctypes.byref(params._c()), ctypes.byref(h))
        else:
            i1_begin, i1_end = _slab
            self.params = replace(params, nx1=i1_end - i1_begin + 2)
            st = self.L.lp_slab_create(ctypes.byref(params._c()), int(i1_begin), int(i1_end), ctypes.byref(h))
        if st != OK:
            raise LPError(st, "lp_ctx_create failed" if _slab is None else "lp_slab_create failed")
        self.h = h
        self.n3 = params.n ** 3
        self.nv3 = params.nv ** 3

    def close(self):
        if getattr(self, "h", None):
            self.L.lp_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st):
        if st != OK:
            raise LPError(st, self.L.lp_last_error(self.h).decode())

    @property
    def device_bytes(self):
        return int(self.L.lp_device_bytes(self.h))

    def set_stream(self, stream_handle):
        self._chk(self.L.lp_set_stream(self.h, _vp(stream_handle)))

    def synchronize(self):
        self._chk(self.L.lp_synchronize(self.h))

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        self._chk(self.L.lp_set_state(self.h, _p(U), U.size))

    def get_state(self):
        U = np.zeros(self.params.size * 7)
        self._chk(self.L.lp_get_state(self.h, _p(U), U.size))
        return U

    def state_device_ptr(self):
        p = _dp()
        self._chk(self.L.lp_state_device_ptr(self.h, ctypes.byref(p)))
        return ctypes.cast(p, ctypes.c_void_p).value

    def set_init(self, kind=0, u=2.0):
        self._chk(self.L.lp_set_init(self.h, int(kind), float(u)))

    def fft3d(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        out = np.zeros_like(x)
        self._chk(self.L.lp_fft3d(self.h, _p(x.view(np.float64)), _p(out.view(np.float64))))
        return out

    def fs(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
        out = np.zeros_like(x)
        self._chk(self.L.lp_fs(self.h, _p(x.view(np.float64)), _p(out.view(np.float64))))
        return out

    def compute_q(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        q = np.zeros(self.n3, np.complex128)
        self._chk(self.L.lp_compute_q(self.h, _p(f), _p(q.view(np.float64))))
        return q

    def conserve(self, q):
        q = np.array(q, dtype=np.complex128).reshape(-1)
        self._chk(self.L.lp_conserve(self.h, _p(q.view(np.float64))))
        return q

    def compute_q_lin(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        q = np.zeros(self.n3, np.complex128)
        ql = np.zeros(self.n3, np.complex128)
        self._chk(self.L.lp_compute_q_lin(self.h, _p(f), _p(q.view(np.float64)), _p(ql.view(np.float64))))
        return q, ql

    def conserve_lin(self, q, ql):
        q = np.array(q, dtype=np.complex128).reshape(-1)
        ql = np.array(ql, dtype=np.complex128).reshape(-1)
        self._chk(self.L.lp_conserve_lin(self.h, _p(q.view(np.float64)), _p(ql.view(np.float64))))
        return q, ql

    def rk4_cell_lin(self, f, cell, qhat, qlin):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(qhat, dtype=np.complex128).reshape(-1)
        ql = np.ascontiguousarray(qlin, dtype=np.complex128).reshape(-1)
        du = np.zeros(self.nv3 * 5)
        self._chk(self.L.lp_rk4_cell_lin(self.h, _p(f), int(cell), _p(q.view(np.float64)),
                                         _p(ql.view(np.float64)), _p(du)))
        return du

    def rk4_cell(self, f, cell, qhat):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(qhat, dtype=np.complex128).reshape(-1)
        du = np.zeros(self.nv3 * 5)
        self._chk(self.L.lp_rk4_cell(self.h, _p(f), int(cell), _p(q.view(np.float64)), _p(du)))
        return du

    def nodes(self, ncollide=None):
        nc = ncollide if ncollide is not None else self.params.ncell
        f = np.zeros(nc * self.n3)
        self._chk(self.L.lp_nodes(self.h, _p(f)))
        return f.reshape(nc, self.n3)

    def weights_rows(self, r0, r1):
        out = np.zeros((r1 - r0) * self.n3)
        self._chk(self.L.lp_weights_rows(self.h, int(r0), int(r1), _p(out)))
        return out.reshape(r1 - r0, self.n3)

    def conservation_rows(self):
        c1 = np.zeros(5 * self.n3); c2 = np.zeros(5 * self.n3); cct = np.zeros(25)
        self._chk(self.L.lp_conservation_rows(self.h, _p(c1), _p(c2), _p(cct)))
        return c1.reshape(5, -1), c2.reshape(5, -1), cct.reshape(5, 5)

    def poisson(self):
        nc = self.params.ncell
        potc, px, py, fl = np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(14 * nc)
        self._chk(self.L.lp_poisson(self.h, _p(potc), _p(px), _p(py), _p(fl)))
        return potc, px, py, fl.reshape(14, nc)

    def last_fields(self):
        nc = self.params.ncell
        potc, px, py, fl = np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(3 * nc), np.zeros(14 * nc)
        self._chk(self.L.lp_last_fields(self.h, _p(potc), _p(px), _p(py), _p(fl)))
        return potc, px, py, fl.reshape(14, nc)

    def advect_step(self):
        self._chk(self.L.lp_advect_step(self.h))

    def collision_step(self, c0=-1, c1=-1):
        self._chk(self.L.lp_collision_step(self.h, int(c0), int(c1)))

    def collision_step_host(self, U_in, U_out, chunks=1, asynchronous=False):
        """Collision step of host buffers (numpy arrays or pinned torch CPU
        tensors of float64, ncell*nv^3*7 values), lp_collision_step_host:
        queued on the context's streams; U_out is complete after
        synchronize()."""
        def ptr(a):
            if isinstance(a, np.ndarray):
                assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] and a.size == self.params.size * 7
                return a.ctypes.data
            assert a.dtype.itemsize == 8 and a.is_contiguous() and a.numel() == self.params.size * 7
            return a.data_ptr()
        self._chk(self.L.lp_collision_step_host(self.h, _vp(ptr(U_in)), _vp(ptr(U_out)), int(chunks),
                                                HOST_ASYNC if asynchronous else 0))

    def collision_graph_kernels(self):
        """Kernel launches in one replay of the captured collision step over
        every collided cell (0 before the first such step)."""
        k = ctypes.c_int()
        self._chk(self.L.lp_collision_graph_kernels(self.h, ctypes.byref(k)))
        return k.value

    def collision_graph_edges(self):
        """Programmatic kernel-to-kernel edges of that graph (0 before the
        first such step, and unless LP_PDL=1 or 2 was in the environment at
        capture)."""
        k = ctypes.c_int()
        self._chk(self.L.lp_collision_graph_edges(self.h, ctypes.byref(k)))
        return k.value

    def step(self, nsteps=1):
        self._chk(self.L.lp_step(self.h, int(nsteps)))

    def time_kernel(self, which=0, reps=10):
        """Average ms per launch of a stage (0 contraction, 1 forward transform,
        2 conservation, 3 DG projection, 4..8 the five kernels of the convolution
        form), CUDA events on the context's stream."""
        ms = ctypes.c_double()
        self._chk(self.L.lp_time_kernel(self.h, int(which), int(reps), ctypes.byref(ms)))
        return ms.value

    def moments(self):
        out = np.zeros(6)
        self._chk(self.L.lp_moments(self.h, _p(out)))
        return out

    def autotune(self, reps=3, cache_path=None):
        """Pick the fastest collision schedule; returns (cells per pass, contraction form):
        the form is 0 for the convolution form, 2 or 4 for the line-tiled sum with that
        many warps per line block."""
        bp, lw = ctypes.c_int(), ctypes.c_int()
        self._chk(self.L.lp_autotune(self.h, int(reps), cache_path.encode() if cache_path else None,
                                     ctypes.byref(bp), ctypes.byref(lw)))
        return bp.value, lw.value

    def set_schedule(self, pass_cells, line_warps):
        """Set the collision schedule (see autotune for the forms)."""
        self._chk(self.L.lp_set_schedule(self.h, int(pass_cells), int(line_warps)))

    def diagnostics(self):
        """{mass, p1, p2, p3, KiE, EleE, sqrt EleE, log sqrt EleE, KiE + EleE, entropy}"""
        out = np.zeros(10)
        self._chk(self.L.lp_diagnostics(self.h, _p(out)))
        return out

    def diagnostics_append(self, moments_path=None, entropy_path=None):
        self._chk(self.L.lp_diagnostics_append(self.h, moments_path.encode() if moments_path else None,
                                               entropy_path.encode() if entropy_path else None))

    def marginal_x1v1(self):
        out = np.zeros(self.params.nx1 * 4 * self.params.nv * 4)
        self._chk(self.L.lp_marginal_x1v1(self.h, _p(out)))
        return out.reshape(self.params.nx1 * 4, self.params.nv * 4)

    def state_append(self, path):
        self._chk(self.L.lp_state_append(self.h, path.encode()))

    def state_restart(self, path):
        self._chk(self.L.lp_state_restart(self.h, path.encode()))

    def set_convolution_form(self, form):
        """Kernels of the convolution form: 1 axis-2 spectra on chip (default), 0 three passes."""
        self._chk(self.L.lp_set_convolution_form(self.h, int(form)))

    def convolution_form(self):
        """1 or 0 (set_convolution_form), -1 when the context has no convolution form."""
        f = ctypes.c_int()
        self._chk(self.L.lp_get_convolution_form(self.h, ctypes.byref(f)))
        return f.value

    def set_adjoint_form(self, form):
        """ComputeQ's VJP in the adjoint: 0 correlations (default), 1 pair-table gather."""
        self._chk(self.L.lp_set_adjoint_form(self.h, int(form)))

    # adjoint: device pointers (e.g. torch tensors' data_ptr()) of state-sized
    # FP64 vectors
    def field_energy(self, lam_ptr=None):
        J = ctypes.c_double()
        self._chk(self.L.lp_field_energy(self.h, ctypes.byref(J), _vp(lam_ptr) if lam_ptr else None))
        return J.value

    def collision_vjp(self, lam_out_ptr, lam_in_ptr):
        d = ctypes.c_double()
        self._chk(self.L.lp_collision_vjp(self.h, _vp(lam_out_ptr), _vp(lam_in_ptr), ctypes.byref(d)))
        return d.value

    def advect_vjp(self, lam_out_ptr, lam_in_ptr):
        self._chk(self.L.lp_advect_vjp(self.h, _vp(lam_out_ptr), _vp(lam_in_ptr)))

    def step_vjp(self, lam_out_ptr, lam_in_ptr):
        d = ctypes.c_double()
        self._chk(self.L.lp_step_vjp(self.h, _vp(lam_out_ptr), _vp(lam_in_ptr), ctypes.byref(d)))
        return d.value

    def field_energy_gradient(self, nsteps, checkpoint, dU0_ptr):
        J, d = ctypes.c_double(), ctypes.c_double()
        self._chk(self.L.lp_field_energy_gradient(self.h, int(nsteps), int(checkpoint), ctypes.byref(J),
                                                  _vp(dU0_ptr), ctypes.byref(d)))
        return J.value, d.value


class SlabContext(Context):
    """Global x1 rows [i1_begin, i1_end) of the grid `params` with one halo
    row on each side (lp_slab_* of the C ABI); `params` of the instance is the
    local geometry (nx1 = i1_end - i1_begin + 2), `global_params` the grid's."""

    def __init__(self, params: Params, i1_begin: int, i1_end: int):
        super().__init__(params, _slab=(i1_begin, i1_end))
        self.global_params = params
        self.i1_begin, self.i1_end = int(i1_begin), int(i1_end)
        self.nown = self.i1_end - self.i1_begin

    def stage_device_ptr(self, stage):
        p = _dp()
        self._chk(self.L.lp_stage_device_ptr(self.h, int(stage), ctypes.byref(p)))
        return ctypes.cast(p, ctypes.c_void_p).value

    def charge(self, stage, rt_dev_ptr):
        self._chk(self.L.lp_slab_charge(self.h, int(stage), _vp(rt_dev_ptr)))

    def fields(self, rt_global_dev_ptr):
        self._chk(self.L.lp_slab_fields(self.h, _vp(rt_global_dev_ptr)))

    def advect_stage(self, stage):
        self._chk(self.L.lp_slab_advect_stage(self.h, int(stage)))

    def global_fields(self):
        n = 3 * self.global_params.ncell
        potc, px, py = np.zeros(n), np.zeros(n), np.zeros(n)
        self._chk(self.L.lp_slab_fields_host(self.h, _p(potc), _p(px), _p(py)))
        return potc, px, py


class Batch:
    """Independent runs stepped together (lp_batch_* of the C ABI)."""

    def __init__(self, params_list):
        self.params = list(params_list)
        self.L = lib()
        arr = (_Params * len(self.params))(*[p._c() for p in self.params])
        h = _vp()
        st = self.L.lp_batch_create(arr, len(self.params), ctypes.byref(h))
        if st != OK:
            raise LPError(st, "lp_batch_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.lp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st):
        if st != OK:
            raise LPError(st, self.L.lp_batch_last_error(self.h).decode())

    @property
    def device_bytes(self):
        return int(self.L.lp_batch_device_bytes(self.h))

    def set_stream(self, stream_handle):
        self._chk(self.L.lp_batch_set_stream(self.h, _vp(stream_handle)))

    def synchronize(self):
        self._chk(self.L.lp_batch_synchronize(self.h))

    def set_state(self, run, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        self._chk(self.L.lp_batch_set_state(self.h, int(run), _p(U), U.size))

    def get_state(self, run):
        U = np.zeros(self.params[run].size * 7)
        self._chk(self.L.lp_batch_get_state(self.h, int(run), _p(U), U.size))
        return U

    def set_init(self, run, kind=1, u=2.0):
        self._chk(self.L.lp_batch_set_init(self.h, int(run), int(kind), float(u)))

    def moments(self, run):
        out = np.zeros(6)
        self._chk(self.L.lp_batch_moments(self.h, int(run), _p(out)))
        return out

    def advect_step(self):
        self._chk(self.L.lp_batch_advect_step(self.h))

    def collision_step(self):
        self._chk(self.L.lp_batch_collision_step(self.h))

    def step(self, nsteps=1):
        self._chk(self.L.lp_batch_step(self.h, int(nsteps)))

    def classes(self):
        """[(n, nv, runs, cells, cells_per_pass, line_warps, tuned_ms)] per class."""
        out = []
        for k in range(self.L.lp_batch_classes(self.h)):
            info = (ctypes.c_int * 6)()
            ms = ctypes.c_double()
            self._chk(self.L.lp_batch_class_info(self.h, k, info, ctypes.byref(ms)))
            out.append(tuple(info) + (ms.value,))
        return out

    def autotune(self, reps=3, cache_path=None):
        self._chk(self.L.lp_batch_autotune(self.h, int(reps),
                                           cache_path.encode() if cache_path else None))
