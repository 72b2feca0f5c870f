"""Host-side Python mirror of the mhd_gb300 C ABI.

The solver itself is the C-ABI library ``lib/libmhd_gb300.so`` (sm_103a
kernels).  This module binds it with ctypes and mirrors the reference's
operator interface (C/spu_function.h:1-15): ``fluidx``, ``advectbyzx``,
``transpose12``, ``transpose13``, ``calcfl`` and ``copy_matrix`` take the
arrays and the (permuted) dimensions exactly as the reference's C driver
passes them (C/mhd.c:62-118).  Arrays may be numpy arrays (host memory,
staged through the device) or CUDA tensors exposing ``data_ptr()``.

There is no CPU fallback: importing the bindings raises if the library has
not been built (``python -c "import __graft_entry__ as g; g.build()"``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from ._build import build as _build_lib
from ._build import lib_path

__all__ = [
    "MHD_OK", "MHD_F32", "MHD_F64", "MHD_MODE_FAST", "MHD_MODE_EXACT", "MHD_PLAIN", "MHD_FUSED",
    "MhdError", "lib", "fluidx", "advectbyzx", "transpose12", "transpose13", "calcfl", "copy_matrix",
    "Context", "init_vortex", "init_turbulence", "host_divb_max", "KERNELS",
]

MHD_OK = 0
MHD_ERR_ARG, MHD_ERR_CUDA, MHD_ERR_TIMEOUT, MHD_ERR_NONFINITE, MHD_ERR_UNSUPPORTED, MHD_ERR_NOMEM = 1, 2, 3, 4, 5, 6
MHD_F32, MHD_F64 = 0, 1
MHD_MODE_FAST, MHD_MODE_EXACT = 0, 2
MHD_HOST, MHD_DEVICE = 0, 1
MHD_PLAIN, MHD_FUSED = 0, 1
KERNELS = {"calcfl": 0, "fluidx": 1, "advectbyzx": 2, "transpose12": 3, "transpose13": 4,
           "copy": 5, "cfl_finalize": 6, "sweep": 7}

DIAG_KEYS = ("min_rho", "min_p", "max_divb", "mass", "kinetic", "magnetic", "energy", "max_speed")

_ERRORS = {1: "bad argument", 2: "CUDA runtime error", 3: "device-side wait timed out",
           4: "non-finite value in the CFL reduction", 5: "unsupported shape or mode",
           6: "device allocation failed"}


class MhdError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {_ERRORS.get(status, 'status %d' % status)} ({status})")


_LIB = None
_vp, _ip, _fp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float)


def lib(build_if_missing: bool = False) -> C.CDLL:
    """The loaded libmhd_gb300.so (raises if it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not path.exists():
        if not build_if_missing:
            raise ImportError(f"{path} is missing: build it with __graft_entry__.build()")
        _build_lib()
    L = C.CDLL(str(path))
    sig = {
        "fluidx": (None, [_vp, _vp, _ip, _ip, _ip, _fp, _vp, _vp, C.c_int]),
        "advectbyzx": (None, [_vp, _vp, _ip, _ip, _ip, _fp, _vp, _vp]),
        "transpose12": (None, [_vp, _vp, _vp, _vp, _ip, _ip, _ip, C.c_int]),
        "transpose13": (None, [_vp, _vp, _vp, _vp, _ip, _ip, _ip]),
        "copy_matrix": (None, [_vp, _vp, _ip, _ip, _ip, _vp, _vp]),
        "calcfl": (C.c_float, [_vp, _vp, _ip, _ip, _ip]),
        "mhd_last_error": (C.c_int, []),
        "mhd_error_string": (C.c_char_p, [C.c_int]),
        "mhd_set_dropin_mode": (C.c_int, [C.c_int]),
        "mhd_create": (C.c_int, [C.POINTER(_vp), C.c_int, C.c_int, C.c_int, C.c_int]),
        "mhd_destroy": (C.c_int, [_vp]),
        "mhd_stream": (_vp, [_vp]),
        "mhd_sync": (C.c_int, [_vp]),
        "mhd_op_fluidx": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_double]),
        "mhd_op_advectbyzx": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_double]),
        "mhd_op_transpose12": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int]),
        "mhd_op_transpose13": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int]),
        "mhd_op_copy": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int]),
        "mhd_op_calcfl": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]),
        "mhd_set_state": (C.c_int, [_vp, _vp, _vp, C.c_int]),
        "mhd_get_state": (C.c_int, [_vp, _vp, _vp, C.c_int]),
        "mhd_state_ptrs": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
        "mhd_clock_ptr": (C.c_int, [_vp, C.POINTER(_vp)]),
        "mhd_step": (C.c_int, [_vp, C.c_int, C.c_double, C.c_int]),
        "mhd_step_host": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_double, C.c_int]),
        "mhd_set_time": (C.c_int, [_vp, C.c_double, C.c_double]),
        "mhd_get_time": (C.c_int, [_vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_longlong)]),
        "mhd_use_graphs": (C.c_int, [_vp, C.c_int]),
        "mhd_check": (C.c_int, [_vp]),
        "mhd_diagnostics": (C.c_int, [_vp, C.POINTER(C.c_double)]),
        "mhd_clear_errors": (C.c_int, [_vp]),
        "mhd_selftest_wait": (C.c_int, [_vp, C.c_double]),
        "mhd_profile": (C.c_int, [_vp, C.c_int]),
        "mhd_profile_read": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
        "mhd_profile_reset": (C.c_int, [_vp]),
        "mhd_launch_count": (C.c_longlong, [_vp]),
        "mhd_divb_max": (C.c_int, [_vp, C.POINTER(C.c_double)]),
        "mhd_init_vortex": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong,
                                      C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]),
        "mhd_init_turbulence": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_ulonglong, C.c_double,
                                          C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                          C.c_int]),
        "mhd_host_divb_max": (C.c_double, [_vp, C.c_int, C.c_int, C.c_int, C.c_int]),
        "mhd_calcfl_noalloc": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp, _vp]),
        "mhd_write_check_value": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p]),
        "mhd_read_init": (C.c_int, [C.c_char_p, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int]),
        "mhd_checkpoint_save": (C.c_int, [C.c_char_p, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                          C.c_longlong]),
        "mhd_checkpoint_info": (C.c_int, [C.c_char_p, _ip, _ip, _ip, _ip, C.POINTER(C.c_double),
                                          C.POINTER(C.c_longlong)]),
        "mhd_checkpoint_load": (C.c_int, [C.c_char_p, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
        "cuda_cfl": (None, [_vp, _vp, _ip, _ip, _ip, _vp, _vp, _ip, _ip, _ip, _fp]),
        "cuda_fluidx": (None, [_vp, _vp, _ip, _ip, _ip, _vp, _ip, _ip, _ip]),
        "cuda_advectbyzx": (None, [_vp, _vp, _ip, _ip, _ip, _vp, _vp, _ip, _ip, _ip]),
        "cuda_transpose12": (None, [_vp, _vp, _vp, _vp, _ip, _ip, _ip, _ip, _ip, _ip]),
        "cuda_transpose13": (None, [_vp, _vp, _vp, _vp, _ip, _ip, _ip, _ip, _ip, _ip]),
        "mhd_batch_create": (C.c_int, [C.POINTER(_vp), C.c_int, _ip, C.c_int]),
        "mhd_batch_destroy": (C.c_int, [_vp]),
        "mhd_batch_set_box": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int]),
        "mhd_batch_get_box": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int]),
        "mhd_batch_step": (C.c_int, [_vp, C.c_int, C.c_double]),
        "mhd_batch_sync": (C.c_int, [_vp]),
        "mhd_batch_time": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "mhd_batch_stream": (_vp, [_vp]),
        "mhd_batch_launch_count": (C.c_longlong, [_vp]),
        "mhd_batch_classes": (C.c_int, [_vp]),
        "mhd_batch_tune_edge": (C.c_int, [_vp, C.c_int, C.c_char_p, C.c_int]),
        "mhd_batch_set_worklist": (C.c_int, [_vp, C.c_int]),
        "mhd_batch_worklist_classes": (C.c_int, [_vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def _ptr(a) -> int:
    """Address of a numpy array or of a tensor exposing data_ptr()."""
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if hasattr(a, "is_contiguous") and not a.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(f"unsupported array type {type(a)!r}")


def _check(status: int, what: str) -> None:
    if status != MHD_OK:
        raise MhdError(status, what)


def _dims(nx, ny, nz):
    return C.byref(C.c_int(nx)), C.byref(C.c_int(ny)), C.byref(C.c_int(nz))


def _last(what: str) -> None:
    _check(lib().mhd_last_error(), what)


# ------------------------------------------------------------- drop-in layer
# Same argument order and meaning as C/spu_function.h:1-15 (dimensions by
# value here; the C symbols take them by pointer).

def fluidx(u, b, nx, ny, nz, dt, update_u, update_b, iter=0):
    """u <- x-sweep of update_u with the cell-centred field of update_b (C/fluidx.c:19)."""
    lib().fluidx(_ptr(u), _ptr(b), *_dims(nx, ny, nz), C.byref(C.c_float(dt)), _ptr(update_u),
                 _ptr(update_b), int(iter))
    _last("fluidx")


def advectbyzx(u, b, nx, ny, nz, dt, update_u, update_b):
    """CT advection of b(2), b(3) along x; b(1) updated in place (C/advectbyzx.c:14)."""
    lib().advectbyzx(_ptr(u), _ptr(b), *_dims(nx, ny, nz), C.byref(C.c_float(dt)), _ptr(update_u),
                     _ptr(update_b))
    _last("advectbyzx")


def transpose12(u, b, update_u, update_b, nx, ny, nz, iter=0):
    """(u,b)(ny,nx,nz) <- update_*(nx,ny,nz) with x<->y swapped (C/transpose12.c:7)."""
    lib().transpose12(_ptr(u), _ptr(b), _ptr(update_u), _ptr(update_b), *_dims(nx, ny, nz), int(iter))
    _last("transpose12")


def transpose13(u, b, update_u, update_b, nx, ny, nz):
    """(u,b)(nz,ny,nx) <- update_* with x<->z swapped; nx == nz only (C/transpose13.c:9)."""
    lib().transpose13(_ptr(u), _ptr(b), _ptr(update_u), _ptr(update_b), *_dims(nx, ny, nz))
    _last("transpose13")


def copy_matrix(u, b, nx, ny, nz, update_u, update_b):
    """update_u <- u, update_b <- b (C/copy_matrix.c:9)."""
    lib().copy_matrix(_ptr(u), _ptr(b), *_dims(nx, ny, nz), _ptr(update_u), _ptr(update_b))
    _last("copy_matrix")


def calcfl(u, b, nx, ny, nz) -> float:
    """1/max_c over all cells (C/calcfl.c:13)."""
    r = lib().calcfl(_ptr(u), _ptr(b), *_dims(nx, ny, nz))
    st = lib().mhd_last_error()
    if st not in (MHD_OK, 4):
        raise MhdError(st, "calcfl")
    return float(r)


def set_dropin_mode(exact: bool) -> None:
    _check(lib().mhd_set_dropin_mode(MHD_MODE_EXACT if exact else MHD_MODE_FAST), "set_dropin_mode")


# ------------------------------------------------------------ context layer

class Context:
    """One solver context: owned device state, one CUDA stream, graphs."""

    def __init__(self, nx: int, ny: int, nz: int, fp64: bool = False, exact: bool = False):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.fp64 = fp64
        self.dtype = np.float64 if fp64 else np.float32
        flags = (MHD_F64 if fp64 else MHD_F32) | (MHD_MODE_EXACT if exact else MHD_MODE_FAST)
        h = C.c_void_p()
        _check(lib().mhd_create(C.byref(h), nx, ny, nz, flags), "mhd_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self) -> None:
        if self._h:
            lib().mhd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # state
    @staticmethod
    def _where(a) -> int:
        if isinstance(a, np.ndarray) or (hasattr(a, "is_cuda") and not a.is_cuda):
            return MHD_HOST
        return MHD_DEVICE

    def set_state(self, u, b) -> None:
        where = self._where(u)
        if isinstance(u, np.ndarray):
            u = np.ascontiguousarray(u, dtype=self.dtype)
            b = np.ascontiguousarray(b, dtype=self.dtype)
        _check(lib().mhd_set_state(self._h, _ptr(u), _ptr(b), where), "mhd_set_state")

    def get_state(self):
        n = self.nx * self.ny * self.nz
        u = np.empty(5 * n, dtype=self.dtype)
        b = np.empty(3 * n, dtype=self.dtype)
        _check(lib().mhd_get_state(self._h, _ptr(u), _ptr(b), MHD_HOST), "mhd_get_state")
        return u, b

    def get_state_into(self, u, b) -> None:
        where = self._where(u)
        _check(lib().mhd_get_state(self._h, _ptr(u), _ptr(b), where), "mhd_get_state")

    def clock_ptr(self) -> int:
        """Device address of the step clock (t, tf, dt, 1/c)."""
        p = C.c_void_p()
        _check(lib().mhd_clock_ptr(self._h, C.byref(p)), "mhd_clock_ptr")
        return p.value

    def state_ptrs(self):
        pu, pb = C.c_void_p(), C.c_void_p()
        _check(lib().mhd_state_ptrs(self._h, C.byref(pu), C.byref(pb)), "mhd_state_ptrs")
        return pu.value, pb.value

    def step(self, nsteps: int = 1, cfl: float = 0.7, fused: bool = False) -> None:
        _check(lib().mhd_step(self._h, nsteps, cfl, MHD_FUSED if fused else MHD_PLAIN), "mhd_step")

    def step_host(self, u, b, nsteps: int = 1, cfl: float = 0.7, fused: bool = False) -> None:
        """nsteps steps on a host state: u and b (contiguous host arrays of the
        context's dtype, e.g. pinned tensors) are copied in, stepped and
        overwritten with the result (mhd_step_host)."""
        n = self.nx * self.ny * self.nz
        for a, k in ((u, 5), (b, 3)):
            if self._where(a) != MHD_HOST:
                raise ValueError("step_host takes host arrays")
            if isinstance(a, np.ndarray) and (not a.flags.c_contiguous or a.dtype != self.dtype or a.size != k * n):
                raise ValueError(f"step_host wants contiguous {self.dtype.__name__} arrays of {k} * nx*ny*nz")
        _check(lib().mhd_step_host(self._h, _ptr(u), _ptr(b), nsteps, cfl, MHD_FUSED if fused else MHD_PLAIN),
               "mhd_step_host")

    def set_time(self, t: float = 0.0, tf: float = float("inf")) -> None:
        _check(lib().mhd_set_time(self._h, t, tf), "mhd_set_time")

    def time(self):
        t, dt, s = C.c_double(), C.c_double(), C.c_longlong()
        _check(lib().mhd_get_time(self._h, C.byref(t), C.byref(dt), C.byref(s)), "mhd_get_time")
        return t.value, dt.value, s.value

    def sync(self) -> None:
        _check(lib().mhd_sync(self._h), "mhd_sync")

    def check(self) -> int:
        return lib().mhd_check(self._h)

    def diagnostics(self) -> dict:
        """Run diagnostics of the current state, reduced on the device in FP64:
        min_rho, min_p, max_divb, mass, kinetic, magnetic, energy, max_speed."""
        out = (C.c_double * len(DIAG_KEYS))()
        _check(lib().mhd_diagnostics(self._h, out), "mhd_diagnostics")
        return dict(zip(DIAG_KEYS, list(out)))

    def clear_errors(self) -> None:
        _check(lib().mhd_clear_errors(self._h), "mhd_clear_errors")

    def selftest_wait(self, seconds: float = 0.01) -> None:
        """Queue a kernel whose bounded wait runs out after `seconds`: the next
        check() returns MHD_ERR_TIMEOUT and the context stays usable."""
        _check(lib().mhd_selftest_wait(self._h, float(seconds)), "mhd_selftest_wait")

    def use_graphs(self, on: bool) -> None:
        _check(lib().mhd_use_graphs(self._h, 1 if on else 0), "mhd_use_graphs")

    def stream(self) -> int:
        return lib().mhd_stream(self._h) or 0

    def divb_max(self) -> float:
        out = C.c_double()
        _check(lib().mhd_divb_max(self._h, C.byref(out)), "mhd_divb_max")
        return out.value

    # per-operator calls on device pointers (queued on the context stream)
    def op_fluidx(self, u, update_u, update_b, nx, ny, nz, dt):
        _check(lib().mhd_op_fluidx(self._h, _ptr(u), _ptr(update_u), _ptr(update_b), nx, ny, nz, dt),
               "mhd_op_fluidx")

    def op_advectbyzx(self, b, update_u, update_b, nx, ny, nz, dt):
        _check(lib().mhd_op_advectbyzx(self._h, _ptr(b), _ptr(update_u), _ptr(update_b), nx, ny, nz, dt),
               "mhd_op_advectbyzx")

    def op_transpose12(self, u, b, update_u, update_b, nx, ny, nz):
        _check(lib().mhd_op_transpose12(self._h, _ptr(u), _ptr(b), _ptr(update_u), _ptr(update_b),
                                        nx, ny, nz), "mhd_op_transpose12")

    def op_transpose13(self, u, b, update_u, update_b, nx, ny, nz):
        _check(lib().mhd_op_transpose13(self._h, _ptr(u), _ptr(b), _ptr(update_u), _ptr(update_b),
                                        nx, ny, nz), "mhd_op_transpose13")

    def op_copy(self, u, b, update_u, update_b, nx, ny, nz):
        _check(lib().mhd_op_copy(self._h, _ptr(u), _ptr(b), _ptr(update_u), _ptr(update_b), nx, ny, nz),
               "mhd_op_copy")

    def op_calcfl(self, u, b, nx, ny, nz) -> float:
        out = C.c_double()
        st = lib().mhd_op_calcfl(self._h, _ptr(u), _ptr(b), nx, ny, nz, C.byref(out))
        if st not in (MHD_OK, 4):
            raise MhdError(st, "mhd_op_calcfl")
        return out.value

    # profiling
    def profile(self, on: bool) -> None:
        _check(lib().mhd_profile(self._h, 1 if on else 0), "mhd_profile")

    def profile_reset(self) -> None:
        _check(lib().mhd_profile_reset(self._h), "mhd_profile_reset")

    def profile_read(self, kernel: str):
        ms, n = C.c_double(), C.c_longlong()
        _check(lib().mhd_profile_read(self._h, KERNELS[kernel], C.byref(ms), C.byref(n)), "mhd_profile_read")
        return ms.value, n.value

    def launch_count(self) -> int:
        return int(lib().mhd_launch_count(self._h))


# ------------------------------------------------------- initial conditions

def init_vortex(nx, ny, nz, seed=0, rho0=1.0, p0=0.6, vscale=1.0, noise=1e-3, bscale=1.0, fp64=False):
    """Seeded Orszag-Tang-like box (the 64^3 parity configuration); returns (u, b)."""
    dt = np.float64 if fp64 else np.float32
    n = nx * ny * nz
    u = np.empty(5 * n, dtype=dt)
    b = np.empty(3 * n, dtype=dt)
    _check(lib().mhd_init_vortex(_ptr(u), _ptr(b), nx, ny, nz, int(fp64), seed, rho0, p0, vscale, noise,
                                 bscale), "mhd_init_vortex")
    return u, b


def init_turbulence(n, seed=0, rho0=1.0, p0=1.0, mach=0.5, bx0=0.3, dbrms=0.1, kmin=2, kmax=8, fp64=False):
    """Seeded decaying-turbulence cube (the 256^3 / 512^3 throughput configuration)."""
    dt = np.float64 if fp64 else np.float32
    u = np.empty(5 * n ** 3, dtype=dt)
    b = np.empty(3 * n ** 3, dtype=dt)
    _check(lib().mhd_init_turbulence(_ptr(u), _ptr(b), n, int(fp64), seed, rho0, p0, mach, bx0, dbrms,
                                     kmin, kmax), "mhd_init_turbulence")
    return u, b


def host_divb_max(b, nx, ny, nz) -> float:
    return float(lib().mhd_host_divb_max(_ptr(b), nx, ny, nz, int(b.dtype == np.float64)))


# ------------------------------------------------------------ file formats

def write_check_value(u, b, nx, ny, nz, directory: str = "") -> None:
    """The reference's check_value dump (C/check_value.c): 8 text files, "%8.6e", i fastest."""
    u = np.ascontiguousarray(u)
    b = np.ascontiguousarray(b)
    _check(lib().mhd_write_check_value(_ptr(u), _ptr(b), nx, ny, nz, int(u.dtype == np.float64),
                                       str(directory).encode()), "mhd_write_check_value")


def read_init(path, nx, ny, nz, fp64: bool = False):
    """A state from a reference init file (C/init.c: 8 values per cell, i outer, k inner)."""
    dt = np.float64 if fp64 else np.float32
    n = nx * ny * nz
    u = np.empty(5 * n, dtype=dt)
    b = np.empty(3 * n, dtype=dt)
    _check(lib().mhd_read_init(str(path).encode(), _ptr(u), _ptr(b), nx, ny, nz, int(fp64)), "mhd_read_init")
    return u, b


def checkpoint_save(path, u, b, nx, ny, nz, t: float = 0.0, step: int = 0) -> None:
    u = np.ascontiguousarray(u)
    b = np.ascontiguousarray(b)
    _check(lib().mhd_checkpoint_save(str(path).encode(), _ptr(u), _ptr(b), nx, ny, nz, int(u.dtype == np.float64),
                                     t, step), "mhd_checkpoint_save")


def checkpoint_load(path):
    """(u, b, (nx, ny, nz), t, step) of a checkpoint written by checkpoint_save."""
    nx, ny, nz, f64 = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    t, step = C.c_double(), C.c_longlong()
    p = str(path).encode()
    _check(lib().mhd_checkpoint_info(p, C.byref(nx), C.byref(ny), C.byref(nz), C.byref(f64), C.byref(t),
                                     C.byref(step)), "mhd_checkpoint_info")
    dt = np.float64 if f64.value else np.float32
    n = nx.value * ny.value * nz.value
    u = np.empty(5 * n, dtype=dt)
    b = np.empty(3 * n, dtype=dt)
    _check(lib().mhd_checkpoint_load(p, _ptr(u), _ptr(b), nx.value, ny.value, nz.value, f64.value, C.byref(t),
                                     C.byref(step)), "mhd_checkpoint_load")
    return u, b, (nx.value, ny.value, nz.value), t.value, step.value


# ------------------------------------------------------------ batched boxes

BATCH_EDGES = (32, 48, 64, 96, 128)


def batch_config(nboxes: int = 256, seed: int = 0, edges=BATCH_EDGES):
    """The batched workload: per box its edge, IC seed, plasma beta and rms Mach.

    Edges are uniform over `edges`, beta log-uniform in [0.1, 10], rms Mach
    uniform in [0.2, 1.0]; each box is a vortex box (init_vortex) with its own
    seed (seed * 100003 + box), drawn from numpy's PCG64 so the table is the
    same on every machine.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    n = rng.choice(np.asarray(edges), size=nboxes)
    beta = 10.0 ** rng.uniform(-1.0, 1.0, size=nboxes)
    mach = rng.uniform(0.2, 1.0, size=nboxes)
    return [dict(n=int(n[i]), seed=int(seed) * 100003 + i, beta=float(beta[i]), mach=float(mach[i]))
            for i in range(nboxes)]


def init_batch_box(box: dict, fp64: bool = False, gamma: float = 5.0 / 3.0):
    """Initial state of one batched box: the vortex field with p set by beta and v by Mach.

    B = (-sin 2pi y, sin 4pi x, 0)/sqrt(4pi) has <B^2> = 1/(4pi), so
    beta = 2p/<B^2> gives p = beta/(8pi); with rho = 1 the sound speed is
    sqrt(gamma p) and <v^2> = 1.005 vscale^2 of the vortex velocity.
    """
    p0 = box["beta"] / (8.0 * np.pi)
    vscale = box["mach"] * np.sqrt(gamma * p0) / np.sqrt(1.005)
    n = box["n"]
    return init_vortex(n, n, n, seed=box["seed"], rho0=1.0, p0=p0, vscale=vscale, noise=1e-3 * vscale,
                       bscale=1.0, fp64=fp64)


class Batch:
    """Many independent periodic cubes stepped together (mhd_batch_* of the C ABI)."""

    def __init__(self, sizes, fp64: bool = False, exact: bool = False):
        self.sizes = [int(s) for s in sizes]
        self.fp64 = fp64
        self.dtype = np.float64 if fp64 else np.float32
        flags = (MHD_F64 if fp64 else MHD_F32) | (MHD_MODE_EXACT if exact else MHD_MODE_FAST)
        arr = (C.c_int * len(self.sizes))(*self.sizes)
        h = C.c_void_p()
        _check(lib().mhd_batch_create(C.byref(h), len(self.sizes), arr, flags), "mhd_batch_create")
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().mhd_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_box(self, box: int, u, b) -> None:
        if isinstance(u, np.ndarray):
            u = np.ascontiguousarray(u, dtype=self.dtype)
            b = np.ascontiguousarray(b, dtype=self.dtype)
        _check(lib().mhd_batch_set_box(self._h, box, _ptr(u), _ptr(b), Context._where(u)), "mhd_batch_set_box")

    def get_box(self, box: int):
        n = self.sizes[box] ** 3
        u = np.empty(5 * n, dtype=self.dtype)
        b = np.empty(3 * n, dtype=self.dtype)
        _check(lib().mhd_batch_get_box(self._h, box, _ptr(u), _ptr(b), MHD_HOST), "mhd_batch_get_box")
        return u, b

    def get_box_into(self, box: int, u, b) -> None:
        _check(lib().mhd_batch_get_box(self._h, box, _ptr(u), _ptr(b), Context._where(u)), "mhd_batch_get_box")

    def step(self, nsteps: int = 1, cfl: float = 0.7) -> None:
        _check(lib().mhd_batch_step(self._h, nsteps, cfl), "mhd_batch_step")

    def sync(self) -> None:
        _check(lib().mhd_batch_sync(self._h), "mhd_batch_sync")

    def time(self, box: int):
        t, dt = C.c_double(), C.c_double()
        _check(lib().mhd_batch_time(self._h, box, C.byref(t), C.byref(dt)), "mhd_batch_time")
        return t.value, dt.value

    def stream(self) -> int:
        return lib().mhd_batch_stream(self._h) or 0

    def launch_count(self) -> int:
        return int(lib().mhd_batch_launch_count(self._h))

    def classes(self) -> int:
        return int(lib().mhd_batch_classes(self._h))

    def tune_edge(self, edge: int, key: str, value: int) -> None:
        """A launch-shape knob for the boxes of one edge only (-1: the global setting)."""
        _check(lib().mhd_batch_tune_edge(self._h, int(edge), key.encode(), int(value)), "mhd_batch_tune_edge")

    def set_worklist(self, on: bool) -> None:
        """Work-list launches (default on): the classes of edge 32, 48, 64, 96
        and 128 step with one launch per operator over all of them; off: one
        launch per class and operator."""
        _check(lib().mhd_batch_set_worklist(self._h, 1 if on else 0), "mhd_batch_set_worklist")

    def worklist_classes(self) -> int:
        """Size classes that step in the work-list launches."""
        return int(lib().mhd_batch_worklist_classes(self._h))
