"""ctypes access to the CPU oracle (test infrastructure only).

Two builds share one interface:
  * the restatement oracle/mhd_oracle.c -> oracle/_build/liboracle_{f32,f64}.so
    (symbols orc_*), built everywhere, including the GPU machine;
  * the reference's own C/ sources -> oracle/_ref/libmhdref_{f32,f64}.so
    (symbols fluidx, advectbyzx, ...), built only where the reference
    sources exist.
Every call takes numpy arrays and the dimensions as the reference driver
passes them (C/mhd.c:62-118).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
PORT = {32: ROOT / "oracle" / "_build" / "liboracle_f32.so", 64: ROOT / "oracle" / "_build" / "liboracle_f64.so"}
REF = {32: ROOT / "oracle" / "_ref" / "libmhdref_f32.so", 64: ROOT / "oracle" / "_ref" / "libmhdref_f64.so"}
# the reference's C/ built without optimisation, as its own makefile does (timing only)
REF_O0 = ROOT / "oracle" / "_ref" / "libmhdref_f32_O0.so"


def build() -> None:
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "all"], check=True)


class Oracle:
    def __init__(self, bits: int = 32, kind: str = "port"):
        path = REF_O0 if kind == "ref_O0" else (PORT if kind == "port" else REF)[bits]
        if not path.exists():
            build()
        if not path.exists():
            raise FileNotFoundError(path)
        self.kind = kind
        self.dtype = np.float32 if bits == 32 else np.float64
        real = C.c_float if bits == 32 else C.c_double
        self._real = real
        L = C.CDLL(str(path))
        pre = "orc_" if kind == "port" else ""
        vp, ip, rp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(real)
        self._f = {}
        for name, res, args in [
            ("fluidx", None, [vp, vp, ip, ip, ip, rp, vp, vp, C.c_int]),
            ("advectbyzx", None, [vp, vp, ip, ip, ip, rp, vp, vp]),
            ("transpose12", None, [vp, vp, vp, vp, ip, ip, ip, C.c_int]),
            ("transpose13", None, [vp, vp, vp, vp, ip, ip, ip]),
            ("copy_matrix", None, [vp, vp, ip, ip, ip, vp, vp]),
            ("calcfl", real, [vp, vp, ip, ip, ip]),
        ]:
            fn = getattr(L, pre + name)
            fn.restype = res
            fn.argtypes = args
            self._f[name] = fn
        if kind == "port":
            L.mhd_init_turbulence.restype = C.c_int
            L.mhd_init_turbulence.argtypes = [vp, vp, C.c_int, C.c_int, C.c_ulonglong, C.c_double, C.c_double,
                                              C.c_double, C.c_double, C.c_double, C.c_int, C.c_int]
            L.mhd_init_vortex.restype = C.c_int
            L.mhd_init_vortex.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.c_double,
                                          C.c_double, C.c_double, C.c_double, C.c_double]
            L.orc_strang_steps.restype = C.c_int
            L.orc_strang_steps.argtypes = [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                           real, rp, rp]
            L.orc_set_threads.argtypes = [C.c_int]
            L.orc_max_threads.restype = C.c_int
        self._L = L

    def _a(self, x):
        assert isinstance(x, np.ndarray) and x.dtype == self.dtype and x.flags["C_CONTIGUOUS"]
        return x.ctypes.data

    @staticmethod
    def _d(nx, ny, nz):
        return C.byref(C.c_int(nx)), C.byref(C.c_int(ny)), C.byref(C.c_int(nz))

    def fluidx(self, u, b, nx, ny, nz, dt, uu, ub):
        self._f["fluidx"](self._a(u), self._a(b), *self._d(nx, ny, nz), C.byref(self._real(dt)), self._a(uu),
                          self._a(ub), 0)

    def advectbyzx(self, u, b, nx, ny, nz, dt, uu, ub):
        self._f["advectbyzx"](self._a(u), self._a(b), *self._d(nx, ny, nz), C.byref(self._real(dt)),
                              self._a(uu), self._a(ub))

    def transpose12(self, u, b, uu, ub, nx, ny, nz):
        self._f["transpose12"](self._a(u), self._a(b), self._a(uu), self._a(ub), *self._d(nx, ny, nz), 0)

    def transpose13(self, u, b, uu, ub, nx, ny, nz):
        self._f["transpose13"](self._a(u), self._a(b), self._a(uu), self._a(ub), *self._d(nx, ny, nz))

    def copy_matrix(self, u, b, nx, ny, nz, uu, ub):
        self._f["copy_matrix"](self._a(u), self._a(b), *self._d(nx, ny, nz), self._a(uu), self._a(ub))

    def calcfl(self, u, b, nx, ny, nz):
        return float(self._f["calcfl"](self._a(u), self._a(b), *self._d(nx, ny, nz)))

    def init_turbulence(self, n, seed=0, rho0=1.0, p0=1.0, mach=0.5, bx0=0.3, dbrms=0.1, kmin=2, kmax=8):
        """The package's seeded turbulence box (the same C source as
        heterogeneous_mhd_gb300.init_turbulence), built into the oracle so a
        CPU-only run needs no GPU library."""
        u = np.empty(5 * n ** 3, dtype=self.dtype)
        b = np.empty(3 * n ** 3, dtype=self.dtype)
        st = self._L.mhd_init_turbulence(self._a(u), self._a(b), n, int(self.dtype == np.float64), seed, rho0, p0,
                                         mach, bx0, dbrms, kmin, kmax)
        assert st == 0, st
        return u, b

    def init_vortex(self, nx, ny, nz, seed=0, rho0=1.0, p0=0.6, vscale=1.0, noise=1e-3, bscale=1.0):
        u = np.empty(5 * nx * ny * nz, dtype=self.dtype)
        b = np.empty(3 * nx * ny * nz, dtype=self.dtype)
        st = self._L.mhd_init_vortex(self._a(u), self._a(b), nx, ny, nz, int(self.dtype == np.float64), seed, rho0,
                                     p0, vscale, noise, bscale)
        assert st == 0, st
        return u, b

    def set_threads(self, n: int) -> None:
        if self.kind == "port":
            self._L.orc_set_threads(n)

    def max_threads(self) -> int:
        return int(self._L.orc_max_threads()) if self.kind == "port" else 1

    def strang(self, u, b, nx, ny, nz, nsteps, cfl=0.7, tf=float("inf"), t=0.0):
        """Full Strang steps (C/mhd.c:59-124) on copies; returns (u, b, t, dt, steps)."""
        u = np.array(u, dtype=self.dtype, copy=True)
        b = np.array(b, dtype=self.dtype, copy=True)
        if self.kind == "port":
            uu, ub = u.copy(), b.copy()
            tt, dt = self._real(t), self._real(0)
            s = self._L.orc_strang_steps(self._a(u), self._a(b), self._a(uu), self._a(ub), nx, ny, nz, nsteps,
                                         cfl, self._real(tf), C.byref(tt), C.byref(dt))
            return u, b, float(tt.value), float(dt.value), int(s)
        return strang_by_ops(self, u, b, nx, ny, nz, nsteps, cfl, tf, t)


def strang_by_ops(o, u, b, nx, ny, nz, nsteps, cfl=0.7, tf=float("inf"), t=0.0):
    """The time loop of C/mhd.c:59-124 written against the six operators (used
    for the reference build and for drop-in libraries with the same names)."""
    f = o.dtype
    uu, ub = u.copy(), b.copy()
    t = f(t)
    tf = f(tf)
    dt = f(0)
    s = 0
    for s in range(nsteps):
        if not (t < tf):
            break
        dt = f(np.float64(cfl) * np.float64(o.calcfl(u, b, nx, ny, nz)))
        if dt > (tf - t) / f(2):
            dt = (tf - t) / f(2)
        t = f(t + f(2) * dt)
        seq = [("F", (nx, ny, nz)), ("A", (nx, ny, nz)), ("T12", (nx, ny, nz)), ("F", (ny, nx, nz)),
               ("A", (ny, nx, nz)), ("T13", (ny, nx, nz)), ("F", (nz, nx, ny)), ("A", (nz, nx, ny)),
               ("A", (nz, nx, ny)), ("F", (nz, nx, ny)), ("T13", (nz, nx, ny)), ("A", (ny, nx, nz)),
               ("F", (ny, nx, nz)), ("T12", (ny, nx, nz)), ("A", (nx, ny, nz)), ("F", (nx, ny, nz))]
        for op, d in seq:
            if op == "F":
                o.fluidx(u, b, *d, dt, uu, ub)
                cd = d
            elif op == "A":
                o.advectbyzx(u, b, *d, dt, uu, ub)
                cd = d
            elif op == "T12":
                o.transpose12(u, b, uu, ub, *d)
                cd = (d[1], d[0], d[2])
            else:
                o.transpose13(u, b, uu, ub, *d)
                cd = (d[2], d[1], d[0])
            o.copy_matrix(u, b, *cd, uu, ub)
    else:
        s = nsteps
    return u, b, float(t), float(dt), s


def ref_src() -> str:
    """Directory of the reference's C/ sources named by MHD_REF_SRC ('' if none)."""
    import os
    d = os.environ.get("MHD_REF_SRC", "")
    return d if d and Path(d).is_dir() else ""


def have_ref() -> bool:
    return REF[32].exists() or bool(ref_src())
