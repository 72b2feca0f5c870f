"""The drop-in boundary: reference-named C functions (C/spu_function.h:1-15).

* A C driver written against the reference's call surface
  (tests/c/strang_driver.c, the loop of C/mhd.c:59-124) links unchanged
  against the reference's own C build (CPU) and against libmhd_gb300.so
  (GPU, host arrays staged, or cudaMalloc arrays used in place).
* The Python mirror of the same six operators, with host and device arrays.
"""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from _oracle import REF, strang_by_ops
from util import bitwise_equal, rel_l2_fields

ROOT = Path(__file__).resolve().parents[1]
DRIVER = ROOT / "tests" / "c" / "strang_driver.c"


def build_driver(out: Path, libdir: Path, libname: str, cuda_mem: bool = False) -> Path:
    cmd = ["gcc", "-O2", "-ffp-contract=off", str(DRIVER), "-o", str(out), f"-L{libdir}", f"-l{libname}",
           f"-Wl,-rpath,{libdir}", "-lm"]
    if cuda_mem:
        cmd[1:1] = ["-DWITH_CUDA_MEMORY", "-I/usr/local/cuda/include"]
        cmd += ["-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"]
    subprocess.run(cmd, check=True)
    return out


def run_driver(exe: Path, tmp: Path, u, b, shape, nsteps, cfl=0.7, extra=(), env=None):
    fin, fout = tmp / "in.bin", tmp / "out.bin"
    with open(fin, "wb") as f:
        f.write(u.tobytes())
        f.write(b.tobytes())
    subprocess.run([str(exe), str(fin), str(fout), *map(str, shape), str(nsteps), str(cfl), *extra], check=True,
                   env={**os.environ, **(env or {})})
    raw = np.fromfile(fout, dtype=np.float32)
    n = u.size
    return raw[:n], raw[n:n + b.size], float(raw[-1])


def test_c_driver_against_reference_build(mhd, oracle32, tmp_path):
    """CPU: the driver linked against the reference's C/ build gives the oracle's bits."""
    from _oracle import have_ref
    if not have_ref():
        pytest.skip("no reference build and no MHD_REF_SRC on this machine")
    from _oracle import build
    build()
    exe = build_driver(tmp_path / "drv_ref", REF[32].parent, "mhdref_f32")
    u0, b0 = mhd.init_vortex(16, 16, 16, seed=4)
    u, b, t = run_driver(exe, tmp_path, u0, b0, (16, 16, 16), 2)
    ref = oracle32.strang(u0, b0, 16, 16, 16, 2)
    assert bitwise_equal(u, ref[0]) and bitwise_equal(b, ref[1]) and np.float32(t) == np.float32(ref[2])


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["host", "device"])
def test_c_driver_against_gpu_library(mode, mhd, cuda, oracle32, tmp_path):
    """GPU: the same driver source linked against libmhd_gb300.so, EXACT
    arithmetic selected by the environment: the reference's bits."""
    libdir = mhd.lib_path().parent
    exe = build_driver(tmp_path / f"drv_gpu_{mode}", libdir, "mhd_gb300", cuda_mem=(mode == "device"))
    shape = (16, 12, 12)
    u0, b0 = mhd.init_vortex(*shape, seed=6)
    ref = oracle32.strang(u0, b0, *shape, 2)
    extra = ("device",) if mode == "device" else ()
    u, b, t = run_driver(exe, tmp_path, u0, b0, shape, 2, extra=extra, env={"MHD_GB300_MODE": "exact"})
    assert bitwise_equal(u, ref[0]) and bitwise_equal(b, ref[1]) and np.float32(t) == np.float32(ref[2])
    u, b, t = run_driver(exe, tmp_path, u0, b0, shape, 2, extra=extra, env={"MHD_GB300_MODE": "fast"})
    e = rel_l2_fields(u, b, ref[0], ref[1])
    assert max(e.values()) < 1e-5, e


class _DropIn:
    """The Python drop-in functions behind the oracle's operator interface."""

    dtype = np.float32

    def __init__(self, mhd, torch=None):
        self.m, self.torch = mhd, torch

    def _w(self, a):
        return self.torch.from_numpy(a).cuda() if self.torch is not None else a

    def fluidx(self, u, b, nx, ny, nz, dt, uu, ub):
        self.m.fluidx(u, b, nx, ny, nz, dt, uu, ub)

    def advectbyzx(self, u, b, nx, ny, nz, dt, uu, ub):
        self.m.advectbyzx(u, b, nx, ny, nz, dt, uu, ub)

    def transpose12(self, u, b, uu, ub, nx, ny, nz):
        self.m.transpose12(u, b, uu, ub, nx, ny, nz)

    def transpose13(self, u, b, uu, ub, nx, ny, nz):
        self.m.transpose13(u, b, uu, ub, nx, ny, nz)

    def copy_matrix(self, u, b, nx, ny, nz, uu, ub):
        self.m.copy_matrix(u, b, nx, ny, nz, uu, ub)

    def calcfl(self, u, b, nx, ny, nz):
        return self.m.calcfl(u, b, nx, ny, nz)


@pytest.mark.gpu
def test_python_dropin_host_arrays_exact(mhd, cuda, oracle32):
    shape = (12, 8, 8)
    u0, b0 = mhd.init_vortex(*shape, seed=9)
    ref = oracle32.strang(u0, b0, *shape, 2)
    mhd.set_dropin_mode(exact=True)
    try:
        u, b, t, _, _ = strang_by_ops(_DropIn(mhd), u0.copy(), b0.copy(), *shape, 2)
    finally:
        mhd.set_dropin_mode(exact=False)
    assert bitwise_equal(u, ref[0]) and bitwise_equal(b, ref[1])


@pytest.mark.gpu
def test_python_dropin_device_tensors(mhd, cuda, oracle32):
    torch = cuda
    nx, ny, nz = 32, 16, 16
    u0, b0 = mhd.init_vortex(nx, ny, nz, seed=10)
    uo = np.full_like(u0, 7)
    oracle32.fluidx(uo, b0.copy(), nx, ny, nz, 0.05, u0.copy(), b0.copy())
    du, db = torch.from_numpy(u0).cuda(), torch.from_numpy(b0).cuda()
    dout = torch.full_like(du, 7)
    mhd.set_dropin_mode(exact=True)
    try:
        mhd.fluidx(dout, db, nx, ny, nz, 0.05, du, db)
    finally:
        mhd.set_dropin_mode(exact=False)
    assert bitwise_equal(dout.cpu().numpy(), uo)


@pytest.mark.gpu
def test_dropin_transpose13_error_leaves_outputs(mhd, cuda):
    u = np.arange(5 * 24, dtype=np.float32)
    b = np.arange(3 * 24, dtype=np.float32)
    uo, bo = np.full_like(u, -1), np.full_like(b, -1)
    with pytest.raises(mhd.MhdError):
        mhd.transpose13(uo, bo, u, b, 4, 3, 2)
    assert (uo == -1).all() and (bo == -1).all()
