"""The reference's CUDA-side names (Cuda/cuda_subroutine.h:4-12) on device
arrays, against the oracle of the C path, bit for bit with the EXACT
kernels.  cuda_fluidx and cuda_advectbyzx update in place like the
reference's kernels; cuda_cfl returns 1/max speed."""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from util import bitwise_equal, rel_l2_fields

pytestmark = pytest.mark.gpu


@pytest.fixture
def exact(mhd, cuda):
    mhd.set_dropin_mode(exact=True)
    yield mhd.lib()
    mhd.set_dropin_mode(exact=False)


def dims(nx, ny, nz):
    h = [C.c_int(nx), C.c_int(ny), C.c_int(nz)]
    return [C.byref(x) for x in h]


@pytest.mark.parametrize("shape", [(32, 16, 32), (64, 8, 64), (24, 5, 24)])
def test_cuda_names_match_oracle(shape, mhd, cuda, exact, oracle32):
    torch = cuda
    L = exact
    nx, ny, nz = shape
    u0, b0 = mhd.init_vortex(nx, ny, nz, seed=9)
    dev = lambda a: torch.from_numpy(a.copy()).cuda()
    dd = dims(nx, ny, nz)   # the "device" dims: unused by the shims
    hd = dims(nx, ny, nz)
    # cuda_cfl
    ud, bd = dev(u0), dev(b0)
    dt_dev = torch.zeros(1, dtype=torch.float32, device="cuda")
    c_scr = torch.zeros(ny * nz, dtype=torch.float32, device="cuda")
    h_dt = C.c_float(0)
    L.cuda_cfl(ud.data_ptr(), bd.data_ptr(), *dd, dt_dev.data_ptr(), c_scr.data_ptr(), *hd, C.byref(h_dt))
    assert L.mhd_last_error() == 0
    ref = np.float32(oracle32.calcfl(u0.copy(), b0.copy(), nx, ny, nz))
    assert np.float32(h_dt.value) == ref and np.float32(dt_dev.item()) == ref
    dt = np.float32(0.3) * ref
    dt_dev.fill_(float(dt))
    # cuda_fluidx: u <- fluidx(u, b) in place
    L.cuda_fluidx(ud.data_ptr(), bd.data_ptr(), *dd, dt_dev.data_ptr(), *hd)
    assert L.mhd_last_error() == 0
    uo = u0.copy()
    oracle32.fluidx(uo, b0.copy(), nx, ny, nz, dt, u0.copy(), b0.copy())
    assert bitwise_equal(ud.cpu().numpy(), uo)
    # cuda_advectbyzx: b <- advectbyzx(u, b) in place
    tmp = torch.zeros(nx * ny * nz, dtype=torch.float32, device="cuda")
    L.cuda_advectbyzx(ud.data_ptr(), bd.data_ptr(), *dd, dt_dev.data_ptr(), tmp.data_ptr(), *hd)
    assert L.mhd_last_error() == 0
    bo = b0.copy()
    oracle32.advectbyzx(uo.copy(), bo, nx, ny, nz, dt, uo.copy(), b0.copy())
    assert bitwise_equal(bd.cpu().numpy(), bo)
    # cuda_transpose12 / 13
    ut, bt = torch.empty_like(ud), torch.empty_like(bd)
    L.cuda_transpose12(ut.data_ptr(), bt.data_ptr(), ud.data_ptr(), bd.data_ptr(), *dd, *hd)
    assert L.mhd_last_error() == 0
    u12, b12 = np.empty_like(uo), np.empty_like(bo)
    oracle32.transpose12(u12, b12, uo.copy(), bo.copy(), nx, ny, nz)
    assert bitwise_equal(ut.cpu().numpy(), u12) and bitwise_equal(bt.cpu().numpy(), b12)
    # copied back into (u, b) as by Cuda/cuda_transpose12.cu:30-34
    assert bitwise_equal(ud.cpu().numpy(), u12) and bitwise_equal(bd.cpu().numpy(), b12)
    ud.copy_(torch.from_numpy(uo))
    bd.copy_(torch.from_numpy(bo))
    L.cuda_transpose13(ut.data_ptr(), bt.data_ptr(), ud.data_ptr(), bd.data_ptr(), *dd, *hd)
    assert L.mhd_last_error() == 0
    u13, b13 = np.empty_like(uo), np.empty_like(bo)
    oracle32.transpose13(u13, b13, uo.copy(), bo.copy(), nx, ny, nz)
    assert bitwise_equal(ut.cpu().numpy(), u13) and bitwise_equal(bt.cpu().numpy(), b13)
    assert bitwise_equal(ud.cpu().numpy(), u13) and bitwise_equal(bd.cpu().numpy(), b13)


@pytest.mark.parametrize("shape", [(8, 6, 1), (1, 6, 8), (5, 3, 1)])
def test_cuda_transpose13_degenerate_boxes(shape, mhd, cuda, exact):
    """nz == 1 and nx == 1, the two extra cases of Cuda/cuda_transpose13.cu:27-42:
    out(k, j, i) = in(i, j, k) with the components of C/transpose13.c
    (u: rho, m_z, m_y, m_x, E; b: b_z, b_y, b_x)."""
    torch = cuda
    L = exact
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 7 + nz)
    u = rng.standard_normal(5 * nx * ny * nz).astype(np.float32)
    b = rng.standard_normal(3 * nx * ny * nz).astype(np.float32)
    ud, bd = torch.from_numpy(u.copy()).cuda(), torch.from_numpy(b.copy()).cuda()
    ut, bt = torch.empty_like(ud), torch.empty_like(bd)
    L.cuda_transpose13(ut.data_ptr(), bt.data_ptr(), ud.data_ptr(), bd.data_ptr(), *dims(nx, ny, nz),
                       *dims(nx, ny, nz))
    assert L.mhd_last_error() == 0
    U = u.reshape(nz, ny, nx, 5)
    B = b.reshape(nz, ny, nx, 3)
    want_u = U.transpose(2, 1, 0, 3)[..., [0, 3, 2, 1, 4]]
    want_b = B.transpose(2, 1, 0, 3)[..., [2, 1, 0]]
    assert bitwise_equal(ut.cpu().numpy(), want_u.reshape(-1))
    assert bitwise_equal(bt.cpu().numpy(), want_b.reshape(-1))
    assert bitwise_equal(ud.cpu().numpy(), want_u.reshape(-1))


DRIVER = Path(__file__).resolve().parent / "c" / "cuda_main_driver.c"


def _build_cuda_main_driver(mhd, out):
    libdir = mhd.lib_path().parent
    root = Path(__file__).resolve().parents[1]
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", str(DRIVER), "-o", str(out), f"-I{root / 'include'}",
                    "-I/usr/local/cuda/include", f"-L{libdir}", "-lmhd_gb300", f"-Wl,-rpath,{libdir}",
                    "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64", "-lm"], check=True)
    return out


@pytest.mark.parametrize("shape", [(16, 12, 12), (32, 16, 16)])
def test_cuda_main_driver_against_oracle(shape, mhd, cuda, oracle32, tmp_path):
    """A driver that replays Cuda/cuda_main.cu:72-116 through the cuda_* names
    (device arrays, device and host dimension copies, the reference's scratch
    arrays), linked against libmhd_gb300.so: EXACT bit for bit against the
    oracle of the C path after three steps, FAST within the one-step tolerance
    after one."""
    exe = _build_cuda_main_driver(mhd, tmp_path / "cuda_main_driver")
    u0, b0 = mhd.init_vortex(*shape, seed=12)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    fin.write_bytes(u0.tobytes() + b0.tobytes())

    def run(nsteps, mode):
        subprocess.run([str(exe), str(fin), str(fout), *map(str, shape), str(nsteps), "0.9"], check=True,
                       env={**os.environ, "MHD_GB300_MODE": mode})
        raw = np.fromfile(fout, dtype=np.float32)
        return raw[:u0.size], raw[u0.size:u0.size + b0.size], raw[-1]

    ref = oracle32.strang(u0, b0, *shape, 3, cfl=0.9)
    u, b, t = run(3, "exact")
    assert bitwise_equal(u, ref[0]) and bitwise_equal(b, ref[1]) and t == np.float32(ref[2])
    ref1 = oracle32.strang(u0, b0, *shape, 1, cfl=0.9)
    u, b, _ = run(1, "fast")
    e = rel_l2_fields(u, b, ref1[0], ref1[1])
    assert max(e.values()) < 1e-5, e
