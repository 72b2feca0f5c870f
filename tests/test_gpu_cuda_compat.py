"""The reference's CUDA-side names (Cuda/cuda_subroutine.h:4-12) on device
arrays, against the oracle of the C path, bit for bit with the EXACT
kernels.  cuda_fluidx and cuda_advectbyzx update in place like the
reference's kernels; cuda_cfl returns 1/max speed."""
import ctypes as C

import numpy as np
import pytest

from util import bitwise_equal

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
    L.cuda_transpose13(ut.data_ptr(), bt.data_ptr(), ud.data_ptr(), bd.data_ptr(), *dd, *hd)
    assert L.mhd_last_error() == 0
    u13, b13 = np.empty_like(uo), np.empty_like(bo)
    oracle32.transpose13(u13, b13, uo.copy(), bo.copy(), nx, ny, nz)
    assert bitwise_equal(ut.cpu().numpy(), u13) and bitwise_equal(bt.cpu().numpy(), b13)
