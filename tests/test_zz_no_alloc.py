"""mhd_calcfl_noalloc: the CFL reduction for callers that cannot let the
library allocate device memory (a stream being captured into a CUDA graph, a
host framework that owns all device memory, an allocation-free real-time
loop).  It keeps its scratch in a fixed device array instead of cudaMalloc.

Checked through the C ABI on two calls in a row with different grids (so a
second call must not be affected by what the first one left in the shared
array) against the regular entry point (mhd_op_calcfl of a FAST context) and
against the CPU oracle of the reference's calcfl (C/calcfl.c:13-63), including
its NaN semantics: max_2num (C/calcfl.c:91-101) restarts the running maximum
after a NaN cell, so a NaN in the middle is skipped and a NaN in the last cell
makes the result NaN.  This file sorts last so that a run stopping at the
first failure has already run every other test; it also passes alone in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6     # the per-operator tolerance of the FAST kernels (test_gpu_ops.py)
ORACLE_TOL = 2e-6  # FAST calcfl against the oracle (test_gpu_ops.py, test_calcfl_nan_semantics)


def _noalloc(mhd, torch, du, db, nx, ny, nz):
    out = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = mhd.lib().mhd_calcfl_noalloc(du.data_ptr(), db.data_ptr(), nx, ny, nz, out.data_ptr(),
                                      C.c_void_p(stream))
    assert st == mhd.MHD_OK
    torch.cuda.synchronize()
    return float(out.item())


def test_noalloc_calcfl_matches_calcfl_twice(mhd, cuda, oracle32):
    torch = cuda
    cases = [((64, 64, 64), mhd.init_vortex(64, 64, 64, seed=21)),
             ((48, 32, 16), mhd.init_vortex(48, 32, 16, seed=22, vscale=2.0))]
    with mhd.Context(1, 1, 1) as ctx:
        for (nx, ny, nz), (u, b) in cases:
            du, db = torch.from_numpy(u).cuda(), torch.from_numpy(b).cuda()
            got = _noalloc(mhd, torch, du, db, nx, ny, nz)
            ref = ctx.op_calcfl(du, db, nx, ny, nz)
            orc = oracle32.calcfl(u, b, nx, ny, nz)
            assert np.isfinite(got) and got > 0
            assert abs(got - ref) <= REL_TOL * abs(ref), (got, ref)
            assert abs(got - orc) <= ORACLE_TOL * abs(orc), (got, orc)


@pytest.mark.parametrize("where", ["middle", "last"])
def test_noalloc_calcfl_nan_cells_match_oracle(where, mhd, cuda, oracle32):
    """A NaN density in a middle cell, then in the last cell, on two calls in
    a row each: the restarted maximum, and NaN when nothing follows."""
    torch = cuda
    nx, ny, nz = 40, 24, 16
    u, b = mhd.init_vortex(nx, ny, nz, seed=23)
    nc = nx * ny * nz
    cell = nc // 2 + 17 if where == "middle" else nc - 1
    u[cell * 5] = np.nan
    orc = oracle32.calcfl(u, b, nx, ny, nz)
    du, db = torch.from_numpy(u).cuda(), torch.from_numpy(b).cuda()
    for _ in range(2):
        got = _noalloc(mhd, torch, du, db, nx, ny, nz)
        if where == "last":
            assert np.isnan(got) and np.isnan(orc)
        else:
            assert np.isfinite(got) and abs(got - orc) <= ORACLE_TOL * abs(orc), (got, orc)


def test_noalloc_calcfl_rejects_oversized_grid(mhd, cuda):
    torch = cuda
    d = torch.zeros(8, device="cuda")
    out = torch.zeros(1, device="cuda")
    st = mhd.lib().mhd_calcfl_noalloc(d.data_ptr(), d.data_ptr(), 1024, 1024, 256, out.data_ptr(), None)
    assert st == 5  # MHD_ERR_UNSUPPORTED: more cells than the static scratch covers
