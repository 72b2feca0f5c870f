"""mhd_calcfl_noalloc: the CFL reduction for callers that cannot let the
library allocate device memory (a stream being captured into a CUDA graph, a
host framework that owns all device memory, an allocation-free real-time
loop).  It keeps its scratch in a fixed device array instead of cudaMalloc.

Checked through the C ABI against the regular entry point (mhd_op_calcfl of
a FAST context) on two calls in a row with different grids, so a second call
must not be affected by what the first one left in the shared array.  This
file sorts last so that a run stopping at the first failure has already run
every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6  # the per-operator tolerance of the FAST kernels (test_gpu_ops.py)


def _noalloc(mhd, torch, du, db, nx, ny, nz):
    out = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = mhd.lib().mhd_calcfl_noalloc(du.data_ptr(), db.data_ptr(), nx, ny, nz, out.data_ptr(),
                                      C.c_void_p(stream))
    assert st == mhd.MHD_OK
    torch.cuda.synchronize()
    return float(out.item())


def test_noalloc_calcfl_matches_calcfl_twice(mhd, cuda):
    torch = cuda
    cases = [((64, 64, 64), mhd.init_vortex(64, 64, 64, seed=21)),
             ((48, 32, 16), mhd.init_vortex(48, 32, 16, seed=22, vscale=2.0))]
    with mhd.Context(1, 1, 1) as ctx:
        for (nx, ny, nz), (u, b) in cases:
            du, db = torch.from_numpy(u).cuda(), torch.from_numpy(b).cuda()
            got = _noalloc(mhd, torch, du, db, nx, ny, nz)
            ref = ctx.op_calcfl(du, db, nx, ny, nz)
            assert np.isfinite(got) and got > 0
            assert abs(got - ref) <= REL_TOL * abs(ref), (got, ref)


def test_noalloc_calcfl_rejects_oversized_grid(mhd, cuda):
    torch = cuda
    d = torch.zeros(8, device="cuda")
    out = torch.zeros(1, device="cuda")
    st = mhd.lib().mhd_calcfl_noalloc(d.data_ptr(), d.data_ptr(), 1024, 1024, 256, out.data_ptr(), None)
    assert st == 5  # MHD_ERR_UNSUPPORTED: more cells than the static scratch covers
