"""Failure detection and resume on the GPU, without a GPU fault.

* A bounded device wait that nothing completes gives up after its limit, the
  host reads MHD_ERR_TIMEOUT from mhd_check, and the context keeps working:
  after mhd_clear_errors the next steps are bit for bit those of a context
  that never timed out.  (The reference's CUDA path exits on any error,
  Cuda/cuda_function.h:4-12; it has no recovery to compare with.)
* A run stopped at a checkpoint and resumed in a new context from the file
  reproduces the uninterrupted run bit for bit, time included.
"""
import numpy as np
import pytest

from util import bitwise_equal

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_recovers(mhd, cuda):
    n = 16
    u0, b0 = mhd.init_vortex(n, n, n, seed=1)
    with mhd.Context(n, n, n) as ctx:
        ctx.set_state(u0, b0)
        ctx.step(1)
        assert ctx.check() == mhd.MHD_OK
        for bad in (0.0, -1.0, 5.0):
            with pytest.raises(mhd.MhdError):
                ctx.selftest_wait(bad)
        ctx.selftest_wait(0.01)
        assert ctx.check() == mhd.MHD_ERR_TIMEOUT
        assert ctx.check() == mhd.MHD_ERR_TIMEOUT  # the word stays set until cleared
        ctx.clear_errors()
        assert ctx.check() == mhd.MHD_OK
        ctx.step(2)
        assert ctx.check() == mhd.MHD_OK
        u, b = ctx.get_state()
    with mhd.Context(n, n, n) as ref:
        ref.set_state(u0, b0)
        ref.step(3)
        ru, rb = ref.get_state()
    assert bitwise_equal(u, ru) and bitwise_equal(b, rb)


@pytest.mark.parametrize("exact", [False, True])
def test_checkpoint_resume_is_bitwise(exact, mhd, cuda, tmp_path):
    n = 32
    u0, b0 = mhd.init_turbulence(n, seed=4)
    with mhd.Context(n, n, n, exact=exact) as ctx:
        ctx.set_state(u0, b0)
        ctx.step(6)
        uf, bf = ctx.get_state()
        tf, dtf, _ = ctx.time()
    path = tmp_path / "state.chk"
    with mhd.Context(n, n, n, exact=exact) as ctx:
        ctx.set_state(u0, b0)
        ctx.step(3)
        u, b = ctx.get_state()
        t, _, s = ctx.time()
        mhd.checkpoint_save(path, u, b, n, n, n, t=t, step=s)
    u2, b2, shape, t2, s2 = mhd.checkpoint_load(path)
    assert shape == (n, n, n) and s2 == 3 and t2 == t
    with mhd.Context(*shape, exact=exact) as ctx:
        ctx.set_state(u2, b2)
        ctx.set_time(t2)
        ctx.step(3)
        ur, br = ctx.get_state()
        tr, dtr, _ = ctx.time()
        assert ctx.check() == mhd.MHD_OK
    assert bitwise_equal(ur, uf) and bitwise_equal(br, bf)
    assert np.float32(tr) == np.float32(tf) and np.float32(dtr) == np.float32(dtf)
