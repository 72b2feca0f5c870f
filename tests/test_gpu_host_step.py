"""mhd_step_host: steps on a state held in host memory, with the copies in
and out overlapped with the step (the first CFL pass per chunk of the state
as it lands, b copied out while the last fluidx runs).  It must give what
mhd_set_state + mhd_step + mhd_get_state give, bit for bit (C/mhd.c:59-124
on host arrays)."""
import numpy as np
import pytest

from util import bitwise_equal

pytestmark = pytest.mark.gpu


def same_clock(a, b) -> bool:
    """(t, dt, steps) equal bit for bit (NaN included)."""
    return np.array(a[:2], dtype=np.float64).tobytes() == np.array(b[:2], dtype=np.float64).tobytes() and a[2] == b[2]


def three_calls(mhd, u0, b0, shape, nsteps, fused, exact):
    with mhd.Context(*shape, exact=exact) as ctx:
        ctx.set_state(u0, b0)
        ctx.step(nsteps, cfl=0.7, fused=fused)
        st = ctx.check()
        u, b = ctx.get_state()
        return u, b, ctx.time(), st


@pytest.mark.parametrize("nsteps", [1, 3])
@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("fused", [False, True])
def test_step_host_equals_set_step_get(fused, exact, nsteps, mhd, cuda):
    shape = (64, 64, 64)
    u0, b0 = mhd.init_vortex(*shape, seed=4, vscale=1.1)
    ur, br, tr, _ = three_calls(mhd, u0, b0, shape, nsteps, fused, exact)
    with mhd.Context(*shape, exact=exact) as ctx:
        u, b = u0.copy(), b0.copy()
        ctx.step_host(u, b, nsteps, cfl=0.7, fused=fused)
        assert ctx.check() == mhd.MHD_OK
        assert bitwise_equal(u, ur) and bitwise_equal(b, br), (fused, exact, nsteps)
        t, dt, s = ctx.time()
        assert same_clock((t, dt, s), tr)
        # the device copy of the state is the result as well
        ud, bd = ctx.get_state()
        assert bitwise_equal(ud, ur) and bitwise_equal(bd, br)
        # and the clock carries on: a second call continues from t
        ctx.step_host(u, b, 1, cfl=0.7, fused=fused)
        assert ctx.time()[2] == nsteps + 1 and ctx.time()[0] > t


def test_step_host_uneven_chunks_and_nan_index(mhd, cuda):
    """76800 cells: eight copy-in chunks of 9728 cells and a short last one.
    A NaN in the fourth chunk must be reported by its index in the box (the
    CFL pass's restart after the last NaN), as the one-pass calcfl does."""
    shape = (48, 40, 40)
    u0, b0 = mhd.init_vortex(*shape, seed=5)
    for nan_cell in (None, 30011, 48 * 40 * 40 - 1):
        u1 = u0.copy()
        if nan_cell is not None:
            u1[5 * nan_cell + 4] = np.nan
        ur, br, tr, str_ = three_calls(mhd, u1, b0, shape, 1, False, True)
        with mhd.Context(*shape, exact=True) as ctx:
            u, b = u1.copy(), b0.copy()
            ctx.step_host(u, b, 1, cfl=0.7, fused=False)
            assert ctx.check() == str_
            assert bitwise_equal(u, ur) and bitwise_equal(b, br), nan_cell
            assert same_clock(ctx.time(), tr), (nan_cell, ctx.time(), tr)


def test_step_host_pinned_tensors_fused_256(mhd, cuda):
    """The benchmark's form: pinned host tensors, the 256^3 turbulence box,
    FAST fused steps."""
    import torch

    n = 256
    u0, b0 = mhd.init_turbulence(n, seed=2)
    ur, br, tr, _ = three_calls(mhd, u0, b0, (n, n, n), 2, True, False)
    hu = torch.empty(u0.size, dtype=torch.float32, pin_memory=True)
    hb = torch.empty(b0.size, dtype=torch.float32, pin_memory=True)
    hu.numpy()[:] = u0
    hb.numpy()[:] = b0
    with mhd.Context(n, n, n) as ctx:
        ctx.step_host(hu, hb, 2, cfl=0.7, fused=True)
        assert ctx.check() == mhd.MHD_OK
        assert bitwise_equal(hu.numpy(), ur) and bitwise_equal(hb.numpy(), br)
        assert same_clock(ctx.time(), tr)


def test_step_host_rejects_bad_arguments(mhd, cuda):
    with mhd.Context(32, 32, 32) as ctx:
        u, b = mhd.init_vortex(32, 32, 32, seed=0)
        with pytest.raises(ValueError):
            ctx.step_host(u[:-5], b)
        with pytest.raises(ValueError):
            ctx.step_host(u.astype(np.float64), b)
        with pytest.raises(mhd.MhdError):
            ctx.step_host(u, b, 0)
    with mhd.Context(32, 16, 32) as ctx:  # the plain step needs ny == nz
        u, b = mhd.init_vortex(32, 16, 32, seed=0)
        with pytest.raises(mhd.MhdError):
            ctx.step_host(u, b, 1, fused=False)


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("shape", [(128, 128, 128), (128, 64, 256), (256, 256, 256)])
def test_step_host_fused_tail_in_slabs(shape, exact, mhd, cuda):
    """Grids whose fused tail runs in slabs of planes along z (the y fluidx,
    x advectbyzx and x fluidx of each slab, each slab copied out when final):
    bit for bit the three-call result, EXACT and FAST.  The slab tail
    launches the three operators once per slab (8 slabs), which the launch
    count shows."""
    nx, ny, nz = shape
    u0, b0 = mhd.init_turbulence(nx, seed=9) if nx == ny == nz else mhd.init_vortex(*shape, seed=9)
    ur, br, tr, _ = three_calls(mhd, u0, b0, shape, 2, True, exact)
    with mhd.Context(*shape, exact=exact) as ctx:
        u, b = u0.copy(), b0.copy()
        n0 = ctx.launch_count()
        ctx.step_host(u, b, 2, cfl=0.7, fused=True)
        launches = ctx.launch_count() - n0
        assert ctx.check() == mhd.MHD_OK
        assert bitwise_equal(u, ur) and bitwise_equal(b, br), (shape, exact)
        assert same_clock(ctx.time(), tr)
    # 8 chunked CFL passes, a whole step (13 launches), a step whose tail is 3 x 8 slab launches
    assert launches >= 8 + 13 + 10 + 24, launches
