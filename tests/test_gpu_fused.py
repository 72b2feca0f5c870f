"""The fused Strang step (MHD_FUSED): sweeps along y and z read the
untransposed state and transpose tiles in shared memory, so the step has no
transpose kernels.  It computes exactly what the plain step computes: with
the EXACT kernels its state is bit for bit the reference's (the 64^3
checksums of the reference C path) and the plain step's."""
import numpy as np
import pytest

from util import bitwise_equal, checksums, rel_l2_fields, sha

pytestmark = pytest.mark.gpu

FAST_FUSED_TOL = 1e-6  # relative L2 per field, fused vs plain FAST, after 5 steps


def run(mhd, u0, b0, shape, nsteps, fused, exact=False, graphs=True):
    with mhd.Context(*shape, exact=exact) as ctx:
        ctx.use_graphs(graphs)
        ctx.set_state(u0, b0)
        ctx.step(nsteps, cfl=0.7, fused=fused)
        assert ctx.check() == mhd.MHD_OK
        u, b = ctx.get_state()
        t, _, s = ctx.time()
        assert s == nsteps
        return u, b, t


def test_fused_exact_reference_checksums_64(mhd, cuda):
    ck = checksums()["f32"]
    u0, b0 = mhd.init_vortex(64, 64, 64, seed=0)
    with mhd.Context(64, 64, 64, exact=True) as ctx:
        ctx.set_state(u0, b0)
        done = 0
        for target in (1, 10, 100):
            ctx.step(target - done, cfl=0.7, fused=True)
            done = target
            u, b = ctx.get_state()
            assert sha(u, b) == ck[str(target)]["sha256"], f"after {target} steps"


@pytest.mark.parametrize("shape,init", [((32, 32, 32), "vortex"), ((128, 128, 128), "turb"),
                                         ((256, 256, 256), "turb"), ((64, 32, 32), "vortex")])
def test_fused_exact_equals_plain(shape, init, mhd, cuda):
    if init == "vortex":
        u0, b0 = mhd.init_vortex(*shape, seed=3)
    else:
        u0, b0 = mhd.init_turbulence(shape[0], seed=3)
    for graphs in (True, False):
        up, bp, tp = run(mhd, u0, b0, shape, 3, fused=False, exact=True, graphs=graphs)
        uf, bf, tf = run(mhd, u0, b0, shape, 3, fused=True, exact=True, graphs=graphs)
        assert bitwise_equal(uf, up) and bitwise_equal(bf, bp), (shape, graphs)
        assert tf == tp


def test_fused_fast_matches_plain(mhd, cuda):
    n = 256
    u0, b0 = mhd.init_turbulence(n, seed=5)
    up, bp, _ = run(mhd, u0, b0, (n, n, n), 5, fused=False)
    uf, bf, _ = run(mhd, u0, b0, (n, n, n), 5, fused=True)
    e = rel_l2_fields(uf, bf, up, bp)
    assert max(e.values()) <= FAST_FUSED_TOL, e


def test_fused_non_cubic_runs_where_plain_cannot(mhd, cuda):
    """No transpose13, so ny != nz is allowed; div B stays at round-off."""
    shape = (64, 32, 128)
    u0, b0 = mhd.init_vortex(*shape, seed=2)
    with mhd.Context(*shape) as ctx:
        ctx.set_state(u0, b0)
        with pytest.raises(mhd.MhdError):
            ctx.step(1, cfl=0.7, fused=False)
        ctx.step(5, cfl=0.7, fused=True)
        u, b = ctx.get_state()
        assert np.all(np.isfinite(u)) and np.all(np.isfinite(b))
        assert ctx.divb_max() <= 2e-6 * float(np.abs(b).max())


@pytest.mark.parametrize("knobs", [{}, {"sweep.k": 2}, {"sweep.k": 8}, {"sweep.slots": 2},
                                   {"sweep.k": 2, "sweep.slots": 2}, {"sweep.kernel": 3}])
@pytest.mark.parametrize("shape", [(32, 64, 64), (128, 32, 32), (64, 128, 128)])
def test_fused_sweep_kernels_exact_vs_oracle(shape, knobs, mhd, cuda, oracle32):
    """Every launch shape of the sweep kernels along y and z (the walking
    advectbyzx with 2, 4 or 8 planes per CTA and 2 or 3 chunk buffers, and the
    marching one by sweep.kernel = 3; fluidx with its tensor-copied tiles) on
    boxes whose three axes have different lengths: EXACT fused steps bit for
    bit against the oracle of the reference's C path.  The x sweeps keep
    their own kernels."""
    from heterogeneous_mhd_gb300 import autotune
    u0, b0 = mhd.init_vortex(*shape, seed=4, vscale=1.3)
    ref = oracle32.strang(u0, b0, *shape, 2)
    try:
        autotune.apply(knobs)
        u, b, t = run(mhd, u0, b0, shape, 2, fused=True, exact=True)
    finally:
        autotune.apply({k: 0 for k in knobs})
    assert bitwise_equal(u, ref[0]) and bitwise_equal(b, ref[1]), (shape, knobs)
    assert np.float32(t) == np.float32(ref[2])


def test_fused_sweeps_of_512_cells_exact_vs_oracle(mhd, cuda):
    """Pencils of 512 cells along y and z: the fluidx sweep moves each CTA's
    rows in two tensor boxes of 256 and runs four 128-thread pencils; EXACT
    fused steps bit for bit against the oracle of the reference's C path and
    against the plain step.  The reference's loop transposes x with z, so its
    boxes have ny == nz."""
    from _oracle import Oracle
    oracle32 = Oracle(32, "port")
    shape = (32, 512, 512)
    u0, b0 = mhd.init_vortex(*shape, seed=6, vscale=1.2)
    ref = oracle32.strang(u0, b0, *shape, 2)
    u, b, t = run(mhd, u0, b0, shape, 2, fused=True, exact=True)
    assert bitwise_equal(u, ref[0]) and bitwise_equal(b, ref[1]), shape
    assert np.float32(t) == np.float32(ref[2])
    up, bp, tp = run(mhd, u0, b0, shape, 2, fused=False, exact=True)
    assert bitwise_equal(u, up) and bitwise_equal(b, bp) and t == tp
