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


def numpy_diagnostics(u, b, shape):
    nx, ny, nz = shape
    U = u.reshape(nz, ny, nx, 5).astype(np.float64)
    B = b.reshape(nz, ny, nx, 3).astype(np.float64)
    rho, m, e = U[..., 0], U[..., 1:4], U[..., 4]
    bx = 0.5 * (B[..., 0] + np.roll(B[..., 0], -1, axis=2))
    by = 0.5 * (B[..., 1] + np.roll(B[..., 1], -1, axis=1))
    bz = 0.5 * (B[..., 2] + np.roll(B[..., 2], -1, axis=0))
    m2 = (m ** 2).sum(-1)
    ek, em = 0.5 * m2 / rho, 0.5 * (bx ** 2 + by ** 2 + bz ** 2)
    p = (5.0 / 3.0 - 1.0) * (e - ek - em)
    div = np.abs((np.roll(B[..., 0], -1, axis=2) - B[..., 0]) + (np.roll(B[..., 1], -1, axis=1) - B[..., 1])
                 + (np.roll(B[..., 2], -1, axis=0) - B[..., 2]))
    return {"min_rho": rho.min(), "min_p": p.min(), "max_divb": div.max(), "mass": rho.sum(), "kinetic": ek.sum(),
            "magnetic": em.sum(), "energy": e.sum(), "max_speed": (np.sqrt(m2) / rho).max()}


@pytest.mark.parametrize("fp64", [False, True])
def test_diagnostics_match_numpy(fp64, mhd, cuda):
    shape = (24, 16, 16)
    u, b = mhd.init_vortex(*shape, seed=5)
    if fp64:
        u, b = u.astype(np.float64), b.astype(np.float64)
    with mhd.Context(*shape, fp64=fp64) as ctx:
        ctx.set_state(u, b)
        ctx.step(2)
        su, sb = ctx.get_state()
        d = ctx.diagnostics()
    ref = numpy_diagnostics(su, sb, shape)
    for key, val in ref.items():
        assert d[key] == pytest.approx(val, rel=1e-12, abs=1e-14), key


def test_run_driver_log_checkpoint_and_resume(mhd, cuda, tmp_path):
    from heterogeneous_mhd_gb300 import run
    log, chk = tmp_path / "run.jsonl", tmp_path / "run.chk"
    cfg = run.parse(["--n", "32", "--ic", "turbulence", "--seed", "2", "--steps", "6", "--every", "2",
                     "--log", str(log), "--checkpoint", str(chk), "--checkpoint-every", "4"])
    recs = run.run(cfg)
    lines = [__import__("json").loads(x) for x in log.read_text().splitlines()]
    assert [r["step"] for r in lines] == [0, 2, 4, 6] and lines == recs
    assert all(r["status"] == 0 for r in lines)
    m0 = lines[0]["mass"]
    assert all(abs(r["mass"] - m0) <= 1e-5 * m0 for r in lines)
    assert all(r["max_divb"] < 1e-4 for r in lines) and all(r["min_p"] > 0 for r in lines)
    # the final checkpoint (step 6) resumed for 2 steps equals 8 uninterrupted steps
    more = run.run(run.parse(["--resume", str(chk), "--steps", "2", "--every", "2",
                              "--log", str(tmp_path / "more.jsonl")]))
    straight = run.run(run.parse(["--n", "32", "--ic", "turbulence", "--seed", "2", "--steps", "8", "--every", "8",
                                  "--log", str(tmp_path / "straight.jsonl")]))
    assert more[-1]["step"] == straight[-1]["step"] == 8
    for key in ("t", "dt", "min_rho", "min_p", "max_divb", "mass", "kinetic", "magnetic", "energy", "max_speed"):
        assert more[-1][key] == straight[-1][key], key


def test_standalone_calcfl_between_steps_changes_nothing(mhd, cuda):
    """mhd_op_calcfl on other (and larger) arrays between two steps of a
    context keeps its own scratch: the steps after it are bit for bit those of
    an uninterrupted run, with graphs and with direct launches."""
    torch = cuda
    n = 32
    u0, b0 = mhd.init_turbulence(n, seed=6)
    ub, bb = mhd.init_vortex(96, 96, 96, seed=7, vscale=3.0)
    du, db = torch.from_numpy(ub).cuda(), torch.from_numpy(bb).cuda()
    for graphs in (True, False):
        with mhd.Context(n, n, n) as ref:
            ref.use_graphs(graphs)
            ref.set_state(u0, b0)
            ref.step(3)
            ru, rb = ref.get_state()
            rt = ref.time()
        with mhd.Context(n, n, n) as ctx:
            ctx.use_graphs(graphs)
            ctx.set_state(u0, b0)
            ctx.step(1)
            inv = ctx.op_calcfl(du, db, 96, 96, 96)
            assert np.isfinite(inv) and inv > 0
            ctx.step(1)
            ctx.op_calcfl(du, db, 96, 96, 96)
            ctx.step(1)
            u, b = ctx.get_state()
            t = ctx.time()
            assert ctx.check() == mhd.MHD_OK
        assert bitwise_equal(u, ru) and bitwise_equal(b, rb), graphs
        assert t == rt
