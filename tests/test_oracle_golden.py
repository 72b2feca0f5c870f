"""The CPU oracle restatement (oracle/mhd_oracle.c) against the golden
fixtures produced by the reference's own C/ sources (tests/golden/make_golden.py).
Bit-for-bit: the oracle follows the reference's operations, order and float/
double promotions, and both are built with -ffp-contract=off."""
import numpy as np
import pytest

from util import bitwise_equal, checksums, load_npz, sha, shapes_in

DT = 0.05


@pytest.mark.parametrize("bits", [32, 64])
def test_ops_match_reference(bits, oracle32, oracle64):
    o = oracle32 if bits == 32 else oracle64
    fix = load_npz(f"ops_f{bits}.npz")
    for nx, ny, nz in shapes_in(fix):
        key = f"{nx}x{ny}x{nz}"
        u, b = fix[f"{key}/u"], fix[f"{key}/b"]
        uo = np.full_like(u, 7)
        o.fluidx(uo, b.copy(), nx, ny, nz, DT, u.copy(), b.copy())
        assert bitwise_equal(uo, fix[f"{key}/fluidx_u"]), f"fluidx {key}"
        bo = fix[f"{key}/advect_bin"].copy()
        o.advectbyzx(u.copy(), bo, nx, ny, nz, DT, u.copy(), b.copy())
        assert bitwise_equal(bo, fix[f"{key}/advect_b"]), f"advectbyzx {key}"
        ut, bt = np.empty_like(u), np.empty_like(b)
        o.transpose12(ut, bt, u.copy(), b.copy(), nx, ny, nz)
        assert bitwise_equal(ut, fix[f"{key}/t12_u"]) and bitwise_equal(bt, fix[f"{key}/t12_b"]), f"t12 {key}"
        if nx == nz:
            ut, bt = np.empty_like(u), np.empty_like(b)
            o.transpose13(ut, bt, u.copy(), b.copy(), nx, ny, nz)
            assert bitwise_equal(ut, fix[f"{key}/t13_u"]) and bitwise_equal(bt, fix[f"{key}/t13_b"]), f"t13 {key}"
        assert bitwise_equal(np.array([o.calcfl(u, b, nx, ny, nz)], dtype=u.dtype), fix[f"{key}/calcfl"])


def test_transpose13_rejects_non_square(oracle32):
    """C/transpose13.c:50-61: nx != nz leaves the outputs untouched."""
    u = np.arange(5 * 4 * 3 * 2, dtype=np.float32)
    b = np.arange(3 * 4 * 3 * 2, dtype=np.float32)
    uo, bo = np.full_like(u, -1), np.full_like(b, -1)
    oracle32.transpose13(uo, bo, u, b, 4, 3, 2)
    assert (uo == -1).all() and (bo == -1).all()


@pytest.mark.parametrize("bits", [32, 64])
def test_strang_steps_match_reference(bits, mhd, oracle32, oracle64):
    o = oracle32 if bits == 32 else oracle64
    fix = load_npz(f"steps_f{bits}.npz")
    for nx, ny, nz in shapes_in(fix):
        key = f"{nx}x{ny}x{nz}"
        u0, b0 = mhd.init_vortex(nx, ny, nz, seed=7, fp64=(bits == 64))
        assert sha(u0, b0) == str(fix[f"{key}/init_sha256"][0]), "initial condition changed"
        u, b, t, dt, s = o.strang(u0, b0, nx, ny, nz, int(fix[f"{key}/nsteps"][0]), cfl=0.7)
        assert bitwise_equal(u, fix[f"{key}/u"]) and bitwise_equal(b, fix[f"{key}/b"]), key
        assert np.array(t, dtype=u.dtype) == fix[f"{key}/t"][0]


def test_vortex_64_checksums(mhd, oracle32):
    """64^3, CFL 0.7, 10 Strang steps: the reference's state hash."""
    ck = checksums()["f32"]
    u, b = mhd.init_vortex(64, 64, 64, seed=0)
    assert sha(u, b) == ck["init"]
    t = 0.0
    u, b, t, dt, s = oracle32.strang(u, b, 64, 64, 64, 1, cfl=0.7, t=t)
    assert sha(u, b) == ck["1"]["sha256"]
    u, b, t, dt, s = oracle32.strang(u, b, 64, 64, 64, 9, cfl=0.7, t=t)
    assert sha(u, b) == ck["10"]["sha256"]
    assert abs(t - ck["10"]["t"]) == 0.0


def test_port_matches_reference_build_random_shapes(mhd, oracle32):
    """Cross-check against oracle/_ref on fresh shapes (development container only)."""
    from _oracle import REF, Oracle
    import os
    from _oracle import have_ref
    if not have_ref():
        pytest.skip("no reference build and no MHD_REF_SRC on this machine")
    ref = Oracle(32, "ref")
    rng = np.random.default_rng(5)
    for _ in range(6):
        nx, ny, nz = (int(x) for x in rng.integers(1, 14, size=3))
        u, b = mhd.init_vortex(nx, ny, nz, seed=int(rng.integers(1 << 30)))
        for o_name in ("fluidx", "advectbyzx"):
            outs = []
            for o in (oracle32, ref):
                uo, bo = np.full_like(u, 3), (b * np.float32(0.5)).astype(np.float32)
                getattr(o, o_name)(uo, bo, nx, ny, nz, 0.1, u.copy(), b.copy())
                outs.append((uo, bo))
            assert bitwise_equal(outs[0][0], outs[1][0]) and bitwise_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("bits", [32, 64])
def test_calcfl_nan_and_inf_cells_match_reference_build(bits, mhd, oracle32, oracle64):
    """calcfl's handling of non-finite speeds, pinned to the reference build
    itself: max_2num (C/calcfl.c:91-101) restarts the running maximum after a
    NaN, so a NaN in a middle cell is skipped, a NaN in the last cell makes
    1/c NaN, and an infinite speed gives 1/c = 0.  The GPU kernels' NaN tests
    check against this oracle (development container only)."""
    from _oracle import Oracle, have_ref
    if not have_ref():
        pytest.skip("no reference build and no MHD_REF_SRC on this machine")
    port = oracle32 if bits == 32 else oracle64
    ref = Oracle(bits, "ref")
    dt = np.float32 if bits == 32 else np.float64
    nx, ny, nz = 12, 6, 5
    nc = nx * ny * nz
    u0, b0 = mhd.init_vortex(nx, ny, nz, seed=41, fp64=(bits == 64))
    cases = {"middle": [(nc // 2 + 3, 0)], "last": [(nc - 1, 0)], "first": [(0, 0)],
             "two": [(17, 0), (nc - 40, 4)], "b only": [(nc // 3, "b")], "inf": [(nc // 4, "inf")]}
    for name, cells in cases.items():
        u, b = u0.astype(dt).copy(), b0.astype(dt).copy()
        for cell, comp in cells:
            if comp == "b":
                b[cell * 3 + 1] = np.nan
            elif comp == "inf":
                u[cell * 5 + 1] = np.inf
            else:
                u[cell * 5 + comp] = np.nan
        got, want = port.calcfl(u, b, nx, ny, nz), ref.calcfl(u, b, nx, ny, nz)
        assert (np.isnan(got) and np.isnan(want)) or got == want, (name, got, want)
        if name == "last":
            assert np.isnan(want)
        if name in ("middle", "first", "two", "b only"):
            assert np.isfinite(want) and want > 0, (name, want)
        if name == "inf":
            assert want == 0, want


@pytest.mark.parametrize("bits", [32, 64])
def test_port_matches_reference_build_every_operator(bits, mhd, oracle32, oracle64):
    """Every operator of the path (fluidx, advectbyzx, transpose12,
    transpose13 where nx == nz, copy_matrix, calcfl) of the restatement
    against oracle/_ref on fresh odd shapes, in both precisions, bit for bit
    (development container only)."""
    from _oracle import Oracle, have_ref
    if not have_ref():
        pytest.skip("no reference build and no MHD_REF_SRC on this machine")
    port = oracle32 if bits == 32 else oracle64
    ref = Oracle(bits, "ref")
    dt = np.float32 if bits == 32 else np.float64
    rng = np.random.default_rng(11 + bits)
    shapes = [tuple(int(x) for x in rng.integers(1, 13, size=3)) for _ in range(5)] + [(9, 4, 9), (7, 7, 7)]
    for nx, ny, nz in shapes:
        u, b = mhd.init_vortex(nx, ny, nz, seed=int(rng.integers(1 << 30)), fp64=(bits == 64))
        u, b = u.astype(dt), b.astype(dt)
        outs = []
        for o in (port, ref):
            res = {}
            uo, bo = np.full_like(u, 3), (b * dt(0.5)).astype(dt)
            o.fluidx(uo, bo, nx, ny, nz, 0.05, u.copy(), b.copy())
            res["fluidx"] = (uo, bo)
            uo, bo = u.copy(), (b * dt(0.75)).astype(dt)
            o.advectbyzx(uo, bo, nx, ny, nz, 0.05, u.copy(), b.copy())
            res["advectbyzx"] = (uo, bo)
            ut, bt = np.zeros_like(u), np.zeros_like(b)
            o.transpose12(ut, bt, u.copy(), b.copy(), nx, ny, nz)
            res["transpose12"] = (ut, bt)
            if nx == nz:
                ut, bt = np.zeros_like(u), np.zeros_like(b)
                o.transpose13(ut, bt, u.copy(), b.copy(), nx, ny, nz)
                res["transpose13"] = (ut, bt)
            uc, bc = np.zeros_like(u), np.zeros_like(b)
            o.copy_matrix(u.copy(), b.copy(), nx, ny, nz, uc, bc)
            res["copy_matrix"] = (uc, bc)
            res["calcfl"] = (np.array([o.calcfl(u, b, nx, ny, nz)], dtype=dt),)
            outs.append(res)
        for name in outs[0]:
            for got, want in zip(outs[0][name], outs[1][name]):
                assert bitwise_equal(got, want), (name, (nx, ny, nz), bits)
