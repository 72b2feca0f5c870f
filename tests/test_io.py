"""File formats (CPU): the reference's check_value text dump and init reader,
and the binary checkpoint."""
import numpy as np
import pytest


def test_check_value_dump_format(mhd, tmp_path):
    nx, ny, nz = 3, 2, 4
    u, b = mhd.init_vortex(nx, ny, nz, seed=1)
    mhd.write_check_value(u, b, nx, ny, nz, tmp_path)
    U, B = u.reshape(-1, 5), b.reshape(-1, 3)
    for q in range(5):
        lines = (tmp_path / f"C_version_check_u{q + 1}.dat").read_text().splitlines()
        assert len(lines) == nx * ny * nz
        # C/check_value.c:63-64: "%8.6e" of each value, cells i fastest then j then k
        assert lines == ["%8.6e" % float(x) for x in U[:, q]]
    for q in range(3):
        vals = np.loadtxt(tmp_path / f"C_version_check_b{q + 1}.dat")
        assert np.allclose(vals, B[:, q], rtol=1e-6, atol=1e-12)


def test_read_init_order(mhd, tmp_path):
    nx, ny, nz = 4, 3, 2
    rng = np.random.default_rng(0)
    U = rng.normal(size=(nz, ny, nx, 5)).astype(np.float32)   # [k, j, i, comp]
    B = rng.normal(size=(nz, ny, nx, 3)).astype(np.float32)
    rows = []
    for i in range(nx):            # C/init.c:34-52: i outer, j, k inner
        for j in range(ny):
            for k in range(nz):
                rows.extend("%.9g" % v for v in list(U[k, j, i]) + list(B[k, j, i]))
    p = tmp_path / "source_init.dat"
    p.write_text("\n".join(rows) + "\n")
    u, b = mhd.read_init(p, nx, ny, nz)
    assert np.array_equal(u, U.reshape(-1)) and np.array_equal(b, B.reshape(-1))
    p.write_text("\n".join(rows[:-1]) + "\n")  # one value short
    with pytest.raises(mhd.MhdError):
        mhd.read_init(p, nx, ny, nz)


@pytest.mark.parametrize("fp64", [False, True])
def test_checkpoint_roundtrip_and_integrity(mhd, tmp_path, fp64):
    u, b = mhd.init_vortex(8, 4, 4, seed=2, fp64=fp64)
    p = tmp_path / "state.ckpt"
    mhd.checkpoint_save(p, u, b, 8, 4, 4, t=1.25, step=17)
    u2, b2, shape, t, step = mhd.checkpoint_load(p)
    assert shape == (8, 4, 4) and t == 1.25 and step == 17
    assert u2.dtype == u.dtype and np.array_equal(u2, u) and np.array_equal(b2, b)
    raw = bytearray(p.read_bytes())
    raw[100] ^= 1  # flip one payload bit
    p.write_bytes(bytes(raw))
    with pytest.raises(mhd.MhdError):
        mhd.checkpoint_load(p)
