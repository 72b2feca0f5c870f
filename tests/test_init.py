"""Seeded initial conditions (the reference's init reads files that do not
ship, C/init.c:28-52): determinism, div B, amplitudes."""
import numpy as np

from util import checksums, sha


def test_vortex_is_deterministic_and_pinned(mhd):
    u, b = mhd.init_vortex(64, 64, 64, seed=0)
    assert sha(u, b) == checksums()["f32"]["init"]
    u2, b2 = mhd.init_vortex(64, 64, 64, seed=0)
    assert sha(u2, b2) == sha(u, b)
    u3, _ = mhd.init_vortex(64, 64, 64, seed=1)
    assert sha(u3) != sha(u)


def test_vortex_fields(mhd):
    n = 32
    u, b = mhd.init_vortex(n, n, n, seed=0, noise=0.0)
    U = u.reshape(n, n, n, 5)  # [k][j][i][c]
    assert np.allclose(U[..., 0], 1.0)
    x = (np.arange(n) + 0.5) / n
    assert np.allclose(U[0, :, 0, 1], -np.sin(2 * np.pi * x), atol=1e-6)  # vx(y)
    assert np.allclose(U[0, 0, :, 2], np.sin(2 * np.pi * x), atol=1e-6)   # vy(x)
    assert mhd.host_divb_max(b, n, n, n) == 0.0
    # pressure p = (gamma-1)(E - rho v^2/2 - Bc^2/2) = 0.6
    B = b.reshape(n, n, n, 3).astype(np.float64)
    bc = np.stack([(B[..., 0] + np.roll(B[..., 0], -1, 2)) / 2, (B[..., 1] + np.roll(B[..., 1], -1, 1)) / 2,
                   (B[..., 2] + np.roll(B[..., 2], -1, 0)) / 2], -1)
    Ud = U.astype(np.float64)
    p = (2 / 3) * (Ud[..., 4] - (Ud[..., 1:4] ** 2).sum(-1) / (2 * Ud[..., 0]) - (bc ** 2).sum(-1) / 2)
    assert np.allclose(p, 0.6, atol=1e-5)


def test_vortex_noise_level(mhd):
    n = 32
    u0, _ = mhd.init_vortex(n, n, n, seed=4, noise=0.0)
    u1, _ = mhd.init_vortex(n, n, n, seed=4, noise=1e-3)
    d = (u1.reshape(-1, 5)[:, 1:4].astype(np.float64) - u0.reshape(-1, 5)[:, 1:4])
    assert abs(d.std() - 1e-3) < 5e-5 and abs(d.mean()) < 5e-5


def test_turbulence_amplitudes_and_divb(mhd):
    n = 32
    u, b = mhd.init_turbulence(n, seed=3, mach=0.5, bx0=0.3, dbrms=0.1, fp64=True)
    U = u.reshape(-1, 5)
    v2 = (U[:, 1:4] ** 2).sum(1) / U[:, 0] ** 2
    cs = np.sqrt(5 / 3 * 1.0 / 1.0)
    assert abs(np.sqrt(v2.mean()) / cs - 0.5) < 1e-9
    B = b.reshape(-1, 3)
    assert abs(B[:, 0].mean() - 0.3) < 1e-12
    db = B.copy()
    db[:, 0] -= 0.3
    assert abs(np.sqrt((db ** 2).sum(1).mean()) - 0.1) < 1e-9
    assert mhd.host_divb_max(b, n, n, n) < 1e-13
    uf, bf = mhd.init_turbulence(n, seed=3)
    assert mhd.host_divb_max(bf, n, n, n) < 1e-6


def test_turbulence_spectrum_band(mhd):
    n = 32
    u, _ = mhd.init_turbulence(n, seed=9, fp64=True)
    v = u.reshape(n, n, n, 5)[..., 1]
    f = np.fft.fftn(v)
    k = np.fft.fftfreq(n, 1.0 / n)
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    p = np.abs(f) ** 2
    inside = (kk >= 2 - 1e-9) & (kk <= 8 + 1e-9)
    assert p[~inside].sum() < 1e-20 * p.sum() + 1e-20
