"""Host-side diagnostics of a state: per-field errors and energy spectra.

These read states copied back to the host (numpy); they measure results and
are not on the step's path.  Layout as the reference: u(5,nx,ny,nz) =
(rho, rho vx, rho vy, rho vz, E) and b(3,nx,ny,nz) face-centred, component
index fastest (C/mhd.c:26-41).
"""
from __future__ import annotations

import numpy as np

FIELDS = ("rho", "mx", "my", "mz", "E", "bx", "by", "bz")


def field_errors(u, b, u_ref, b_ref) -> dict:
    """Relative L2 error of each of the eight fields against a reference state.

    rho and E are normalised by their own norm; each momentum component by the
    norm of the whole momentum field and each B component by that of the whole
    B field, so a component that is zero in the reference (bz of the vortex
    box) is measured against the field's magnitude rather than against zero.
    """
    U = np.asarray(u, dtype=np.float64).reshape(-1, 5)
    Ur = np.asarray(u_ref, dtype=np.float64).reshape(-1, 5)
    B = np.asarray(b, dtype=np.float64).reshape(-1, 3)
    Br = np.asarray(b_ref, dtype=np.float64).reshape(-1, 3)
    mom = np.linalg.norm(Ur[:, 1:4])
    mag = np.linalg.norm(Br)
    out = {}
    for c in range(5):
        d = np.linalg.norm(U[:, c] - Ur[:, c])
        nrm = mom if c in (1, 2, 3) else np.linalg.norm(Ur[:, c])
        out[FIELDS[c]] = float(d / nrm) if nrm > 0 else float(d)
    for c in range(3):
        d = np.linalg.norm(B[:, c] - Br[:, c])
        out[FIELDS[5 + c]] = float(d / mag) if mag > 0 else float(d)
    return out


def cell_centred_b(b, n: int) -> np.ndarray:
    """(n,n,n,3) cell-centred B, each component the mean of its two faces (C/fluidx.c:71-81)."""
    B = np.asarray(b, dtype=np.float64).reshape(n, n, n, 3)  # [k, j, i, c]
    return 0.5 * (B + np.stack([np.roll(B[..., c], -1, axis=2 - c) for c in range(3)], axis=-1))


def shell_spectrum(f: np.ndarray) -> np.ndarray:
    """Shell-summed power spectrum E(k), k = 0..n/2, of a (n,n,n,m) vector field (sum over m)."""
    n = f.shape[0]
    F = np.fft.fftn(f, axes=(0, 1, 2)) / n ** 3
    P = (np.abs(F) ** 2).sum(axis=-1)
    k = np.fft.fftfreq(n, d=1.0 / n)
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    shell = np.rint(kk).astype(np.int64)
    spec = np.bincount(shell.ravel(), weights=P.ravel(), minlength=n // 2 + 1)
    return 0.5 * spec[: n // 2 + 1]


def energy_spectra(u, b, n: int) -> dict:
    """Kinetic (of sqrt(rho) v) and magnetic shell spectra of a cubic state."""
    U = np.asarray(u, dtype=np.float64).reshape(n, n, n, 5)
    w = U[..., 1:4] / np.sqrt(U[..., :1])
    return {"kinetic": shell_spectrum(w), "magnetic": shell_spectrum(cell_centred_b(b, n))}


def spectrum_error(s, s_ref, kmax: int | None = None) -> float:
    """Relative L2 distance of two spectra over shells 1..kmax."""
    s = np.asarray(s, dtype=np.float64)
    s_ref = np.asarray(s_ref, dtype=np.float64)
    kmax = kmax or (len(s_ref) - 1)
    a, r = s[1: kmax + 1], s_ref[1: kmax + 1]
    return float(np.linalg.norm(a - r) / np.linalg.norm(r))
