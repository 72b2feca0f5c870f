"""Shared helpers for the tests."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def sha(*arrs) -> str:
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def load_npz(name: str) -> dict:
    with np.load(GOLDEN / name) as z:
        return {k: z[k] for k in z.files}


def checksums() -> dict:
    return json.loads((GOLDEN / "checksums.json").read_text())


def shapes_in(fix: dict):
    keys = sorted({k.split("/")[0] for k in fix})
    return [tuple(int(x) for x in k.split("x")) for k in keys]


def bitwise_equal(a, b) -> bool:
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and a.tobytes() == b.tobytes()


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(a - b)
    n = np.linalg.norm(b)
    return float(d / n) if n > 0 else float(d)


def rel_l2_fields(u, b, u_ref, b_ref) -> dict:
    """Relative L2 error of each field u1..u5, b1..b3.

    Scalars (rho, E) are normalised by their own norm; each component of a
    vector field (momentum u2..u4, magnetic field b1..b3) by the norm of the
    whole vector field, so a component that is identically zero in the
    initial state (b3 and most of u4 in the vortex) is measured against the
    field's magnitude instead of against zero."""
    out = {}
    U, Ur = np.asarray(u, dtype=np.float64).reshape(-1, 5), np.asarray(u_ref, dtype=np.float64).reshape(-1, 5)
    B, Br = np.asarray(b, dtype=np.float64).reshape(-1, 3), np.asarray(b_ref, dtype=np.float64).reshape(-1, 3)
    mom = np.linalg.norm(Ur[:, 1:4])
    mag = np.linalg.norm(Br)
    for c in range(5):
        d = np.linalg.norm(U[:, c] - Ur[:, c])
        n = mom if c in (1, 2, 3) else np.linalg.norm(Ur[:, c])
        out[f"u{c + 1}"] = float(d / n) if n > 0 else float(d)
    for c in range(3):
        d = np.linalg.norm(B[:, c] - Br[:, c])
        out[f"b{c + 1}"] = float(d / mag) if mag > 0 else float(d)
    return out
