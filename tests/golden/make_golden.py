"""Generate the golden fixtures from the reference's own C/ sources.

Run in the development container, with MHD_REF_SRC naming the reference's
C/ directory:

    MHD_REF_SRC=/root/reference/C python tests/golden/make_golden.py

It builds oracle/_ref (the reference's C/ files compiled in place by
oracle/Makefile), runs them on seeded inputs and writes

  * ops_f32.npz / ops_f64.npz - per-operator inputs and outputs on small
    grids, including non-cubic and odd shapes;
  * steps_f32.npz / steps_f64.npz - whole Strang steps (C/mhd.c:59-124) on
    small grids: the output arrays, and the SHA-256 of the seed-7 vortex
    initial state they start from (regenerated by the tests);
  * checksums.json - SHA-256 of the state after 1, 10 and 100 Strang steps of
    the 64^3 vortex configuration (CFL 0.7), and of its initial state, so runs
    at full size are checked without storing the arrays.

Inputs come from the library's deterministic initial conditions
(mhd_init_vortex, identical bits on x86-64 and aarch64) perturbed by a seeded
numpy generator; the perturbed inputs are stored in the fixtures.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import heterogeneous_mhd_gb300 as mhd  # noqa: E402
from _oracle import Oracle  # noqa: E402

OP_SHAPES = [(8, 8, 8), (12, 8, 6), (6, 10, 4), (10, 6, 10), (1, 4, 3), (32, 4, 2)]
STEP_SHAPES = [((16, 16, 16), 3), ((12, 8, 8), 2)]
DT = 0.05


def sha(*arrs) -> str:
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def perturbed_state(nx, ny, nz, seed, fp64):
    u, b = mhd.init_vortex(nx, ny, nz, seed=seed, fp64=fp64)
    rng = np.random.default_rng(1000 + seed)
    dt = u.dtype
    u = (u.astype(np.float64) * (1.0 + 0.02 * rng.standard_normal(u.shape))).astype(dt)
    b = (b.astype(np.float64) + 0.02 * rng.standard_normal(b.shape)).astype(dt)
    return u, b


def op_fixture(o: Oracle, fp64: bool) -> dict:
    out = {}
    for s, (nx, ny, nz) in enumerate(OP_SHAPES):
        key = f"{nx}x{ny}x{nz}"
        u, b = perturbed_state(nx, ny, nz, s, fp64)
        out[f"{key}/u"] = u
        out[f"{key}/b"] = b
        # fluidx: u <- F(update); the output array starts as garbage (7)
        uo = np.full_like(u, 7)
        o.fluidx(uo, b.copy(), nx, ny, nz, DT, u.copy(), b.copy())
        out[f"{key}/fluidx_u"] = uo
        # advectbyzx: b(1) is read from b in place; give it a distinct value
        b_inplace = (b * np.asarray(1.5, dtype=b.dtype)).astype(b.dtype)
        out[f"{key}/advect_bin"] = b_inplace
        bo = b_inplace.copy()
        o.advectbyzx(u.copy(), bo, nx, ny, nz, DT, u.copy(), b.copy())
        out[f"{key}/advect_b"] = bo
        ut, bt = np.empty_like(u), np.empty_like(b)
        o.transpose12(ut, bt, u.copy(), b.copy(), nx, ny, nz)
        out[f"{key}/t12_u"], out[f"{key}/t12_b"] = ut, bt
        if nx == nz:
            ut, bt = np.empty_like(u), np.empty_like(b)
            o.transpose13(ut, bt, u.copy(), b.copy(), nx, ny, nz)
            out[f"{key}/t13_u"], out[f"{key}/t13_b"] = ut, bt
        out[f"{key}/calcfl"] = np.array([o.calcfl(u, b, nx, ny, nz)], dtype=u.dtype)
    return out


def step_fixture(o: Oracle, fp64: bool) -> dict:
    out = {}
    for (nx, ny, nz), nsteps in STEP_SHAPES:
        key = f"{nx}x{ny}x{nz}"
        u, b = mhd.init_vortex(nx, ny, nz, seed=7, fp64=fp64)
        uo, bo, t, dt, s = o.strang(u, b, nx, ny, nz, nsteps, cfl=0.7)
        out[f"{key}/init_sha256"] = np.array([sha(u, b)])
        out[f"{key}/u"], out[f"{key}/b"] = uo, bo
        out[f"{key}/t"] = np.array([t], dtype=u.dtype)
        out[f"{key}/nsteps"] = np.array([nsteps])
    return out


def checksums(o32: Oracle, o64: Oracle) -> dict:
    res = {"config": "vortex 64^3 seed 0, rho=1 p=0.6 noise 1e-3, CFL 0.7", "f32": {}, "f64": {}}
    for bits, o, steps in ((32, o32, (1, 10, 100)), (64, o64, (1, 10))):
        n = 64
        u, b = mhd.init_vortex(n, n, n, seed=0, fp64=(bits == 64))
        rec = {"init": sha(u, b)}
        done = 0
        t = 0.0
        for target in steps:
            u, b, t, dt, s = o.strang(u, b, n, n, n, target - done, cfl=0.7, t=t)
            done = target
            rec[str(target)] = {"sha256": sha(u, b), "t": t, "dt": dt,
                                "sum_u": [float(x) for x in u.reshape(-1, 5).astype(np.float64).sum(0)],
                                "sum_b": [float(x) for x in b.reshape(-1, 3).astype(np.float64).sum(0)]}
            print(f"  f{bits} step {target}: t={t:.6f}")
        res[f"f{bits}"] = rec
    return res


def main() -> None:
    mhd.lib(build_if_missing=True)
    o32, o64 = Oracle(32, "ref"), Oracle(64, "ref")
    for bits, o in ((32, o32), (64, o64)):
        np.savez_compressed(HERE / f"ops_f{bits}.npz", **op_fixture(o, bits == 64))
        np.savez_compressed(HERE / f"steps_f{bits}.npz", **step_fixture(o, bits == 64))
    (HERE / "checksums.json").write_text(json.dumps(checksums(o32, o64), indent=1) + "\n")
    for p in sorted(HERE.glob("*")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
