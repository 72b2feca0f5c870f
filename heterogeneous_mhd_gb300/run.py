"""Run driver: the time loop of the reference's main program (C/mhd.c:55-126)
on the GPU library, with JSON-lines diagnostics and checkpoints.

    python -m heterogeneous_mhd_gb300.run --n 64 --ic vortex --steps 100 \\
        --log run.jsonl --every 10 --checkpoint run.chk --checkpoint-every 50
    python -m heterogeneous_mhd_gb300.run --config run.json   # keys as the flags
    python -m heterogeneous_mhd_gb300.run --resume run.chk --steps 100

Every `every` steps (and at the start) one JSON line: step, t, dt, the
device diagnostics (min rho, min p, max |div B|, mass, kinetic, magnetic and
total energy, max speed), the mean wall time per step of the interval and
the context status.  The reference prints t, the iteration and two sample
values per step (C/mhd.c:66) and has no checkpoints.  The run stops after
`steps` steps, at t >= tf, or at the first device error (reported in the
last line).
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from pathlib import Path

DEFAULTS = {
    "n": 64,              # cube edge (nx = ny = nz unless given)
    "nx": 0, "ny": 0, "nz": 0,
    "ic": "vortex",       # vortex (64^3 Orszag-Tang-like vortex) or turbulence (decaying turbulence)
    "seed": 0,
    "steps": 100,
    "cfl": 0.7,
    "tf": math.inf,
    "log": None,          # JSON-lines file (stdout when None)
    "every": 10,
    "checkpoint": None,   # checkpoint file, rewritten every checkpoint_every steps and at the end
    "checkpoint_every": 0,
    "resume": None,       # start from this checkpoint instead of an initial condition
    "exact": False,
    "fp64": False,
    "fused": False,
}


def parse(argv=None) -> dict:
    """Defaults, then the --config JSON file, then the command-line flags."""
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--config", help="JSON file with any of the keys below")
    for key, val in DEFAULTS.items():
        flag = "--" + key.replace("_", "-")
        if isinstance(val, bool):
            ap.add_argument(flag, action="store_const", const=True, default=None)
        elif val is None:
            ap.add_argument(flag, default=None)
        else:
            ap.add_argument(flag, type=type(val), default=None)
    args = ap.parse_args(argv)
    cfg = dict(DEFAULTS)
    if args.config:
        extra = json.loads(Path(args.config).read_text())
        unknown = set(extra) - set(DEFAULTS)
        if unknown:
            raise SystemExit(f"unknown config keys: {sorted(unknown)}")
        cfg.update(extra)
    for key in DEFAULTS:
        v = getattr(args, key)
        if v is not None:
            cfg[key] = v
    if cfg["ic"] not in ("vortex", "turbulence"):
        raise SystemExit("ic must be vortex or turbulence")
    return cfg


def _reached(t: float, tf: float) -> bool:
    # the device clock is FP32 in an FP32 context: compare with a relative margin
    return math.isfinite(tf) and t >= tf * (1.0 - 1e-6)


def run(cfg: dict) -> list[dict]:
    """Advance as configured; returns the records written to the log."""
    import heterogeneous_mhd_gb300 as mhd

    step0, t0 = 0, 0.0
    if cfg["resume"]:
        u, b, shape, t0, step0 = mhd.checkpoint_load(cfg["resume"])
    else:
        shape = tuple(cfg[k] or cfg["n"] for k in ("nx", "ny", "nz"))
        if cfg["ic"] == "vortex":
            u, b = mhd.init_vortex(*shape, seed=int(cfg["seed"]))
        else:
            if len(set(shape)) != 1:
                raise SystemExit("the turbulence initial condition is a cube")
            u, b = mhd.init_turbulence(shape[0], seed=int(cfg["seed"]))
    out = open(cfg["log"], "w") if cfg["log"] else sys.stdout
    records = []

    def emit(rec):
        records.append(rec)
        out.write(json.dumps(rec) + "\n")
        out.flush()

    try:
        with mhd.Context(*shape, fp64=bool(cfg["fp64"]), exact=bool(cfg["exact"])) as ctx:
            ctx.set_state(u, b)
            ctx.set_time(t0, float(cfg["tf"]))

            def save(step, t):
                if cfg["checkpoint"]:
                    cu, cb = ctx.get_state()
                    mhd.checkpoint_save(cfg["checkpoint"], cu, cb, *shape, t=t, step=step)

            step, last_ckpt = step0, step0
            emit({"step": step, "t": t0, "dt": None, **ctx.diagnostics(), "ms_per_step": None, "status": 0})
            end = step0 + int(cfg["steps"])
            while step < end:
                k = min(int(cfg["every"]), end - step)
                w0 = time.perf_counter()
                ctx.step(k, cfl=float(cfg["cfl"]), fused=bool(cfg["fused"]))
                status = ctx.check()  # synchronises
                wall = (time.perf_counter() - w0) * 1e3 / k
                step += k
                t, dt, _ = ctx.time()
                emit({"step": step, "t": t, "dt": dt, **ctx.diagnostics(), "ms_per_step": wall,
                      "status": status})
                if status != mhd.MHD_OK:
                    break
                if cfg["checkpoint_every"] and step - last_ckpt >= int(cfg["checkpoint_every"]):
                    save(step, t)
                    last_ckpt = step
                if _reached(t, float(cfg["tf"])):
                    break
            if records[-1]["status"] == mhd.MHD_OK:
                save(step, records[-1]["t"])
    finally:
        if out is not sys.stdout:
            out.close()
    return records


def main(argv=None) -> int:
    recs = run(parse(argv))
    return 0 if recs and recs[-1]["status"] == 0 else 1


if __name__ == "__main__":
    raise SystemExit(main())
