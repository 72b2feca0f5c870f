"""Autotuner for the launch shapes of the register-resident kernels.

The planners in the library pick pencil tiles by rule (threads per CTA of
fluidx, cells per thread / ring depth / pencils per CTA / planes per CTA of
the marching advectbyzx).  This module times the candidates on the actual
device and grid through the library itself (per-launch CUDA events of
`mhd_profile`), keeps the fastest value of each knob and sets it with
`mhd_tune_set`.  Results are cached per (device name, grid) in a JSON file so
a later process applies them without re-timing.

    from heterogeneous_mhd_gb300 import autotune
    best = autotune.tune(256)          # times candidates, applies the best
    autotune.apply(autotune.load(256)) # reuse a cached result
"""
from __future__ import annotations

import json
import os
from pathlib import Path

from . import Context, init_turbulence, lib

CACHE = Path(os.environ.get("MHD_GB300_TUNE_CACHE", Path(__file__).resolve().parent / "lib" / "tuning.json"))
KNOBS = ("fluidx.threads", "advect.cells", "advect.slots", "advect.J", "advect.K", "fluidx.cells", "advect.kernel",
         "advect.xk", "sweep.kernel", "sweep.k", "sweep.slots")


def set_knob(key: str, value: int) -> None:
    if lib().mhd_tune_set(key.encode(), int(value)) != 0:
        raise ValueError(f"bad tuning knob {key}={value}")


def get_knob(key: str) -> int:
    return int(lib().mhd_tune_get(key.encode()))


def apply(cfg: dict) -> None:
    for k in KNOBS:
        set_knob(k, int(cfg.get(k, 0)))


def _divisors(n: int, lo: int, hi: int):
    return [d for d in range(lo, min(n, hi) + 1) if n % d == 0]


def _device_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:  # pragma: no cover - device query only
        return "cuda"


def _time_kernel(ctx: Context, kernel: str, steps: int) -> float:
    """Mean launch time (ms) of one kernel over `steps` profiled Strang steps."""
    ctx.step(1, cfl=0.7)  # warm: compiles nothing, but settles caches and clocks
    ctx.profile(True)
    ctx.profile_reset()
    ctx.step(steps, cfl=0.7)
    ms, n = ctx.profile_read(kernel)
    ctx.profile(False)
    return ms / max(n, 1)


def candidates(n: int):
    """(knob settings) to try for fluidx and for advectbyzx on an n^3 grid."""
    fx = [{"fluidx.threads": t, "fluidx.cells": 4} for t in (64, 128, 256)]
    if n % 8 == 0 and 8 <= n // 8 <= 64 and (n // 8) & (n // 8 - 1) == 0:
        fx += [{"fluidx.threads": t, "fluidx.cells": 8} for t in (32, 64, 128, 256) if t >= n // 8]
    adv = []
    if n in (64, 128, 256):  # the warp-per-pencil kernel
        for j in (2, 4):
            for k in (4, 8, 16, 32):
                if n % j == 0 and n % k == 0:
                    adv.append({"advect.kernel": 6, "advect.J": j, "advect.K": k})
    if n % 4 == 0 and n % 32 == 0:  # the x-walking kernel
        for xk in (2, 4, 8):
            for slots in (2, 3):
                if n % xk == 0:
                    adv.append({"advect.kernel": 4, "advect.xk": xk, "advect.slots": slots})
    for cells in (4, 8):
        t = n // cells
        if n % cells or t < 4 or t > 128 or (t & (t - 1)):
            continue
        for slots in (2, 3):
            for j in _divisors(n, 1, 8):
                if (2 * j + 1) * t > 384:
                    continue
                for k in (4, 8, 16, 32):
                    if n % k == 0:
                        adv.append({"advect.kernel": 3, "advect.cells": cells, "advect.slots": slots,
                                    "advect.J": j, "advect.K": k})
    return fx, adv


def tune(n: int = 256, steps: int = 3, verbose: bool = False, save: bool = True) -> dict:
    """Time the candidates on an n^3 turbulence box and apply the fastest."""
    u, b = init_turbulence(n, seed=0)
    fx, adv = candidates(n)
    results = {"fluidx": [], "advectbyzx": []}
    with Context(n, n, n) as ctx:
        ctx.set_state(u, b)
        apply({})
        for cfg in fx:
            apply(cfg)
            t = _time_kernel(ctx, "fluidx", steps)
            results["fluidx"].append((t, cfg))
            if verbose:
                print(f"fluidx {cfg} {t * 1e3:.1f} us", flush=True)
        best_fx = min(results["fluidx"], key=lambda r: r[0])[1]
        for cfg in adv:
            apply({**best_fx, **cfg})
            t = _time_kernel(ctx, "advectbyzx", steps)
            results["advectbyzx"].append((t, cfg))
            if verbose:
                print(f"advect {cfg} {t * 1e3:.1f} us", flush=True)
        best_adv = min(results["advectbyzx"], key=lambda r: r[0])[1]
    best = {**best_fx, **best_adv}
    apply(best)
    if save:
        store = json.loads(CACHE.read_text()) if CACHE.exists() else {}
        store[f"{_device_name()}:{n}"] = {
            "best": best,
            "fluidx_ms": min(r[0] for r in results["fluidx"]),
            "advect_ms": min(r[0] for r in results["advectbyzx"]),
            "tried": len(fx) + len(adv),
        }
        CACHE.parent.mkdir(parents=True, exist_ok=True)
        CACHE.write_text(json.dumps(store, indent=1))
    best["_results"] = {k: [(round(t * 1e3, 2), c) for t, c in sorted(v, key=lambda r: r[0])[:5]]
                        for k, v in results.items()}
    return best


def batch_candidates(n: int):
    """Launch shapes to try for the boxes of edge n of a batch: the fluidx CTA
    width and the marching advectbyzx (the planner's kernel for classes
    without the side array; classes with it, edges 96, 128 and 256, run the
    warp-per-pencil kernel, against which the marching shapes are timed)."""
    out = [{}]
    out += [{"fluidx.threads": t} for t in (128, 256)]
    t = n // 4
    if n % 4 == 0 and 4 <= t <= 128 and not (t & (t - 1)):
        for slots in (2, 3):
            for j in _divisors(n, 1, 8):
                if (2 * j + 1) * t > 384:
                    continue
                for k in (4, 8, 16, 32):
                    if n % k == 0:
                        out.append({"advect.kernel": 3, "advect.slots": slots, "advect.J": j, "advect.K": k})
    return out


def tune_batch(bt, cfg, steps: int = 3, verbose: bool = False, min_gain: float = 0.02) -> dict:
    """Per size class of a batch (`bt`, built from the box table `cfg` of
    batch_config): time every candidate shape on a batch of that class's
    boxes alone (the same count and initial states, one launch per operator),
    and set the fastest on `bt` with Batch.tune_edge when it beats the
    planner's shapes by more than min_gain (a class given its own shapes
    leaves the work-list launches).  Returns {edge: (knobs, ms per step, ms
    with the planner)}."""
    import torch

    from . import Batch, init_batch_box

    edges = sorted({x["n"] for x in cfg})
    keys = ("fluidx.threads", "advect.kernel", "advect.slots", "advect.J", "advect.K")
    chosen = {}
    for edge in edges:
        boxes = [x for x in cfg if x["n"] == edge]
        with Batch([edge] * len(boxes)) as one:
            one.set_worklist(False)  # the planner's own launches are the baseline
            for i, box in enumerate(boxes):
                one.set_box(i, *init_batch_box(box))
            stream = torch.cuda.ExternalStream(one.stream())
            timed = []
            for cand in batch_candidates(edge):
                for k in keys:
                    one.tune_edge(edge, k, int(cand.get(k, 0)) if cand else -1)
                one.step(1)
                one.sync()
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                one.step(steps)
                ev1.record(stream)
                ev1.synchronize()
                ms = ev0.elapsed_time(ev1) / steps
                timed.append((ms, cand))
                if verbose:
                    print(f"batch edge {edge} {cand} {ms:.3f} ms", flush=True)
        base = timed[0][0]
        best_ms, best = min(timed, key=lambda r: r[0])
        if best_ms < base * (1.0 - min_gain):
            for k in keys:
                bt.tune_edge(edge, k, int(best.get(k, 0)))
            chosen[edge] = (best, best_ms, base)
        else:
            chosen[edge] = ({}, base, base)
    return chosen


def load(n: int) -> dict | None:
    if not CACHE.exists():
        return None
    rec = json.loads(CACHE.read_text()).get(f"{_device_name()}:{n}")
    return rec["best"] if rec else None


if __name__ == "__main__":
    import sys

    size = int(sys.argv[1]) if len(sys.argv) > 1 else 256
    print(json.dumps(tune(size, verbose=True), indent=1))
