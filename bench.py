"""Throughput of the relaxing-TVD split MHD step on GB300.

One "step" is one full Strang step x(F,A) T12 y(F,A) T13 z(F,A,A,F) T13 y(A,F)
T12 x(A,F) (C/mhd.c:59-124) of the 256^3 decaying-turbulence box (FP32,
gamma 5/3, CFL 0.7, seeded k^-2 velocity at rms Mach 0.5, B = 0.3 x + dB).
Metric: cell-updates/s = 256^3 * steps / time.  The headline variant is the
fused step (the same twelve operators on the untransposed state, no
transposes; --variant fused, the default); the plain step (the reference's
operator sequence with its four transposes) is timed in the same run and
reported beside it, and --variant plain makes it the headline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--size N] [--variant plain|fused]

Our arm prints one JSON line with:
  value       device throughput, state resident in HBM, timed with CUDA events
              on the library's stream (max over ranks);
  e2e         the same metric through the C ABI with host buffers: every step
              copies the state in from pinned host memory and back out
              (mhd_step_host, which overlaps the copies with the step; the
              three-call path without overlap is reported beside it);
  roofline    the dominant kernel's algorithmic bytes per launch over its mean
              launch time (events around every launch in the timed region),
              against the measured HBM copy bandwidth;
  cpu_baseline  the CPU oracle (the reference's C path) on this host's cores;
  clocks      nvidia-smi samples taken during the timed region.
The state (537 MB at 256^3) is larger than L2 (126 MB), so no L2 flush is
needed between steps.  With --gpus N > 1 (torchrun) every rank advances its
own box: replicas with no collective ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# Algorithmic HBM bytes per cell of one launch of each kernel, FP32 AoS (u 20
# B, b 12 B per cell), in the fixed convention of the reference's operators:
# fluidx reads u and b and writes u (52), advectbyzx reads u and b and writes
# b (44), a transpose reads and writes the state (64), calcfl reads it (32).
ALG_BYTES = {"fluidx": 52, "advectbyzx": 44, "transpose12": 64, "transpose13": 64, "calcfl": 32, "copy": 64,
             "cfl_finalize": 0, "sweep": 64}
# What the kernels move on average per launch.  Plain step: the three forward
# fluidx launches and the two backward transposes also write the (rho, m_x)
# side array (8 B), and every advectbyzx reads it in place of u (8 B, not 20).
# Fused step: every fluidx but the last writes (rho, m_d) for the advectbyzx
# after it (m_d the momentum along that sweep), and every advectbyzx reads it.
MOVED_BYTES = {"plain": {"fluidx": 52 + 8 * 3 / 6, "advectbyzx": 32, "transpose12": 64 + 8 / 2,
                         "transpose13": 64 + 8 / 2},
               "fused": {"fluidx": 52 + 8 * 5 / 6, "advectbyzx": 32}}
# per-cell bytes of a whole step: the reference's operator sequence (6 fluidx
# x 52 + 6 advectbyzx x 44 + 4 transposes x 64 + a calcfl 32 = 864), what the
# fused step's operators move (no transposes: 6 x 52 + 6 x 44 = 576), and the
# five-pass bound of a step that fuses each sweep's operators (5 x 64 = 320)
STEP_BYTES = {"plain": 864, "fused": 576, "fused_5pass": 320}
STEP_MOVED = {"plain": 6 * 52 + 3 * 8 + 6 * 32 + 4 * 64 + 2 * 8, "fused": 6 * 52 + 5 * 8 + 6 * 32}
METRIC = "cell-updates/s at 256^3 (plain vs fused); closure speedup at matched error"
E2E_TRIALS = 5


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        t0 = time.perf_counter()  # nvidia-smi takes a moment to start: wait for its first sample
        while time.perf_counter() - t0 < 5.0 and self.path.stat().st_size == 0 and self.proc.poll() is None:
            time.sleep(0.02)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sms) if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


def measured_traffic(kernel: str, n: int, variant: str = "plain"):
    """DRAM bytes per launch of `kernel` from the committed ncu capture
    (profiles/traffic_256.json) when it was taken on this grid, else None."""
    p = ROOT / "profiles" / "traffic_256.json"
    try:
        t = json.loads(p.read_text())
    except (OSError, ValueError):
        return None
    t = t.get(variant, {})
    if t.get("grid") != [n, n, n] or kernel not in t:
        return None
    return t[kernel]["dram_bytes_per_launch"]


def cpu_baseline(size: int, seconds: float = 12.0):
    """The oracle (the reference's C arithmetic) on this host's cores."""
    sys.path.insert(0, str(ROOT / "tests"))
    from _oracle import Oracle  # the checker, timed as the CPU baseline

    port = Oracle(32, "port")
    u, b = port.init_turbulence(size, seed=0)
    cores = port.max_threads()
    t0 = time.perf_counter()
    steps = 0
    while True:
        u, b, _, _, _ = port.strang(u, b, size, size, size, 1)
        steps += 1
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    # one core, as the reference's C path runs when built as shipped (64^3, a few seconds)
    port.set_threads(1)
    u1, b1 = port.init_vortex(64, 64, 64, seed=0)
    t1, steps1 = time.perf_counter(), 0
    while True:
        u1, b1, _, _, _ = port.strang(u1, b1, 64, 64, 64, 1)
        steps1 += 1
        if time.perf_counter() - t1 > 3.0:
            break
    single = 64 ** 3 * steps1 / (time.perf_counter() - t1)
    port.set_threads(cores)
    out = {"value": size ** 3 * steps / el, "unit": "cell-updates/s", "cores": cores, "kind": "port",
            "sample": f"{steps} full Strang steps of the {size}^3 turbulence box, oracle restatement of the "
                      f"reference C path with OpenMP over pencils ({cores} threads)",
            "single_core": {"value": single, "unit": "cell-updates/s", "cores": 1,
                            "sample": f"{steps1} Strang steps of the 64^3 vortex on one thread"}}
    rb = reference_build_timing()
    if rb:
        out["reference_build"] = rb
    return out


def reference_build_timing(o2_size: int = 128, o0_size: int = 64):
    """The reference's own C/ operators (oracle/_ref, compiled from its
    sources on this host), single-threaded as written, driven by the loop of
    C/mhd.c:59-124 with its copy_matrix calls: one Strang step of the
    turbulence box at o2_size^3 with -O2, and at o0_size^3 built as
    C/makefile builds it (no optimisation flags).  None when this host has no
    build of the reference."""
    sys.path.insert(0, str(ROOT / "tests"))
    from _oracle import REF, REF_O0, Oracle

    if not REF[32].exists():
        return None
    port = Oracle(32, "port")
    out = {}
    for key, kind, n, path in (("O2", "ref", o2_size, REF[32]), ("O0", "ref_O0", o0_size, REF_O0)):
        if not path.exists():
            continue
        ref = Oracle(32, kind)
        u, b = port.init_turbulence(n, seed=0)
        t0 = time.perf_counter()
        ref.strang(u, b, n, n, n, 1)
        el = time.perf_counter() - t0
        out[key] = {"value": n ** 3 / el, "unit": "cell-updates/s", "cores": 1, "kind": "reference",
                    "sample": f"one Strang step of the {n}^3 turbulence box, the reference's C/ operators built "
                              f"with {'-O2' if key == 'O2' else 'no optimisation flags (as C/makefile)'}, "
                              f"one thread, {el:.2f} s"}
    return out


def reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "tests"))
    from _oracle import Oracle  # the CPU arm: nothing of the GPU library is loaded here

    n = args.size
    kind, o = "port", Oracle(32, "port")
    u, b = o.init_turbulence(n, seed=0)  # the same seeded box, from the C source built into the oracle
    cores = o.max_threads()
    for _ in range(args.warmup):
        u, b, _, _, _ = o.strang(u, b, n, n, n, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        u, b, _, _, _ = o.strang(u, b, n, n, n, 1)
    el = time.perf_counter() - t0
    v = n ** 3 * args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": f"decaying turbulence {n}^3, FP32, CFL 0.7, plain Strang step",
                                            "grid": [n, n, n], "cpu": True},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": cores, "kind": kind,
                             "sample": f"full {n}^3 Strang steps; the reference's C/ arithmetic restated in "
                                       f"oracle/mhd_oracle.c (bit-identical to the reference build), OpenMP over "
                                       f"pencils, {cores} threads"},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    rb = reference_build_timing()
    if rb:
        line["cpu_baseline"]["reference_build"] = rb
    print(json.dumps(line), flush=True)


def fp64_error_leg(mhd, n: int, steps: int):
    """Per-field relative L2 of the FP32 kernels (FAST, the production path,
    and EXACT) against the FP64 build of the same method, after `steps`
    steps of the turbulence box from the same initial state."""
    from heterogeneous_mhd_gb300.diagnostics import field_errors

    out = {"grid": [n, n, n], "steps": steps, "reference": "FP64 build of the same kernels (EXACT policy)"}
    u64, b64 = mhd.init_turbulence(n, seed=0, fp64=True)
    u32, b32 = u64.astype(np.float32), b64.astype(np.float32)
    t0 = time.perf_counter()
    with mhd.Context(n, n, n, fp64=True, exact=True) as ctx:
        ctx.set_state(u64, b64)
        ctx.step(steps, cfl=0.7)
        ru, rb = ctx.get_state()
    out["fp64_seconds"] = time.perf_counter() - t0
    for name, exact in (("fast_f32", False), ("exact_f32", True)):
        with mhd.Context(n, n, n, exact=exact) as ctx:
            ctx.set_state(u32, b32)
            ctx.step(steps, cfl=0.7)
            fu, fb = ctx.get_state()
        out[name] = {k: float(f"{v:.3e}") for k, v in field_errors(fu, fb, ru, rb).items()}
    return out


CLOSURE_WEIGHTS = ROOT / "heterogeneous_mhd_gb300" / "closure_weights.npz"


def closure_conv_leg(torch, nb=4, n=64):
    """The closure net's tensor-core convolutions on nb boxes of n^3 seeded
    random inputs: one forward pass (four 3^3 layers and the 1^3 head) and
    one training iteration (forward, loss, backward, AdamW), CUDA events, for
    the warp-specialised tcgen05 kernel (the default), the two-buffer
    tcgen05 kernel and the mma.sync kernel."""
    from heterogeneous_mhd_gb300 import closure

    lib = closure.cl()
    g = torch.Generator(device="cuda").manual_seed(0)
    x = (torch.randn((nb, n ** 3 * 16), generator=g, device="cuda") * 0.5).to(torch.bfloat16)
    t = (torch.randn((nb, n ** 3 * 8), generator=g, device="cuda") * 0.1).to(torch.bfloat16)
    net = closure.ClosureNet(seed=0)
    flops = 2 * nb * n ** 3 * 27 * 32 * (16 + 3 * 32)  # the four 3^3 layers of one forward pass
    out = {"workload": f"{nb} boxes of {n}^3, BF16 in / FP32 accumulate", "fwd_3x3_gflop": flops / 1e9}
    prev = lib.mhd_cl_use_tcgen05(1)
    try:
        for mode, name in ((1, "tcgen05_warp_specialised"), (2, "tcgen05_two_buffer"), (0, "mma_sync")):
            lib.mhd_cl_use_tcgen05(mode)
            for _ in range(3):
                net.forward(x, nb, n)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(20):
                net.forward(x, nb, n)
            e1.record()
            e1.synchronize()
            fwd = e0.elapsed_time(e1) / 20
            e0.record()
            for _ in range(10):
                net.forward(x, nb, n)
                net.loss(t, nb, n)
                net.backward(x, nb, n)
                net.adamw(1e-4)
            e1.record()
            e1.synchronize()
            it = e0.elapsed_time(e1) / 10
            out[name] = {"forward_ms": round(fwd, 4), "fwd_3x3_tflops": round(flops / (fwd * 1e-3) / 1e12, 1),
                         "train_iter_ms": round(it, 4)}
        out["device_errors"] = int(lib.mhd_cl_device_errors())
    finally:
        lib.mhd_cl_use_tcgen05(prev)
    return out


def closure_leg(seeds=(1000, 1001, 1002, 1003), fine=256, factor=4, horizons=(0.5, 1.0, 2.0)):
    """The closure at matched error: held-out vortex seeds run to each horizon
    (turbulent crossing times) at fine^3 (plain) and at (fine/factor)^3
    (plain, and plain + the trained closure after every step, with the
    correction gain calibrated on validation seeds), compared after filtering
    the fine run; errors are means over the seeds; GPU time of the fine run
    over the closure run; the 5% target per quantity at the last horizon."""
    if not CLOSURE_WEIGHTS.exists():
        return {"unavailable": "no trained closure weights in the package"}
    from heterogeneous_mhd_gb300 import closure, closure_train

    net = closure.ClosureNet.load(CLOSURE_WEIGHTS)
    rep = closure_train.evaluate(net, list(seeds), fine, factor, horizons, log=None, gains=[net.gain])
    runs, sm = rep["runs"], rep["summary"]
    keys = ("rho_rel_l2", "magnetic_spectrum_err", "kinetic_spectrum_err")
    out = {"workload": f"vortex seeds {list(seeds)}, {fine}^3 plain vs {fine // factor}^3 plain and "
                       f"{fine // factor}^3 + closure, horizons {list(horizons)} crossing times",
           "gain": net.gain, "fine_ms": float(np.mean([r["fine_ms"] for r in runs])),
           "closure_ms": float(np.mean([r["closure"]["wall_ms"] for r in runs])),
           "plain_coarse_ms": float(np.mean([r["plain"]["wall_ms"] for r in runs])),
           "speedup_vs_fine": sm["speedup_vs_fine"], "fallback_rate": sm["fallback_rate"],
           "closure_divb_max": max(r["closure"]["per_horizon"][-1]["divb_max"] for r in runs)}
    for h in rep["horizons"]:
        out[f"t{h}"] = {k: {"plain": round(sm[f"plain_{k}@{h}"], 5), "closure": round(sm[f"closure_{k}@{h}"], 5)}
                        for k in keys}
    last = rep["horizons"][-1]
    out["target_5pct_at_last_horizon"] = {k: ("met" if sm[f"closure_{k}@{last}"] <= 0.05 else "missed")
                                          for k in ("rho_rel_l2", "magnetic_spectrum_err")}
    out["beats_plain_coarse_at_last_horizon"] = {k: bool(sm[f"closure_{k}@{last}"] < sm[f"plain_{k}@{last}"])
                                                 for k in keys}
    return out


def batch_leg(mhd, torch, rank, nboxes=256, steps=50, warmup=3, tune=True):
    """The batched workload: 256 vortex boxes of edge 32..128 with their own
    beta, Mach and dt, FP32, one graph per step; 50 timed steps, in two
    groupings of the same boxes: the work-list launches (one launch per
    operator over every size class, the library's default) and one launch
    per class and operator, whose launch shapes (with `tune`) are timed on
    each class alone first (autotune.tune_batch) and the fastest kept per
    class.  The faster grouping is the headline; both are reported."""
    cfg = mhd.batch_config(nboxes, seed=rank)
    cells = sum(x["n"] ** 3 for x in cfg)
    hbm, _ = peaks()

    def timed(bt):
        stream = torch.cuda.ExternalStream(bt.stream())
        bt.step(warmup)
        bt.sync()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = bt.launch_count()
        ev0.record(stream)
        bt.step(steps)
        ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1)
        bt.sync()
        step_gbs = STEP_BYTES["plain"] * cells / (ms / steps * 1e-3) / 1e9
        return {"ms_per_step": ms / steps, "value": cells * steps / (ms * 1e-3), "unit": "cell-updates/s",
                "step_alg_gbs": step_gbs, "step_frac": step_gbs / hbm,
                "gpu_launches": int(bt.launch_count() - l0)}

    def loaded_boxes(boxes):
        bt = mhd.Batch([x["n"] for x in boxes])
        for i, box in enumerate(boxes):
            bt.set_box(i, *mhd.init_batch_box(box))
        return bt

    def loaded():
        return loaded_boxes(cfg)

    bt = loaded()
    worklist = timed(bt)
    worklist["classes_in_worklist"] = bt.worklist_classes()
    worklist["launches_per_step"] = worklist["gpu_launches"] / steps
    bt.close()

    bt = loaded()
    bt.set_worklist(False)
    shapes = {}
    if tune:
        from heterogeneous_mhd_gb300 import autotune
        shapes = {str(e): {"knobs": k, "ms": round(ms, 3), "planner_ms": round(b, 3)}
                  for e, (k, ms, b) in autotune.tune_batch(bt, cfg).items()}
    per_class = timed(bt)
    per_class["launches_per_step"] = per_class["gpu_launches"] / steps
    per_class["launch_shapes_per_edge"] = shapes or "planner defaults"
    size_classes = bt.classes()
    bt.close()

    # each size class alone, in both groupings (the planner's launch shapes), after the
    # whole batch
    per_edge = {}
    for e in sorted({x["n"] for x in cfg}):
        boxes = [x for x in cfg if x["n"] == e]
        row = {"boxes": len(boxes)}
        for name, on in (("worklist_ms", True), ("per_class_ms", False)):
            one = loaded_boxes(boxes)
            one.set_worklist(on)
            row[name] = round(timed(one)["ms_per_step"], 4)
            one.close()
        per_edge[str(e)] = row

    head, grouping = (worklist, "worklist") if worklist["ms_per_step"] <= per_class["ms_per_step"] else \
        (per_class, "per_class")
    out = {"workload": f"{nboxes} vortex boxes, edges {sorted(set(x['n'] for x in cfg))}, beta 0.1-10, "
                       f"Mach 0.2-1.0, FP32, CFL 0.7, own dt per box",
           "boxes": nboxes, "cells": cells, "size_classes": size_classes, "steps": steps,
           "grouping": grouping}
    out.update({k: head[k] for k in ("ms_per_step", "value", "unit", "step_alg_gbs", "step_frac", "gpu_launches")})
    out["worklist"] = worklist
    out["per_class"] = per_class
    out["each_class_alone"] = per_edge
    return out


def time_steps(ctx, stream, torch, barrier, steps: int, fused: bool):
    """Graph-replay steps timed with CUDA events on the library's stream, and
    the same steps launched directly with an event pair around every kernel
    (per-kernel times).  Returns (ms, launches, ms_profiled, kernels)."""
    import heterogeneous_mhd_gb300 as mhd

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    l0 = ctx.launch_count()
    ev0.record(stream)
    ctx.step(steps, cfl=0.7, fused=fused)
    ev1.record(stream)
    ev1.synchronize()
    barrier()
    launches = ctx.launch_count() - l0
    ms = ev0.elapsed_time(ev1)
    ctx.profile(True)
    ctx.profile_reset()
    barrier()
    ev0.record(stream)
    ctx.step(steps, cfl=0.7, fused=fused)
    ev1.record(stream)
    ev1.synchronize()
    ms_prof = ev0.elapsed_time(ev1)
    kern = {k: ctx.profile_read(k) for k in mhd.KERNELS}
    ctx.profile(False)
    return ms, launches, ms_prof, kern


def variant_summary(variant: str, cells: int, steps: int, ms: float, kern: dict, hbm: float, n: int):
    """Throughput, step bandwidth in the fixed conventions and the roofline of
    the dominant kernel of one step variant."""
    sec = ms / steps * 1e-3
    out = {"ms_per_step": ms / steps, "value": cells / sec, "unit": "cell-updates/s"}
    out["step_alg_bytes_per_cell"] = STEP_BYTES[variant]
    out["step_alg_gbs"] = STEP_BYTES[variant] * cells / sec / 1e9
    out["step_frac"] = out["step_alg_gbs"] / hbm
    out["step_moved_bytes_per_cell"] = STEP_MOVED[variant]
    out["step_moved_frac"] = STEP_MOVED[variant] * cells / sec / 1e9 / hbm
    if variant == "fused":  # the five-pass bound of a fully fused sweep
        out["step_frac_5pass_320"] = STEP_BYTES["fused_5pass"] * cells / sec / 1e9 / hbm
    if kern:
        dom = max((k for k in kern if kern[k][1] > 0), key=lambda k: kern[k][0])
        tot_ms, nl = kern[dom]
        mean_ms = tot_ms / nl
        alg = ALG_BYTES[dom]
        achieved = alg * cells / (mean_ms * 1e-3) / 1e9
        moved = MOVED_BYTES.get(variant, {}).get(dom, alg)
        total = sum(x[0] for x in kern.values())
        out["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                           "frac": achieved / hbm, "alg_bytes_per_cell": alg, "alg_bytes_per_launch": alg * cells,
                           "mean_launch_ms": mean_ms, "traffic": measured_traffic(dom, n, variant),
                           "moved_bytes_per_cell": moved,
                           "frac_moved": moved * cells / (mean_ms * 1e-3) / 1e9 / hbm}
        out["kernels"] = {k: {"ms_total": round(v[0], 4), "launches": v[1], "share": round(v[0] / total, 4),
                              "mean_us": round(1e3 * v[0] / v[1], 2),
                              "frac": round(ALG_BYTES[k] * cells / (v[0] / v[1] * 1e-3) / 1e9 / hbm, 4)
                              if ALG_BYTES.get(k) else None}
                          for k, v in kern.items() if v[1] > 0}
    return out


def size512_leg(mhd, torch, steps=5, warmup=3):
    """The decaying-turbulence box at 512^3 (4.3 GB of state): the fused and
    the plain step, graph replay timed with CUDA events; the grid's headline
    figures are those of the faster variant (named in headline_variant)."""
    n = 512
    cells = n ** 3
    u0, b0 = mhd.init_turbulence(n, seed=0)
    hbm, _ = peaks()
    out = {"workload": "decaying turbulence 512^3, FP32, CFL 0.7, fused and plain Strang steps", "grid": [n, n, n],
           "steps": steps}
    with mhd.Context(n, n, n) as ctx:
        stream = torch.cuda.ExternalStream(ctx.stream())
        for variant in ("fused", "plain"):
            ctx.set_state(u0, b0)
            ctx.step(warmup, cfl=0.7, fused=(variant == "fused"))
            ctx.sync()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            ctx.step(steps, cfl=0.7, fused=(variant == "fused"))
            ev1.record(stream)
            ev1.synchronize()
            ms = ev0.elapsed_time(ev1)
            res = {"status": int(ctx.check())}
            res.update(variant_summary(variant, cells, steps, ms, {}, hbm, n))
            out[variant] = res
    del u0, b0
    # the headline figures of this grid are the faster variant's
    best = min(("fused", "plain"), key=lambda v: out[v]["ms_per_step"])
    out["headline_variant"] = best
    out.update({k: out[best][k] for k in ("ms_per_step", "value", "unit", "step_frac")})
    return out


def our_arm(args):
    import torch

    import heterogeneous_mhd_gb300 as mhd

    from heterogeneous_mhd_gb300.replicas import Replicas

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    rep = Replicas("nccl")
    n = args.size
    cells = n ** 3
    u0, b0 = mhd.init_turbulence(n, seed=rep.seed())
    tuned = {}
    if not args.no_tune:  # time the launch-shape candidates on this device first
        from heterogeneous_mhd_gb300 import autotune
        tuned = {k: v for k, v in autotune.tune(n, steps=2).items() if not k.startswith("_")}
    ctx = mhd.Context(n, n, n)
    ctx.set_state(u0, b0)
    stream = torch.cuda.ExternalStream(ctx.stream())
    main = args.variant
    other = "plain" if main == "fused" else "fused"
    hbm, src = peaks()

    def barrier():
        ctx.sync()
        torch.cuda.synchronize()
        rep.barrier()

    # warm-up of both variants (captures their step graphs), then one step of
    # each through the profiled direct-launch path
    for v in (main, other):
        ctx.step(args.warmup, cfl=0.7, fused=(v == "fused"))
        ctx.profile(True)
        ctx.step(1, cfl=0.7, fused=(v == "fused"))
        ctx.profile(False)
    barrier()

    # timed region: the production path of the headline variant, one CUDA graph replay per step
    with ClockSampler(torch.cuda.current_device()) as clk:
        ms, launches, ms_profiled, kern = time_steps(ctx, stream, torch, barrier, args.steps, main == "fused")
        ms_o, launches_o, ms_profiled_o, kern_o = time_steps(ctx, stream, torch, barrier, args.steps,
                                                             other == "fused")
        status = ctx.check()
    value, t_max = rep.throughput(cells, args.steps, ms)
    value_o, _ = rep.throughput(cells, args.steps, ms_o)

    # e2e: host state in and out of the C ABI every step
    hu = torch.empty(5 * cells, dtype=torch.float32, pin_memory=True)
    hb = torch.empty(3 * cells, dtype=torch.float32, pin_memory=True)
    hu.numpy()[:] = u0
    hb.numpy()[:] = b0
    e2e_steps = max(3, min(args.steps, 10))
    ctx.step_host(hu, hb, 1, cfl=0.7, fused=(main == "fused"))  # warm-up (the copy stream's first use)
    # The host link is shared with the rest of the machine and its speed varies
    # from second to second: E2E_TRIALS interleaved trials of both paths, the
    # median trial of each is reported (all trials are listed).
    t_host, t_three = [], []
    for _ in range(E2E_TRIALS):
        hu.numpy()[:] = u0
        hb.numpy()[:] = b0
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            # H2D from pinned memory, one step, D2H into the same buffers (synchronous)
            ctx.step_host(hu, hb, 1, cfl=0.7, fused=(main == "fused"))
        t_host.append(time.perf_counter() - t0)
        # the same with the three calls and no overlap of the copies with the step
        hu.numpy()[:] = u0
        hb.numpy()[:] = b0
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ctx.set_state(hu, hb)
            ctx.step(1, cfl=0.7, fused=(main == "fused"))
            ctx.get_state_into(hu, hb)
        t_three.append(time.perf_counter() - t0)
    t_host = rep.max(t_host)
    t_three = rep.max(t_three)
    e2e = world * cells * e2e_steps / statistics.median(t_host)
    e2e3 = world * cells * e2e_steps / statistics.median(t_three)
    e2e_trials = {"mhd_step_host": [world * cells * e2e_steps / t for t in t_host],
                  "three_calls": [world * cells * e2e_steps / t for t in t_three]}
    if rank != 0:
        ctx.close()
        rep.close()
        return

    head = variant_summary(main, cells, args.steps, ms, kern, hbm, n)
    sub = variant_summary(other, cells, args.steps, ms_o, kern_o, hbm, n)
    sub.update({"value": value_o, "gpu_launches": int(launches_o), "profiled_ms_per_step": ms_profiled_o / args.steps})
    roof = head["roofline"]
    roof["peak_source"] = src
    roof.update({"step_alg_gbs": head["step_alg_gbs"], "step_frac": head["step_frac"],
                 "step_alg_bytes_per_cell": head["step_alg_bytes_per_cell"],
                 "step_moved_bytes_per_cell": head["step_moved_bytes_per_cell"],
                 "step_moved_frac": head["step_moved_frac"]})
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"decaying turbulence {n}^3, FP32, CFL 0.7, {main} Strang step",
                   "grid": [n, n, n], "variant": main, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "state 537 MB > L2, no flush", "launch_shapes": tuned or "planner defaults"},
        "e2e": {"value": e2e, "unit": "cell-updates/s", "h2d_bytes_per_step": 32 * cells,
                "d2h_bytes_per_step": 32 * cells, "steps": e2e_steps,
                "api": "mhd_step_host (copies overlapped with the step)",
                "three_calls_value": e2e3, "three_calls_api": "mhd_set_state + mhd_step + mhd_get_state",
                "trials": e2e_trials, "statistic": f"median of {E2E_TRIALS} interleaved trials of {e2e_steps} steps"},
        "roofline": roof,
        "kernels": head["kernels"],
        "profiled_ms_per_step": ms_profiled / args.steps,
        "gpu_launches": int(launches),
        other: sub,
        "clocks": clk.summary(),
        "status": int(status),
    }
    if main == "fused":
        line["step_frac_5pass_320"] = head["step_frac_5pass_320"]
    ctx.close()
    del hu, hb
    if not args.no_512 and world == 1:
        # the 256^3 launch shapes do not carry over: the 512^3 leg runs the planner's own choices
        from heterogeneous_mhd_gb300 import autotune
        autotune.apply({})
        line["size512"] = size512_leg(mhd, torch)
        autotune.apply(tuned)
    if not args.no_fp64:
        line["fp64_error"] = fp64_error_leg(mhd, n, args.fp64_steps)
    if not args.no_batch:
        # the batch's launch shapes are the planner's: the tuned single-box knobs do not carry over
        from heterogeneous_mhd_gb300 import autotune
        autotune.apply({})
        line["batch"] = batch_leg(mhd, torch, rank, tune=not args.no_tune)
    if not args.no_closure:
        line["closure"] = closure_leg()
        line["closure"]["conv"] = closure_conv_leg(torch)
    if world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(n)
    print(json.dumps(line), flush=True)
    rep.close()


def ncu_case(args):
    """A short run for ncu captures: `--size`^3 turbulence, planner launch
    shapes (no autotuner), graphs off so every kernel is a direct launch;
    one warm-up step and two measured steps, no JSON line."""
    import heterogeneous_mhd_gb300 as mhd

    n = args.size
    u0, b0 = mhd.init_turbulence(n, seed=0)
    for kv in args.knob:
        key, val = kv.split("=")
        if mhd.lib().mhd_tune_set(key.encode(), int(val)) != 0:
            raise SystemExit(f"bad knob {kv}")
    with mhd.Context(n, n, n) as ctx:
        ctx.use_graphs(False)
        ctx.set_state(u0, b0)
        ctx.step(3, cfl=0.7, fused=args.variant == "fused")
        ctx.sync()
        assert ctx.check() == mhd.MHD_OK


def ncu_closure_case(args):
    """A short run of the closure's kernels for ncu captures: three training
    iterations (forward, loss, backward, AdamW) of the net on 4 boxes of
    64^3 seeded random inputs and targets, no JSON line."""
    import torch

    from heterogeneous_mhd_gb300 import closure

    nb, n = 4, 64
    closure.cl().mhd_cl_use_tcgen05(args.tcgen05)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = (torch.randn((nb, n ** 3 * 16), generator=g, device="cuda") * 0.5).to(torch.bfloat16)
    t = (torch.randn((nb, n ** 3 * 8), generator=g, device="cuda") * 0.1).to(torch.bfloat16)
    net = closure.ClosureNet(seed=0)
    for _ in range(3):
        net.forward(x, nb, n)
        net.loss(t, nb, n)
        net.backward(x, nb, n)
        net.adamw(1e-4)
    torch.cuda.synchronize()


def ncu_batch_case(args):
    """A short run of the batch's work-list kernels for ncu captures: the
    first 32 boxes of the batched workload's table (edges 32-128, 26 M
    cells, 1.9 GB of states and side arrays), three work-list steps, no
    JSON line."""
    import heterogeneous_mhd_gb300 as mhd

    cfg = mhd.batch_config(32, seed=0)
    with mhd.Batch([x["n"] for x in cfg]) as bt:
        for i, box in enumerate(cfg):
            bt.set_box(i, *mhd.init_batch_box(box))
        bt.step(3)
        bt.sync()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--variant", default="fused", choices=["plain", "fused"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-tune", action="store_true", help="skip the launch-shape autotuner")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-boxes leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 error leg")
    ap.add_argument("--no-closure", action="store_true", help="skip the learned-closure leg")
    ap.add_argument("--no-512", action="store_true", help="skip the 512^3 plain-step leg")
    ap.add_argument("--ncu-case", action="store_true", help="run the short profiling case only")
    ap.add_argument("--ncu-closure", action="store_true", help="run the short closure profiling case only")
    ap.add_argument("--ncu-batch", action="store_true", help="run the short work-list batch profiling case only")
    ap.add_argument("--tcgen05", type=int, default=1,
                    help="--ncu-closure: 1 warp-specialised tcgen05 convolution, 2 two-buffer, 0 mma.sync")
    ap.add_argument("--knob", action="append", default=[], help="launch-shape knob key=value for --ncu-case")
    ap.add_argument("--fp64-steps", type=int, default=100, help="steps of the FP64 error leg")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.ncu_closure:
        ncu_closure_case(args)
    elif args.ncu_batch:
        ncu_batch_case(args)
    elif args.ncu_case:
        ncu_case(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        our_arm(args)


if __name__ == "__main__":
    main()
