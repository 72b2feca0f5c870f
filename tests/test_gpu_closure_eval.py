"""What the trained closure gains over the method without it, on held-out
seeds: the 64^3 run corrected after every step (with the package's
calibrated correction gain) against the plain 64^3 run, both compared with
the 256^3 plain run filtered to 64^3 after half a turbulent crossing time and
after two (weights: heterogeneous_mhd_gb300/closure_weights.npz, trained on
the solver's own pairs from seeds 0-47, gain chosen on seeds 48-55).

At two crossing times the closure is asserted to beat the plain coarse run
on density and on the magnetic spectrum (means over four seeds); the kinetic
spectrum at that horizon is recorded, not asserted: there the corrected run
is worse than the plain one."""
import json
import os
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WEIGHTS = Path(__file__).resolve().parents[1] / "heterogeneous_mhd_gb300" / "closure_weights.npz"


def _record(name, s):
    out = Path(os.environ.get("MHD_METRICS_DIR", "")) if os.environ.get("MHD_METRICS_DIR") else None
    if out is not None and out.is_dir():
        (out / name).write_text(json.dumps(s, indent=1))


def test_trained_closure_beats_plain_coarse(mhd, cuda):
    from heterogeneous_mhd_gb300 import closure, closure_train
    net = closure.ClosureNet.load(WEIGHTS)
    rep = closure_train.evaluate(net, [1000], fine=256, factor=4, crossings=[0.5], log=None, gains=[net.gain])
    s = rep["summary"]
    _record("closure_eval_test.json", s)
    assert s["closure_rho_rel_l2@0.5"] < s["plain_rho_rel_l2@0.5"]
    assert s["closure_magnetic_spectrum_err@0.5"] < s["plain_magnetic_spectrum_err@0.5"]
    assert s["closure_kinetic_spectrum_err@0.5"] < s["plain_kinetic_spectrum_err@0.5"]
    run = rep["runs"][0]["closure"]["per_horizon"][0]
    assert run["reached_t"]
    # the B correction is a curl: div B of the corrected run stays at FP32 round-off
    assert run["divb_max"] < 1e-5
    assert s["speedup_vs_fine"] > 10


def test_trained_closure_at_two_crossing_times(mhd, cuda):
    from heterogeneous_mhd_gb300 import closure, closure_train
    net = closure.ClosureNet.load(WEIGHTS)
    rep = closure_train.evaluate(net, [1000, 1001, 1002, 1003], fine=256, factor=4, crossings=[1.0, 2.0], log=None,
                                 gains=[net.gain])
    s = rep["summary"]
    _record("closure_eval_t2_test.json", s)
    for h in (1.0, 2.0):
        assert s[f"closure_rho_rel_l2@{h}"] < s[f"plain_rho_rel_l2@{h}"], h
        assert s[f"closure_magnetic_spectrum_err@{h}"] < s[f"plain_magnetic_spectrum_err@{h}"], h
    assert s["closure_kinetic_spectrum_err@1.0"] < s["plain_kinetic_spectrum_err@1.0"]
    for r in rep["runs"]:
        last = r["closure"]["per_horizon"][-1]
        assert last["reached_t"] and last["divb_max"] < 1e-5 and last["rho_min"] > 0
    assert s["speedup_vs_fine"] > 10
