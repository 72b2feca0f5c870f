"""What the trained closure gains over the method without it, on a held-out
seed: the 64^3 run corrected after every step against the plain 64^3 run,
both compared with the 256^3 plain run filtered to 64^3 after half a
turbulent crossing time (weights: heterogeneous_mhd_gb300/closure_weights.npz,
trained on the solver's own pairs from seeds 0-47)."""
import json
import os
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WEIGHTS = Path(__file__).resolve().parents[1] / "heterogeneous_mhd_gb300" / "closure_weights.npz"


def test_trained_closure_beats_plain_coarse(mhd, cuda):
    from heterogeneous_mhd_gb300 import closure, closure_train
    net = closure.ClosureNet.load(WEIGHTS)
    rep = closure_train.evaluate(net, [1000], fine=256, factor=4, crossings=[0.5], log=None)
    s = rep["summary"]
    out = Path(os.environ.get("MHD_METRICS_DIR", "")) if os.environ.get("MHD_METRICS_DIR") else None
    if out is not None and out.is_dir():
        (out / "closure_eval_test.json").write_text(json.dumps(s, indent=1))
    assert s["closure_rho_rel_l2@0.5"] < s["plain_rho_rel_l2@0.5"]
    assert s["closure_magnetic_spectrum_err@0.5"] < s["plain_magnetic_spectrum_err@0.5"]
    assert s["closure_kinetic_spectrum_err@0.5"] < s["plain_kinetic_spectrum_err@0.5"]
    run = rep["runs"][0]["closure"]["per_horizon"][0]
    assert run["reached_t"]
    # the B correction is a curl: div B of the corrected run stays at FP32 round-off
    assert run["divb_max"] < 1e-5
    assert s["speedup_vs_fine"] > 10
