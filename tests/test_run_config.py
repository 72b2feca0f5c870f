"""Configuration of the run driver (no GPU): defaults, then the JSON file,
then the command-line flags."""
import json
import math

import pytest

from heterogeneous_mhd_gb300 import run


def test_defaults():
    cfg = run.parse([])
    assert cfg["n"] == 64 and cfg["ic"] == "vortex" and cfg["cfl"] == 0.7 and math.isinf(cfg["tf"])
    assert cfg["exact"] is False and cfg["log"] is None


def test_config_file_then_flags(tmp_path):
    p = tmp_path / "run.json"
    p.write_text(json.dumps({"n": 32, "ic": "turbulence", "steps": 7, "exact": True, "checkpoint_every": 3}))
    cfg = run.parse(["--config", str(p), "--steps", "9", "--cfl", "0.5", "--log", "x.jsonl"])
    assert cfg["n"] == 32 and cfg["ic"] == "turbulence" and cfg["exact"] is True
    assert cfg["steps"] == 9 and cfg["cfl"] == 0.5 and cfg["log"] == "x.jsonl" and cfg["checkpoint_every"] == 3


def test_bad_config_is_refused(tmp_path):
    p = tmp_path / "run.json"
    p.write_text(json.dumps({"n": 32, "gamma": 1.4}))
    with pytest.raises(SystemExit):
        run.parse(["--config", str(p)])
    with pytest.raises(SystemExit):
        run.parse(["--ic", "shock"])
