"""bench.py's reference arm (the CPU restatement, all host threads) on small
samples of its configs: one JSON line with the contract's keys."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("config", ["robertson", "robertson_ros23", "lorenz_dense", "bouncing_ball", "van_der_pol",
                                    "serving"])
def test_reference_arm_prints_one_json_line(config):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", config,
                        "--trajectories", "64", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    if config == "serving":
        assert "unavailable" in d
        return
    assert d["value"] > 0 and d["unit"] == "trajectories/s" and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
