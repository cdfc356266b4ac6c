"""The benchmark's reference arm (the CPU FP64 oracle on the host cores) runs
without a GPU and prints the contract's JSON line."""
from __future__ import annotations

import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line(oracle_mod):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "2", "--warmup", "0", "--N", "4096"],
                         capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["higher_is_better"] is False
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    # every timed sample is one complete map, scaled by the stated maps per step
    assert len(line["map_ms"]) == 2 and line["extrapolated"] is True
    assert abs(line["value"] - line["per_map_ms"] * line["maps_per_step"]) <= 0.1 * line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    # `steps` is the fraction of a converged step the timed maps make up, so that
    # ms_per_step x steps matches the timed region
    assert line["maps_timed"] == 2
    assert abs(line["steps"] - 2 / line["maps_per_step"]) < 1e-4
    assert abs(line["ms_per_step"] * line["steps"] - sum(line["map_ms"])) <= 0.2 * sum(line["map_ms"])
