"""bench.py's reference arm (--impl reference): the reference's CPU algorithm
(the oracle port, GMRES(30)+ILU(0) per system) timed on the host cores over
two outer iterations and scaled to the workload's outer-iteration count.  It
needs no GPU, so its JSON line is checked here."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_its_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "square20k",
                        "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["config"]["workload"] == "square20k" and line["config"]["outer_iterations"] == 198
    assert line["value"] > 0 and line["value"] == line["config"]["s_per_outer_iteration"] * 198
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
