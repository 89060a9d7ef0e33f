"""The reference arm of bench.py runs on the CPU (no GPU needed): its one JSON
line keeps the driver's contract -- the metric, value and unit, the
reference tag, a cpu_baseline describing the run, an e2e block without host
copies, and the noiseless rate beside the noisy one."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "surface_d5", "--steps", "1", "--warmup", "1", "--cpu-shots", "64"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "shot-gates/s" and d["value"] > 0
    assert d["metric"].startswith("shot-gates/s") and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["noiseless"]["value"] > 0
    assert d["config"]["num_qubits"] == 49 and d["config"]["gates_per_shot"] > 0
