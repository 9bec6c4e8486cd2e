"""bench.py --impl reference on the CPU (no GPU needed): one JSON line with the keys the
line must carry, the requested numbers of timed and warm-up samples, and timed samples
that tile the GPU arm's window of the same trajectories."""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_reference_line():
    out = subprocess.check_output([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                                   "--steps", "3", "--warmup", "1", "--cpu-steps", "6000"], text=True, cwd=ROOT)
    line = json.loads([l for l in out.splitlines() if l.startswith("{")][-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "cpu_baseline",
              "e2e", "config"):
        assert k in line, k
    assert line["impl"] == "reference" and line["steps"] == 3 and line["warmup"] == 1
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "3 samples tiling steps" in cb["sample"]
