"""bench.py's CPU arms on small samples: whole SR steps of the CPU restatement (never scaled),
and the reference arm's line carrying the same workload `config` as the GPU arm."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def test_whole_cpu_steps_both_workloads():
    sys.path.insert(0, str(ROOT))
    import bench
    for wl, chains in (("rbm", 64), ("resconv", 8)):
        n, t, phases, energies = bench.time_cpu_steps(wl, chains, 2, 0.0)
        assert n == 1 and t > 0  # the budget is spent after the first whole step
        assert {"sweep", "eloc", "gram", "solve"} <= set(phases)
        assert np.isfinite(energies).all()


def test_reference_line_config_matches_gpu_arm():
    sys.path.insert(0, str(ROOT))
    import bench
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "rbm",
                          "--steps", "3", "--warmup", "2", "--ref-budget", "0"], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 1 and line["warmup"] == 0
    assert line["config"] == bench.WORKLOADS["rbm"]
    assert line["value"] == line["cpu_baseline"]["value"] == line["e2e"]["value"]
    assert line["cpu_baseline"]["scaled"] is False
