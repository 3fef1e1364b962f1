"""bench.py's reference arm runs the oracle port on the host cores only, so
its JSON line can be checked here at a small scale: the keys the bench
contract names, the reference-arm extras (impl, cpu_baseline, an e2e that
moves no bytes) and the metric label following --scale."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    out = subprocess.run(
        [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--scale", "12",
         "--steps", "1", "--warmup", "0"],
        cwd=ROOT, capture_output=True, text=True, timeout=600, check=True).stdout
    d = json.loads(out.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == "GTEPS (SSSP x8 + CC, R-MAT scale 12)"
    assert d["unit"] == "GTEPS" and d["higher_is_better"] is True and d["value"] > 0
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "GTEPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
