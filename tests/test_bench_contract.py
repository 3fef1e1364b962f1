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


def test_reference_arm_never_loads_the_product_library():
    """The CPU arm builds its inputs with the oracle's own generators: after
    a run, neither the package nor libgas.so is in the process."""
    code = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--scale', '11', '--steps', '9',"
        " '--warmup', '0']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libgas' not in maps, 'libgas.so mapped'\n"
        "assert not any(m.startswith('graphreduce_gb300') for m in sys.modules)\n"
        "assert 'liboracle' in maps\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    assert "CC" in d["cpu_baseline"]["sample"] and "sssp7" in d["cpu_baseline"]["sample"]
