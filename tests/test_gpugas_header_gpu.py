"""The drop-in header path: user programs compiled through include/gpugas.h
(tests/cpp/gpugas_driver.cu, the reference apps' programs and driver loops
written anew) against the reference's golden outputs."""
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden
from graphreduce_gb300 import _lib
from test_oracle import pr_histogram_ok

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(libgas, tmp_path_factory):
    out = tmp_path_factory.mktemp("drv") / "gpugas_driver"
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    libdir = str(_lib.lib_path().parent)
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
           f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "gpugas_driver.cu"),
           f"-L{libdir}", "-lgas", "-Xlinker", f"-rpath={libdir}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.mark.parametrize("host_loop", [False, True])
@pytest.mark.parametrize("name", golden_names())
def test_header_engine_matches_reference(driver, tmp_path, name, host_loop):
    """BFS and SSSP through the step API (as bfs.cu / sssp.cu drive it), CC
    and PageRank through run() (connected_component.cu, pagerank.cu): run()
    is one CUDA-graph launch with the loop on the device, or direct launches
    with GAS_HOST_LOOP=1; both give the reference's results."""
    import os
    g = load_golden(name)
    nV = int(g["nV"])
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        np.array([nV, len(g["src"]), int(g["source"])], np.int32).tofile(f)
        for k in ("src", "dst", "w"):
            np.asarray(g[k], np.int32).tofile(f)
    env = dict(os.environ)
    env.pop("GAS_HOST_LOOP", None)
    if host_loop:
        env["GAS_HOST_LOOP"] = "1"
    r = subprocess.run([str(driver), str(fin), str(fout)], capture_output=True, text=True,
                       env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(fout, np.int32)
    parts = []
    for _ in range(4):
        parts.append((raw[:nV], raw[nV]))
        raw = raw[nV + 1:]
    launches = raw[:2]
    (bfs, bit), (sssp, sit), (cc, cit), (pr, pit) = parts
    # run() with an empty start set returns at once; otherwise one launch
    want = 0 if host_loop else 1
    assert launches[0] == (want if g["cc_iters"] > 0 else 0)
    assert launches[1] == (want if g["pr_iters"] > 0 else 0)
    assert pit == g["pr_iters"]
    assert r.stdout.count("Iterations: ") == 2
    np.testing.assert_array_equal(bfs, g["bfs_depth"])
    assert bit == g["bfs_iters"]
    np.testing.assert_array_equal(sssp, g["sssp_dist"])
    assert sit == g["sssp_iters"]
    np.testing.assert_array_equal(cc, g["cc_label"])
    assert cit == g["cc_iters"]
    prf = pr.view(np.float32)
    assert pr_histogram_ok(prf, g["pr_rank"])
    np.testing.assert_allclose(prf, g["pr_rank"], rtol=1e-5, atol=1e-5)
