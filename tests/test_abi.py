"""The C ABI library loads without a GPU and exports every entry point that
include/gas.h declares; the drop-in header path compiles the reference's
unchanged apps.  CPU only."""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import HAVE_REF, REF_DIR, REF_SKIP, ROOT
from graphreduce_gb300 import _lib


def declared_functions():
    text = (ROOT / "include" / "gas.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    # function names; a type name before "(" (a function-pointer typedef) is not one
    return sorted({f for f in re.findall(r"\b(gas_[a-z0-9_]+)\s*\(", text)
                   if not f.endswith("_t")})


def test_library_exports_every_declared_symbol(libgas):
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.lib_path())],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    for f in declared_functions():
        assert hasattr(libgas, f)


def test_python_binding_covers_header():
    assert set(declared_functions()) == set(_lib.exported_symbols())


def test_status_strings(libgas):
    assert libgas.gas_status_string(0) == b"ok"
    assert libgas.gas_status_string(4) == b"iteration cap reached"
    assert b"sm_103a" in libgas.gas_version()


def test_engine_rejects_calls_out_of_order(libgas):
    import graphreduce_gb300 as g
    eng = g.GASEngineGPU("cc")
    with pytest.raises(g.GasError) as ei:
        eng.setActive(0, 1)
    assert ei.value.status == 6
    with pytest.raises(ValueError):
        g.GASEngineGPU("nope")


@pytest.mark.skipif(not HAVE_REF, reason=REF_SKIP)
def test_reference_apps_compile_unchanged_against_gpugas_h(libgas, tmp_path):
    """bfs.cu, sssp.cu, pagerank.cu and connected_component.cu, byte for byte
    as the reference ships them, build against include/gpugas.h + libgas."""
    for f in ["bfs.cu", "sssp.cu", "pagerank.cu", "connected_component.cu", "refgas.h",
              "util.cuh", "util.cu", "graphio.h", "graphio.cpp"]:
        shutil.copy(REF_DIR / f, tmp_path / f)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    arch = ["-gencode", "arch=compute_103a,code=sm_103a"]
    inc = f"-I{ROOT / 'include'}"
    libdir = str(_lib.lib_path().parent)

    def run(cmd):
        r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]

    run([nvcc, *arch, "-c", "util.cu", "-o", "util.o"])
    run([nvcc, "-O0", "-Xcompiler", "-fno-unreachable-traps", "-c", "graphio.cpp",
         "-o", "graphio.o"])
    for app in ["bfs", "sssp", "connected_component", "pagerank"]:
        run([nvcc, *arch, "-std=c++17", "-Xcompiler", "-fpermissive", inc, "-c",
             f"{app}.cu", "-o", f"{app}.o"])
        run([nvcc, *arch, f"{app}.o", "util.o", "graphio.o", f"-L{libdir}", "-lgas",
             f"-Xlinker", f"-rpath={libdir}", "-lz", "-o", app])
        assert (tmp_path / app).exists()


def test_sssp_weights_outside_the_programs_margin_are_rejected(libgas):
    """sssp.cu:32-33 sets gatherZero = INT_MAX - 100000, so dist + w only
    fits for weights in [0, 100000]: set_graph and the batch refuse others
    before any device work."""
    import numpy as np

    import graphreduce_gb300 as g
    from graphreduce_gb300.engine import initial_vertex_data
    src = np.array([0, 1, 2], np.int32)
    dst = np.array([1, 2, 0], np.int32)
    for bad in (100001, -1, 2**31 - 1):
        w = np.array([1, bad, 3], np.int32)
        eng = g.GASEngineGPU("sssp")
        with pytest.raises(g.GasError) as ei:
            eng.setGraph(3, initial_vertex_data("sssp", 3, 0), 3, w, src, dst)
        assert ei.value.status == 1 and "100000" in str(ei.value)
        eng.close()
        b = g.Batch()
        with pytest.raises(g.GasError) as ei:
            b.add_graph(3, src, dst, w)
        assert ei.value.status == 1
        b.close()
