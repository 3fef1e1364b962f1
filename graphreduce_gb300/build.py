"""Builds libgas.so (sm_103a) in-tree, and the oracle's C library.

``python -m graphreduce_gb300.build`` compiles every translation unit of
``graphreduce_gb300/csrc`` with nvcc in parallel and links
``graphreduce_gb300/_lib/libgas.so``.  Nothing is installed: the library is
loaded from the source tree by ``graphreduce_gb300._lib``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
BUILD_DIR = PKG / "_build"
LIB = OUT_DIR / "libgas.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-fopenmp,-fvisibility=default",
    f"-I{INCLUDE}", f"-I{CSRC}",
]
SOURCES = ["gas_engine.cu", "gas_runs.cu", "gas_sched.cu", "gas_small.cu", "gas_noalloc.cu",
           "gas_batch.cu", "gas_build.cu", "gas_learn.cu", "gas_host_graph.cpp"]
# Programs built against libgas and include/gpugas.h: the drop-in path's
# benchmark driver (bench.py runs it for the user-program figures).
TOOLS = ["bench_user_programs.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; libgas needs the CUDA toolkit to build")
    return cand


def _compile(src: Path) -> Path:
    obj = BUILD_DIR / (src.name + ".o")
    deps = [src] + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(
        INCLUDE.glob("*.h")) + sorted(INCLUDE.glob("*.cuh"))
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd[1:1] = ["-x", "c++"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    """Compiles (incrementally) and links libgas.so; returns its path."""
    OUT_DIR.mkdir(exist_ok=True)
    BUILD_DIR.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs),
               "-Xcompiler", "-fopenmp", "-lgomp"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    for tool in TOOLS:
        src = CSRC / tool
        exe = OUT_DIR / Path(tool).stem
        deps = [src, LIB] + sorted(INCLUDE.glob("*.h")) + sorted(INCLUDE.glob("*.cuh"))
        if exe.exists() and all(exe.stat().st_mtime >= d.stat().st_mtime for d in deps):
            continue
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", f"-I{INCLUDE}", str(src),
               f"-L{OUT_DIR}", "-lgas", "-Xlinker", f"-rpath={OUT_DIR}", "-o", str(exe)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {tool}:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(with_reference: bool = True) -> None:
    """Builds oracle/_build/liboracle.so, and oracle/_ref/libref.so when the
    environment names a reference checkout in REF_DIR (test infrastructure
    only)."""
    oracle = ROOT / "oracle"
    res = subprocess.run(["make", "-s", "-C", str(oracle)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    ref = os.environ.get("REF_DIR", "")
    ref_dir = Path(ref) if ref else None
    if with_reference and ref_dir is not None and (ref_dir / "refgas.h").exists():
        res = subprocess.run(["make", "-s", "-C", str(oracle), "ref", f"REF_DIR={ref_dir}"],
                             capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{res.stdout}\n{res.stderr}")


if __name__ == "__main__":
    build(verbose=True)
    build_oracle()
    sys.exit(0)
