"""Program::scatter on the GPU through include/gpugas.h: a user program whose
scatter writes edge data that later gathers read, against a restatement of
refgas.h's loop (refgas.h:143-229) for that program.  The reference GPU
engine never runs scatter (gpugas.h:942); programs opt in with
`static const bool runScatter = true;`."""
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_names, load_golden
from graphreduce_gb300 import _lib
from graphreduce_gb300.graph import edge_list_to_csr

pytestmark = pytest.mark.gpu

INT_MAX = 2**31 - 1


def refgas_aging(nV, src, dst, uses):
    """refgas.h's gather / apply / scatterActivate / nextIter for the aging
    program, all vertices active at the start."""
    uses = uses.astype(np.int64).copy()
    label = 3 * np.arange(nV, dtype=np.int64)
    csc_off, csc_src, csc_perm = edge_list_to_csr(nV, dst, src)
    csr_off, csr_dst, csr_perm = edge_list_to_csr(nV, src, dst)
    active = list(range(nV))
    iters = 0
    while active:
        g = []
        for v in active:
            acc = INT_MAX
            for ie in range(csc_off[v], csc_off[v + 1]):
                acc = min(acc, label[csc_src[ie]] + uses[csc_perm[ie]])
            g.append(acc)
        ret = []
        for v, acc in zip(active, g):
            ret.append(acc < label[v])
            if acc < label[v]:
                label[v] = acc
        flags = np.zeros(nV, bool)
        for v, r in zip(active, ret):
            if not r:
                continue
            for ie in range(csr_off[v], csr_off[v + 1]):
                d = csr_dst[ie]
                flags[d] = True
                uses[csr_perm[ie]] += 1 + ((label[v] + label[d]) & 1)
        active = list(np.nonzero(flags)[0])
        iters += 1
    return label.astype(np.int32), uses.astype(np.int32), iters


@pytest.fixture(scope="module")
def driver(libgas, tmp_path_factory):
    out = tmp_path_factory.mktemp("scat") / "scatter_driver"
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    libdir = str(_lib.lib_path().parent)
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
           f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "scatter_driver.cu"),
           f"-L{libdir}", "-lgas", "-Xlinker", f"-rpath={libdir}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.mark.parametrize("name", golden_names())
def test_gpu_scatter_matches_refgas_loop(driver, tmp_path, name):
    g = load_golden(name)
    nV, src, dst = int(g["nV"]), g["src"], g["dst"]
    w = np.asarray(g["w"], np.int32) & 3    # small ages: labels keep falling for a while
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        np.array([nV, len(src)], np.int32).tofile(f)
        for a in (src, dst, w):
            np.asarray(a, np.int32).tofile(f)
    r = subprocess.run([str(driver), str(fin), str(fout)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(fout, np.int32)
    label, uses, iters = raw[:nV], raw[nV:nV + len(src)], int(raw[-1])
    ref_label, ref_uses, ref_iters = refgas_aging(nV, np.asarray(src), np.asarray(dst),
                                                  np.asarray(w))
    np.testing.assert_array_equal(label, ref_label)
    np.testing.assert_array_equal(uses, ref_uses)
    assert iters == ref_iters
