"""gas_pagerank_step_noalloc: the PageRank step for callers that cannot
allocate device memory (their allocator owns the device, or their request
path must not call cudaMalloc).  It is called through the C ABI with
caller-owned device buffers, iterated to convergence, and compared with
gas_engine_pagerank_precision (which allocates its own buffers) within the
precision-form tolerance used everywhere else: L1 distance <= 1e-6.  Two full
runs in a row must both match, since every call shares one scratch array.

This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from graphreduce_gb300 import GASEngineGPU, _lib
from graphreduce_gb300.engine import initial_vertex_data
from graphreduce_gb300.graph import EdgeList, edge_list_to_csr

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _bind(lib):
    fn = lib.gas_pagerank_step_noalloc
    fn.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int32
    return fn


def _run_noalloc(step, el, torch, max_iter=1000):
    dev = torch.device("cuda", 0)
    off, src_csc, _ = edge_list_to_csr(el.nV, el.dst, el.src)
    d_off = torch.from_numpy(off).to(dev)
    d_src = torch.from_numpy(src_csc).to(dev)
    d_deg = torch.from_numpy(el.out_degree()).to(dev)
    r = torch.full((el.nV,), 1.0 / el.nV, dtype=torch.float32, device=dev)
    r2 = torch.empty_like(r)
    l1 = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for it in range(1, max_iter + 1):
        st = step(el.nV, el.nE, d_off.data_ptr(), d_src.data_ptr(), d_deg.data_ptr(),
                  r.data_ptr(), r2.data_ptr(), 0.85, l1.data_ptr(), stream)
        assert st == 0, _lib.load().gas_last_error()
        r, r2 = r2, r
        if float(l1.item()) <= TOL:
            return r.cpu().numpy(), it
    raise AssertionError("no convergence")


def test_noalloc_step_matches_engine_twice():
    torch = pytest.importorskip("torch")
    step = _bind(_lib.load())
    el = EdgeList.rmat(14, 16, seed=4, symmetrize=False)
    eng = GASEngineGPU("pagerank")
    vd = initial_vertex_data("pagerank", el.nV, 0, el.out_degree())
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    ref, st = eng.pagerank_precision(0.85, TOL)
    for _ in range(2):
        ranks, it = _run_noalloc(step, el, torch)
        assert np.abs(ranks.astype(np.float64) - ref.astype(np.float64)).sum() <= TOL
        assert it == st.iterations


def test_noalloc_rejects_graphs_beyond_its_scratch():
    step = _bind(_lib.load())
    too_big = (1 << 29) - 100
    st = step(200, too_big, None, None, None, None, None, 0.85, None, None)
    assert st == 9  # GAS_ERR_TOO_LARGE
    assert b"scratch" in _lib.load().gas_last_error()
