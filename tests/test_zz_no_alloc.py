"""gas_pagerank_step_noalloc: the PageRank step for callers that cannot
allocate device memory (their allocator owns the device, or their request
path must not call cudaMalloc).  It is called through the C ABI with
caller-owned device buffers, iterated to convergence, and compared with
gas_engine_pagerank_precision (which allocates its own buffers) and with the
FP64 oracle, within the precision-form tolerance used everywhere else: L1
distance <= 1e-6.  Two full runs in a row must both match, since every call
shares one scratch array; once the first call has loaded the array, further
calls must leave the device's free memory unchanged.

This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

import oracle
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


def _device_graph(el, torch):
    dev = torch.device("cuda", 0)
    off, src_csc, _ = edge_list_to_csr(el.nV, el.dst, el.src)
    return (torch.from_numpy(off).to(dev), torch.from_numpy(src_csc).to(dev),
            torch.from_numpy(el.out_degree()).to(dev))


def _run_noalloc(step, el, torch, max_iter=1000, free_check=False):
    dev = torch.device("cuda", 0)
    d_off, d_src, d_deg = _device_graph(el, torch)
    r = torch.full((el.nV,), 1.0 / el.nV, dtype=torch.float32, device=dev)
    r2 = torch.empty_like(r)
    l1 = torch.zeros(1, dtype=torch.float64, device=dev)
    l1_host = torch.zeros(1, dtype=torch.float64).pin_memory()
    stream = torch.cuda.current_stream().cuda_stream
    free0 = None
    for it in range(1, max_iter + 1):
        st = step(el.nV, el.nE, d_off.data_ptr(), d_src.data_ptr(), d_deg.data_ptr(),
                  r.data_ptr(), r2.data_ptr(), 0.85, l1.data_ptr(), stream)
        assert st == 0, _lib.load().gas_last_error()
        if free_check and free0 is None:
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
        r, r2 = r2, r
        l1_host.copy_(l1)
        if float(l1_host.item()) <= TOL:
            break
    else:
        raise AssertionError("no convergence")
    if free_check:
        torch.cuda.synchronize()
        # the steps after the first allocated nothing on the device
        assert torch.cuda.mem_get_info()[0] == free0
    return r.cpu().numpy(), it


def test_noalloc_first_call_with_no_graph_sets_up_the_device():
    """The call a pool-owning caller makes before its pool takes the device:
    no vertices, no edges, a zero residual."""
    torch = pytest.importorskip("torch")
    step = _bind(_lib.load())
    l1 = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    st = step(0, 0, None, None, None, None, None, 0.85, l1.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    assert st == 0, _lib.load().gas_last_error()
    assert float(l1.item()) == 0.0


def test_noalloc_step_matches_engine_twice():
    torch = pytest.importorskip("torch")
    step = _bind(_lib.load())
    el = EdgeList.rmat(14, 16, seed=4, symmetrize=False)
    eng = GASEngineGPU("pagerank")
    vd = initial_vertex_data("pagerank", el.nV, 0, el.out_degree())
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    ref, st = eng.pagerank_precision(0.85, TOL)
    eng.close()
    r64, _, _ = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, TOL)
    for k in range(2):
        ranks, it = _run_noalloc(step, el, torch, free_check=k == 1)
        assert np.abs(ranks.astype(np.float64) - ref.astype(np.float64)).sum() <= TOL
        assert np.abs(ranks.astype(np.float64) - r64).sum() <= TOL
        assert it == st.iterations


def test_noalloc_step_against_fp64_oracle_across_many_tiles():
    """A scale-18 graph (about 4.4 M merge-path items, hundreds of tiles and
    hub rows spanning many of them) against the FP64 oracle."""
    torch = pytest.importorskip("torch")
    step = _bind(_lib.load())
    el = EdgeList.rmat(18, 16, seed=9, symmetrize=False)
    r64, it64, _ = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, TOL)
    ranks, it = _run_noalloc(step, el, torch, free_check=True)
    d = np.abs(ranks.astype(np.float64) - r64)
    assert d.sum() <= TOL and abs(it - it64) <= 1


def test_noalloc_rejects_graphs_beyond_its_scratch():
    step = _bind(_lib.load())
    too_big = (1 << 29) - 100
    st = step(200, too_big, None, None, None, None, None, 0.85, None, None)
    assert st == 9  # GAS_ERR_TOO_LARGE
    assert b"scratch" in _lib.load().gas_last_error()
