"""CSR / CSC built on the device (stable LSD radix sort, gas_build.cu)
against the host build and the oracle's edgeListToCSR restatement: identical
offsets, neighbour order and permuted edge data, and identical runs."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, golden_names, load_golden
from graphreduce_gb300 import GASEngineGPU, GasError
from graphreduce_gb300.engine import initial_vertex_data
from graphreduce_gb300.graph import EdgeList

pytestmark = pytest.mark.gpu


def _engine(el, mode, program="sssp"):
    os.environ["GAS_GRAPH_BUILD"] = mode
    try:
        e = GASEngineGPU(program)
        vd = initial_vertex_data(program, el.nV, 0)
        e.setGraph(el.nV, vd, el.nE, el.weights if program == "sssp" else None,
                   el.src, el.dst)
    finally:
        del os.environ["GAS_GRAPH_BUILD"]
    return e


def _graphs():
    rng = np.random.default_rng(7)
    out = {}
    for name in golden_names():
        g = load_golden(name)
        out[name] = EdgeList(int(g["nV"]), g["src"], g["dst"], g["w"])
    with np.load(GOLDEN / "csr_ties.npz") as z:
        out["csr_ties"] = EdgeList(int(z["nV"]), z["src"], z["dst"], z["w"])
    el = EdgeList.rmat(14, 16, seed=3).with_uniform_weights(1, 64, 3)
    order = rng.permutation(el.nE)          # unsorted input, many ties per key
    out["rmat14_shuffled"] = EdgeList(el.nV, el.src[order], el.dst[order], el.weights[order])
    out["one_vertex"] = EdgeList(1, np.zeros(5, np.int32), np.zeros(5, np.int32),
                                 np.arange(5, dtype=np.int32))
    big = EdgeList.rmat(9, 8, seed=4, symmetrize=False).with_uniform_weights(1, 64, 5)
    # ids up to 2^20 + 3 (six 4-bit passes) with most vertices isolated
    out["sparse_ids"] = EdgeList((1 << 20) + 4, big.src * 2048 + 3, big.dst * 2048,
                                 big.weights)
    return out


NAMES = sorted(golden_names() + ["csr_ties", "rmat14_shuffled", "one_vertex", "sparse_ids"])


@pytest.fixture(scope="module")
def graphs(libgas):
    return _graphs()


@pytest.mark.parametrize("name", NAMES)
def test_device_build_equals_host_build(graphs, name):
    el = graphs[name]
    h = _engine(el, "host").graph_arrays()
    d = _engine(el, "device").graph_arrays()
    for k in h:
        np.testing.assert_array_equal(d[k], h[k], err_msg=k)
    off, out, perm = oracle.edge_list_to_csr(el.nV, el.src, el.dst)
    np.testing.assert_array_equal(d["csr_off"], off)
    np.testing.assert_array_equal(d["csr_dst"], out)
    np.testing.assert_array_equal(d["csr_w"], el.weights[perm])
    off, out, perm = oracle.edge_list_to_csr(el.nV, el.dst, el.src)
    np.testing.assert_array_equal(d["csc_off"], off)
    np.testing.assert_array_equal(d["csc_src"], out)
    np.testing.assert_array_equal(d["csc_w"], el.weights[perm])


def test_device_build_runs_bit_exact(graphs):
    el = graphs["rmat14_shuffled"]
    s = int(el.sample_sources(1, 3)[0])
    ref, it = oracle.sssp(el.nV, el.src, el.dst, el.weights, s)
    for mode in ("host", "device"):
        e = _engine(el, mode)
        vd = initial_vertex_data("sssp", el.nV, s)
        e.upload_vertex_data(vd)
        e.setActive(0, el.nV)
        st = e.run_schedule("push", max_iterations=el.nV + 2)
        out = np.empty(el.nV, np.int32)
        e.download_vertex_data(out)
        np.testing.assert_array_equal(out, ref)
        assert st.iterations == it


def test_device_build_rejects_bad_ids(libgas):
    el = EdgeList(4, np.array([0, 1, 2], np.int32), np.array([1, 2, 3], np.int32))
    bad = EdgeList(3, el.src, el.dst)            # dst 3 is outside [0, 3)
    os.environ["GAS_GRAPH_BUILD"] = "device"
    try:
        e = GASEngineGPU("cc")
        with pytest.raises(GasError) as ei:
            e.setGraph(3, initial_vertex_data("cc", 3), 3, None, bad.src, bad.dst)
        assert ei.value.status == 1
        e.setGraph(4, initial_vertex_data("cc", 4), 3, None, el.src, el.dst)  # still usable
    finally:
        del os.environ["GAS_GRAPH_BUILD"]
