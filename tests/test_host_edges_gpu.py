"""Edge arrays in pinned host memory read over NVLink-C2C
(gas_engine_set_edge_placement): the same results as with the edges in
HBM, for every schedule, both graph builds, and precision PageRank."""
import os

import numpy as np
import pytest

import oracle
from graphreduce_gb300 import GASEngineGPU
from graphreduce_gb300.engine import initial_vertex_data
from graphreduce_gb300.graph import EdgeList

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graph(libgas):
    return EdgeList.rmat(14, 16, seed=8).with_uniform_weights(1, 64, 3).with_grid_islands(16, 8)


@pytest.mark.parametrize("build", ["host", "device"])
@pytest.mark.parametrize("program", ["sssp", "cc", "bfs"])
def test_host_edges_bit_exact(graph, program, build):
    el = graph
    s = int(el.sample_sources(1, 5)[0])
    ref, it = {"sssp": lambda: oracle.sssp(el.nV, el.src, el.dst, el.weights, s),
               "cc": lambda: oracle.cc(el.nV, el.src, el.dst),
               "bfs": lambda: oracle.bfs(el.nV, el.src, el.dst, s)}[program]()
    os.environ["GAS_GRAPH_BUILD"] = build
    try:
        e = GASEngineGPU(program)
        e.set_edge_placement("host")
        vd = initial_vertex_data(program, el.nV, s)
        e.setGraph(el.nV, vd, el.nE, el.weights if program == "sssp" else None,
                   el.src, el.dst)
    finally:
        del os.environ["GAS_GRAPH_BUILD"]
    for schedule in ("auto", "push", "pull", "generic"):
        e.upload_vertex_data(initial_vertex_data(program, el.nV, s))
        e.setActive(*((s, s + 1) if program == "bfs" else (0, el.nV)))
        st = e.run_schedule(schedule, max_iterations=el.nV + 2)
        out = np.empty(el.nV, np.int32)
        e.download_vertex_data(out)
        np.testing.assert_array_equal(out, ref, err_msg=schedule)
        assert st.iterations == it
    d = GASEngineGPU(program)
    d.setGraph(el.nV, initial_vertex_data(program, el.nV, s), el.nE,
               el.weights if program == "sssp" else None, el.src, el.dst)
    a, b = e.graph_arrays(), d.graph_arrays()
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_host_edges_step_api_and_pagerank(graph):
    el = EdgeList.rmat(13, 16, seed=9, symmetrize=False)
    e = GASEngineGPU("pagerank")
    e.set_edge_placement("host")
    vd = initial_vertex_data("pagerank", el.nV, 0, el.out_degree())
    e.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    r, st = e.pagerank_precision(0.85, 1e-6)
    ref, _, _ = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, 1e-6)
    assert np.abs(r.astype(np.float64) - ref).sum() <= 1e-6
    # the reference's step loop (pagerank.cu:85-101) on host-resident edges
    e.setActive(0, el.nV)
    n = e.countActive()
    it = 0
    while n and it < 5:
        e.gather()
        e.apply()
        e.scatterActivate()
        n = e.nextIter()
        it += 1
    e.getResults()
    assert np.all(np.isfinite(vd["rank"])) and vd["rank"].max() > 0.15
