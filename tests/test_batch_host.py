"""Batched engine, host side (no kernel launches): graph bookkeeping and
argument checks of gas_batch_*, and the FP64 personalized-PageRank oracle
pinned to the global PageRank oracle by linearity."""
import numpy as np
import pytest

import oracle
from graphreduce_gb300 import Batch, GasError
from graphreduce_gb300.graph import EdgeList


@pytest.fixture(scope="module", autouse=True)
def _built(libgas):
    return libgas


def test_union_bookkeeping():
    b = Batch()
    a = EdgeList.rmat(6, 4, seed=1)
    c = EdgeList.erdos_renyi(50, 200, seed=2)
    assert b.add_graph(a.nV, a.src, a.dst) == 0
    assert b.add_graph(7, np.zeros(0, np.int32), np.zeros(0, np.int32)) == 1
    assert b.add_graph(c.nV, c.src, c.dst) == 2
    assert b.num_graphs == 3
    assert b.num_vertices == a.nV + 7 + c.nV
    assert b.num_edges == a.nE + c.nE
    assert [b.vertex_offset(g) for g in range(4)] == [0, a.nV, a.nV + 7, b.num_vertices]
    assert b.vertex_offset(4) == -1
    b.close()


def test_add_graph_rejects_bad_edges_and_run_before_build():
    b = Batch()
    with pytest.raises(GasError) as ei:
        b.add_graph(3, np.array([0, 3], np.int32), np.array([1, 1], np.int32))
    assert ei.value.status == 1
    with pytest.raises(GasError) as ei:
        b.add_graph(-1, np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert ei.value.status == 1
    assert b.num_graphs == 0
    b.add_graph(2, np.array([0], np.int32), np.array([1], np.int32))
    with pytest.raises(GasError) as ei:
        b.run(bfs_sources=np.zeros((1, 1), np.int32))
    assert ei.value.status == 6
    with pytest.raises(GasError) as ei:
        b.tune(4)
    assert ei.value.status == 6
    b.close()


def test_weighted_graphs_bookkeeping_and_checks():
    b = Batch()
    a = EdgeList.rmat(6, 4, seed=1)
    assert b.add_graph(a.nV, a.src, a.dst) == 0            # weighs 1 per edge
    w = np.arange(a.nE, dtype=np.int32) % 7 + 1
    assert b.add_graph(a.nV, a.src, a.dst, w) == 1
    assert b.num_edges == 2 * a.nE
    with pytest.raises(ValueError):
        b.add_graph(a.nV, a.src, a.dst, w[:-1])
    for bad in (-1, 100001):
        wb = w.copy()
        wb[3] = bad
        with pytest.raises(GasError) as ei:
            b.add_graph(a.nV, a.src, a.dst, wb)
        assert ei.value.status == 1
    with pytest.raises(GasError) as ei:                     # not built yet
        b.run(sssp_sources=np.zeros((2, 1), np.int32))
    assert ei.value.status == 6
    with pytest.raises(ValueError):
        b.run(sssp_sources=np.zeros((3, 1), np.int32))      # 2 graphs
    b.close()


def test_ppr_oracle_linearity_and_mass():
    el = EdgeList.erdos_renyi(40, 200, seed=3)
    glob, _, _ = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, 1e-14, 100000)
    acc = np.zeros(el.nV)
    for s in range(el.nV):
        r, it, l1 = oracle.ppr_fp64(el.nV, el.src, el.dst, s, 0.85, 1e-14)
        assert l1 <= 1e-14 and it > 0
        assert r.sum() <= 1.0 + 1e-12 and r.min() >= 0
        assert r[s] >= 1 - 0.85 - 1e-12
        acc += r
    assert np.abs(acc / el.nV - glob).max() <= 1e-13


def test_ppr_oracle_rejects_bad_seed():
    el = EdgeList.erdos_renyi(10, 20, seed=4)
    with pytest.raises(Exception):
        oracle.ppr_fp64(el.nV, el.src, el.dst, el.nV)
