"""Pins the oracle (oracle/gas_oracle.c) to the reference's own outputs.

The golden vectors were produced by the reference's refgas.h and graphio.cpp
(tests/golden/make_golden.py).  Integer programs must match bit for bit,
iteration counts included; PageRank (reference form) may differ in the last
ulp because refgas orders equal keys with an unstable std::sort, so it is
held to the reference's own regression rule (checkPageRank.py:77-83) and a
relative bound.
"""
import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden

CASES = golden_names()


def pr_histogram_ok(test, gold):
    """checkPageRank.py:40-83: fraction of |diff| per decade must stay under
    [1, 1e-2, 5e-3, 5e-4, 5e-5, 5e-6, 0] for bins [1e-4 .. 10]."""
    tol_vals = [1e-4, 1e-3, 1e-2, 0.1, 1, 10]
    allowed = [1.0, 1e-2, 5e-3, 5e-4, 5e-5, 5e-6, 0]
    diff = np.abs(test.astype(np.float64) - gold.astype(np.float64))
    counts = np.zeros(len(tol_vals) + 1)
    for dv in diff:
        pos = len(tol_vals) - 1
        while pos >= 0 and dv < tol_vals[pos]:
            pos -= 1
        counts[pos + 1] += 1
    frac = counts / max(1, len(diff))
    return all(f <= a for f, a in zip(frac, allowed))


@pytest.fixture(scope="module", autouse=True)
def _built(libgas):
    return libgas


@pytest.mark.parametrize("name", CASES)
def test_oracle_bfs_sssp_cc_match_reference(name):
    g = load_golden(name)
    nV = int(g["nV"])
    src, dst, w, s = g["src"], g["dst"], g["w"], int(g["source"])
    depth, it = oracle.bfs(nV, src, dst, s)
    assert it == g["bfs_iters"]
    np.testing.assert_array_equal(depth, g["bfs_depth"])
    dist, it = oracle.sssp(nV, src, dst, w, s)
    assert it == g["sssp_iters"]
    np.testing.assert_array_equal(dist, g["sssp_dist"])
    lab, it = oracle.cc(nV, src, dst)
    assert it == g["cc_iters"]
    np.testing.assert_array_equal(lab, g["cc_label"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_pagerank_matches_reference(name):
    g = load_golden(name)
    nV = int(g["nV"])
    rank, it = oracle.pagerank(nV, g["src"], g["dst"])
    assert it == g["pr_iters"]
    gold = g["pr_rank"]
    assert pr_histogram_ok(rank, gold)
    np.testing.assert_allclose(rank, gold, rtol=2e-6, atol=1e-6)


def test_oracle_csr_matches_reference_edge_list_to_csr():
    with np.load(oracle.HERE.parent / "tests" / "golden" / "csr_ties.npz") as z:
        nV, s, d = int(z["nV"]), z["src"], z["dst"]
        ref_off, ref_out, ref_perm = z["ref_off"], z["ref_out"], z["ref_perm"]
    off, out, perm = oracle.edge_list_to_csr(nV, s, d)
    np.testing.assert_array_equal(off, ref_off)
    # the same multiset of (dst, edge id) per source; stable order within one
    for v in range(nV):
        a, b = off[v], off[v + 1]
        assert sorted(zip(out[a:b], perm[a:b])) == sorted(zip(ref_out[a:b], ref_perm[a:b]))
        assert list(perm[a:b]) == sorted(perm[a:b])
    np.testing.assert_array_equal(out, d[perm])


def _numpy_pagerank(nV, src, dst, d=0.85, tol=1e-6, max_iter=1000):
    outdeg = np.bincount(src, minlength=nV).astype(np.float64)
    r = np.full(nV, 1.0 / nV)
    for it in range(1, max_iter + 1):
        contrib = np.where(outdeg > 0, r / np.maximum(outdeg, 1), 0.0)
        rn = (1 - d) / nV + d * np.bincount(dst, weights=contrib[src], minlength=nV)
        l1 = np.abs(rn - r).sum()
        r = rn
        if l1 <= tol:
            return r, it, l1
    raise AssertionError("no convergence")


@pytest.mark.parametrize("name", ["rmat10_directed", "er1000_directed", "directed_dag",
                                  "rmat10_sym"])
def test_fp64_pagerank_oracle_against_numpy(name):
    g = load_golden(name)
    nV = int(g["nV"])
    r, it, l1 = oracle.pagerank_fp64(nV, g["src"], g["dst"])
    rn, itn, l1n = _numpy_pagerank(nV, g["src"], g["dst"])
    assert it == itn
    assert l1 <= 1e-6
    np.testing.assert_allclose(r, rn, rtol=1e-12, atol=1e-15)
    # one step from the fixed point moves by the last residual at most
    r2, l1s = oracle.pagerank_fp64_step(nV, g["src"], g["dst"], r)
    assert l1s <= l1 * 0.86 + 1e-15


def test_oracle_rejects_bad_source():
    with pytest.raises(RuntimeError):
        oracle.bfs(3, np.array([0, 1]), np.array([1, 2]), 5)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference not built here")
@pytest.mark.parametrize("scale,seed", [(9, 31), (11, 32)])
def test_oracle_against_live_reference(scale, seed):
    """Fresh random graphs through both the reference and the oracle."""
    from graphreduce_gb300.graph import EdgeList
    el = EdgeList.rmat(scale, 8, seed=seed).with_uniform_weights(1, 64, 3)
    s = int(el.sample_sources(1, seed)[0])
    a, ia = oracle.sssp(el.nV, el.src, el.dst, el.weights, s)
    b, ib = oracle.ref_sssp(el.nV, el.src, el.dst, el.weights, s)
    assert ia == ib
    np.testing.assert_array_equal(a, b)
    a, ia = oracle.cc(el.nV, el.src, el.dst)
    b, ib = oracle.ref_cc(el.nV, el.src, el.dst)
    assert ia == ib
    np.testing.assert_array_equal(a, b)
    a, ia = oracle.bfs(el.nV, el.src, el.dst, s)
    b, ib = oracle.ref_bfs(el.nV, el.src, el.dst, s)
    assert ia == ib
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("scale,ef,sym,seed", [(9, 16, True, 2), (11, 8, False, 4),
                                               (12, 16, True, 1)])
def test_oracle_generators_match_library(scale, ef, sym, seed):
    """The oracle's own input generators (what the CPU baseline builds its
    workload with, never loading the product library) give the product
    library's graphs, islands, weights and sources exactly."""
    from graphreduce_gb300.graph import EdgeList
    el = EdgeList.rmat(scale, ef, seed=seed, symmetrize=sym)
    nV, s, d = oracle.rmat(scale, ef, seed=seed, symmetrize=sym)
    assert nV == el.nV
    np.testing.assert_array_equal(s, el.src)
    np.testing.assert_array_equal(d, el.dst)
    isl = el.with_grid_islands(12, 5)
    nV2, s2, d2 = oracle.with_grid_islands(nV, s, d, 12, 5)
    assert nV2 == isl.nV
    np.testing.assert_array_equal(s2, isl.src)
    np.testing.assert_array_equal(d2, isl.dst)
    np.testing.assert_array_equal(oracle.uniform_weights(s, d, 1, 64, 3),
                                  el.with_uniform_weights(1, 64, 3).weights)
    np.testing.assert_array_equal(oracle.sample_sources(nV, s, d, 8, seed),
                                  el.sample_sources(8, seed))


def test_oracle_results_do_not_depend_on_thread_count():
    nV, s, d = oracle.rmat(12, 16, seed=5, symmetrize=True)
    w = oracle.uniform_weights(s, d, 1, 64, 3)
    src = int(oracle.sample_sources(nV, s, d, 1, 5)[0])
    nd, sd, dd = oracle.rmat(12, 16, seed=6, symmetrize=False)
    runs = []
    before = oracle.threads()
    try:
        for th in (1, 3, 8):
            oracle.set_threads(th)
            runs.append((oracle.sssp(nV, s, d, w, src), oracle.cc(nV, s, d),
                         oracle.bfs(nV, s, d, src), oracle.pagerank(nd, sd, dd),
                         oracle.pagerank_fp64(nd, sd, dd), oracle.edge_list_to_csr(nV, d, s)))
    finally:
        oracle.set_threads(before)
    for other in runs[1:]:
        for a, b in zip(runs[0], other):
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y)


def test_oracle_graph_handle_matches_per_call_runs():
    nV, s, d = oracle.rmat(11, 16, seed=8, symmetrize=True)
    w = oracle.uniform_weights(s, d, 1, 64, 3)
    srcs = oracle.sample_sources(nV, s, d, 3, 8)
    g = oracle.Graph(nV, s, d)
    for x in srcs:
        a, ia = g.sssp(w, x)
        b, ib = oracle.sssp(nV, s, d, w, x)
        assert ia == ib
        np.testing.assert_array_equal(a, b)
        a, ia = g.bfs(x)
        b, ib = oracle.bfs(nV, s, d, x)
        assert ia == ib
        np.testing.assert_array_equal(a, b)
    a, ia = g.cc()
    b, ib = oracle.cc(nV, s, d)
    assert ia == ib
    np.testing.assert_array_equal(a, b)
    a, ia, la = g.pagerank_fp64()
    b, ib, lb = oracle.pagerank_fp64(nV, s, d)
    assert ia == ib and la == lb
    np.testing.assert_array_equal(a, b)
    a, ia, _ = g.ppr_fp64(int(srcs[0]), tol=1e-10)
    b, ib, _ = oracle.ppr_fp64(nV, s, d, int(srcs[0]), tol=1e-10)
    assert ia == ib
    np.testing.assert_array_equal(a, b)
    g.close()
