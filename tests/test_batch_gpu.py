"""Batched engine on the GPU: multi-source BFS depths bit-exact against one
oracle BFS per (graph, source); multi-seed personalized PageRank within the
stated L1 tolerance of the FP64 oracle; the plain single-seed PPR; graph and
direct-launch modes identical; autotuner; caps and bad jobs."""
import os

import numpy as np
import pytest

import oracle
from graphreduce_gb300 import Batch, GASEngineGPU, GasError
from graphreduce_gb300.engine import initial_vertex_data
from graphreduce_gb300.graph import EdgeList

pytestmark = pytest.mark.gpu

# A lane stops when its L1 step is <= tol; PPR is a d-contraction in L1, so
# the lane is within d/(1-d) * tol of the fixed point (5.67e-6 at d = 0.85,
# tol = 1e-6), plus FP32 rounding of ranks that sum to at most 1.
PPR_TOL = 1e-6
PPR_L1 = 8e-6


def _graphs():
    path = EdgeList(6, np.arange(5, dtype=np.int32), np.arange(1, 6, dtype=np.int32))
    return [
        EdgeList.rmat(8, 8, seed=1),
        EdgeList.rmat(10, 16, seed=2, symmetrize=False),
        EdgeList.erdos_renyi(700, 2800, seed=3),
        EdgeList(5, np.zeros(0, np.int32), np.zeros(0, np.int32)),  # no edges
        path,
        EdgeList.rmat(9, 4, seed=4).with_grid_islands(6, 5),
        EdgeList.rmat(11, 32, seed=5),
    ]


@pytest.fixture(scope="module")
def batch():
    gs = _graphs()
    b = Batch()
    for el in gs:
        b.add_graph(el.nV, el.src, el.dst)
    b.build()
    yield b, gs
    b.close()


def _lanes(gs, L, seed, unused=0.1):
    rng = np.random.default_rng(seed)
    out = np.empty((len(gs), L), np.int32)
    for g, el in enumerate(gs):
        out[g] = rng.integers(0, el.nV, L)
        out[g, rng.random(L) < unused] = -1
    if L >= 3:
        out[0, :2] = out[0, 2]  # duplicate sources share a vertex's mask bits
    return out


def _check_bfs(b, gs, depth, srcs):
    for g, el in enumerate(gs):
        d = b.slice(depth, g)
        for l in range(srcs.shape[1]):
            s = int(srcs[g, l])
            if s < 0:
                assert np.all(d[:, l] == -1)
                continue
            ref, _ = oracle.bfs(el.nV, el.src, el.dst, s)
            np.testing.assert_array_equal(d[:, l], ref, err_msg=f"graph {g} lane {l}")


def _check_ppr(b, gs, rank, seeds, tol=PPR_L1):
    worst = 0.0
    for g, el in enumerate(gs):
        r = b.slice(rank, g)
        for l in range(seeds.shape[1]):
            s = int(seeds[g, l])
            if s < 0:
                assert np.all(r[:, l] == 0)
                continue
            ref, _, _ = oracle.ppr_fp64(el.nV, el.src, el.dst, s, 0.85, 1e-13)
            err = np.abs(r[:, l].astype(np.float64) - ref).sum()
            worst = max(worst, err)
            assert err <= tol, f"graph {g} lane {l}: L1 {err:.3e}"
    return worst


@pytest.mark.parametrize("L", [1, 16, 32])
def test_multi_source_bfs_bit_exact(batch, L):
    b, gs = batch
    srcs = _lanes(gs, L, seed=L)
    res = b.run(bfs_sources=srcs)
    assert res.rank is None
    _check_bfs(b, gs, res.depth, srcs)
    assert res.stats.graph_launches == 1
    assert res.stats.bfs_edges > 0


@pytest.mark.parametrize("L", [1, 4, 5, 8, 12, 16, 20, 32])
def test_multi_seed_ppr_within_tolerance(batch, L):
    b, gs = batch
    seeds = _lanes(gs, L, seed=100 + L)
    res = b.run(ppr_seeds=seeds, tol=PPR_TOL)
    assert res.depth is None
    assert res.stats.ppr_residual <= PPR_TOL
    assert all(res.stats.ppr_lane_residual[l] <= PPR_TOL for l in range(L))
    _check_ppr(b, gs, res.rank, seeds)


def test_both_in_one_launch_and_repeatable(batch):
    b, gs = batch
    srcs, seeds = _lanes(gs, 16, 7), _lanes(gs, 16, 8)
    a = b.run(bfs_sources=srcs, ppr_seeds=seeds, tol=PPR_TOL)
    assert a.stats.graph_launches == 1
    _check_bfs(b, gs, a.depth, srcs)
    _check_ppr(b, gs, a.rank, seeds)
    again = b.run(bfs_sources=srcs, ppr_seeds=seeds, tol=PPR_TOL)
    np.testing.assert_array_equal(a.depth, again.depth)
    np.testing.assert_array_equal(a.rank, again.rank)      # deterministic sums
    other = _lanes(gs, 16, 9)                               # same graph, new sources
    c = b.run(bfs_sources=other, ppr_seeds=seeds, tol=PPR_TOL)
    _check_bfs(b, gs, c.depth, other)


@pytest.mark.parametrize("P", [64, 100, 2048])
def test_piece_sizes_agree(batch, P):
    b, gs = batch
    seeds = _lanes(gs, 8, 11)
    res = b.run(ppr_seeds=seeds, tol=PPR_TOL, piece_edges=P)
    assert res.stats.piece_edges == P
    _check_ppr(b, gs, res.rank, seeds)


def test_autotuner_picks_a_candidate(batch):
    b, gs = batch
    P, ms = b.tune(16)
    assert P in (64, 128, 256, 512, 1024, 2048) and ms > 0
    seeds = _lanes(gs, 16, 12)
    res = b.run(ppr_seeds=seeds, tol=PPR_TOL)
    assert res.stats.piece_edges == P
    _check_ppr(b, gs, res.rank, seeds)


def test_direct_launch_mode_identical(batch):
    b, gs = batch
    srcs, seeds = _lanes(gs, 16, 13), _lanes(gs, 16, 14)
    g = b.run(bfs_sources=srcs, ppr_seeds=seeds, tol=PPR_TOL, piece_edges=256)
    os.environ["GAS_HOST_LOOP"] = "1"
    try:
        d = b.run(bfs_sources=srcs, ppr_seeds=seeds, tol=PPR_TOL, piece_edges=256)
    finally:
        del os.environ["GAS_HOST_LOOP"]
    assert d.stats.graph_launches == 0
    np.testing.assert_array_equal(g.depth, d.depth)
    np.testing.assert_array_equal(g.rank, d.rank)
    assert g.stats.ppr_iterations == d.stats.ppr_iterations
    assert g.stats.bfs_iterations == d.stats.bfs_iterations


def test_ppr_linearity_gives_global_pagerank():
    """Mean of the PPR vectors over every seed = normalised PageRank."""
    el = EdgeList.erdos_renyi(32, 160, seed=21)
    b = Batch()
    b.add_graph(el.nV, el.src, el.dst)
    b.build()
    # tol 1e-7 is near the FP32 floor of ranks of order 1/32; each lane is
    # then within d/(1-d) * 1e-7 = 5.7e-7 of its fixed point in L1
    res = b.run(ppr_seeds=np.arange(32, dtype=np.int32)[None, :], tol=1e-7)
    glob, _, _ = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, 1e-13, 100000)
    mean = res.rank.astype(np.float64).mean(axis=1)
    assert np.abs(mean - glob).sum() <= 1e-6
    b.close()


def test_plain_ppr_matches_oracle():
    el = EdgeList.rmat(12, 16, seed=6, symmetrize=False)
    eng = GASEngineGPU("pagerank")
    vd = initial_vertex_data("pagerank", el.nV, 0, el.out_degree())
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    for s in (0, 17, el.nV - 1):
        r, st = eng.ppr_precision(s, 0.85, PPR_TOL)
        ref, _, _ = oracle.ppr_fp64(el.nV, el.src, el.dst, s, 0.85, 1e-13)
        assert st.residual <= PPR_TOL
        assert np.abs(r.astype(np.float64) - ref).sum() <= PPR_L1
    # the global form is unchanged by the personalised one
    g, st = eng.pagerank_precision(0.85, 1e-6)
    ref, _, _ = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, 1e-6)
    assert np.abs(g.astype(np.float64) - ref).sum() <= 1e-6
    with pytest.raises(GasError):
        eng.ppr_precision(el.nV)
    eng.close()


def test_caps_and_bad_jobs(batch):
    b, gs = batch
    srcs = _lanes(gs, 4, 15)
    with pytest.raises(GasError) as ei:
        b.run(bfs_sources=srcs, max_bfs_levels=1)
    assert ei.value.status == 4
    with pytest.raises(GasError) as ei:
        b.run(ppr_seeds=srcs, tol=1e-9, max_ppr_iterations=2)
    assert ei.value.status == 4
    bad = srcs.copy()
    bad[3, 0] = gs[3].nV              # graph 3 has 5 vertices
    with pytest.raises(GasError) as ei:
        b.run(bfs_sources=bad)
    assert ei.value.status == 1
    with pytest.raises(GasError):
        b.run(bfs_sources=np.zeros((len(gs), 33), np.int32))
    with pytest.raises(ValueError):
        b.run(bfs_sources=np.zeros((2, 4), np.int32))
    # the batch is still usable after the errors
    res = b.run(bfs_sources=srcs)
    _check_bfs(b, gs, res.depth, srcs)


def test_device_result_pointers(batch):
    torch = pytest.importorskip("torch")
    b, gs = batch
    srcs, seeds = _lanes(gs, 16, 16), _lanes(gs, 16, 17)
    V = b.num_vertices
    dd = torch.empty((V, 16), dtype=torch.int32, device="cuda")
    rd = torch.empty((V, 16), dtype=torch.float32, device="cuda")
    b.run(bfs_sources=srcs, ppr_seeds=seeds, tol=PPR_TOL, depth_out=dd.data_ptr(),
          rank_out=rd.data_ptr())
    host = b.run(bfs_sources=srcs, ppr_seeds=seeds, tol=PPR_TOL)
    np.testing.assert_array_equal(dd.cpu().numpy(), host.depth)
    np.testing.assert_array_equal(rd.cpu().numpy(), host.rank)


# ---------------------------------------------------------------------------
# multi-source SSSP lanes
# ---------------------------------------------------------------------------
SSSP_INF = 2**31 - 1 - 100000


def _weighted_graphs():
    gs = _graphs()
    out = []
    for k, el in enumerate(gs):
        if k == 1:
            out.append((el, None))  # an unweighted graph among weighted ones: weight 1
        else:
            w = el.with_uniform_weights(1, 64, 10 + k).weights if el.nE else np.zeros(0, np.int32)
            out.append((el, w))
    return out


@pytest.fixture(scope="module")
def wbatch():
    gw = _weighted_graphs()
    b = Batch()
    for el, w in gw:
        b.add_graph(el.nV, el.src, el.dst, w)
    b.build()
    yield b, gw
    b.close()


def _check_sssp(b, gw, dist, srcs, stats=None):
    for g, (el, w) in enumerate(gw):
        d = b.slice(dist, g)
        ww = w if w is not None else np.ones(el.nE, np.int32)
        for l in range(srcs.shape[1]):
            s = int(srcs[g, l])
            if s < 0:
                assert np.all(d[:, l] == SSSP_INF)
                continue
            ref, rit = oracle.sssp(el.nV, el.src, el.dst, ww, s)
            np.testing.assert_array_equal(d[:, l], ref, err_msg=f"graph {g} lane {l}")


@pytest.mark.parametrize("L", [1, 5, 8, 32])
def test_multi_source_sssp_bit_exact(wbatch, L):
    b, gw = wbatch
    srcs = _lanes([el for el, _ in gw], L, seed=200 + L)
    res = b.run(sssp_sources=srcs)
    assert res.depth is None and res.rank is None
    _check_sssp(b, gw, res.dist, srcs)
    assert res.stats.sssp_edges > 0 and res.stats.graph_launches == 1


def test_sssp_lane_iterations_equal_single_source_runs():
    """One graph, 8 lanes: every lane runs as many pushes as one SSSP from its
    source through the engine (and as the oracle's rounds)."""
    el = EdgeList.rmat(11, 16, seed=2).with_uniform_weights(1, 64, 3)
    srcs = el.sample_sources(8, 2).astype(np.int32)
    b = Batch()
    b.add_graph(el.nV, el.src, el.dst, el.weights)
    b.build()
    res = b.run(sssp_sources=srcs[None, :])
    eng = GASEngineGPU("sssp")
    eng.setGraph(el.nV, initial_vertex_data("sssp", el.nV, int(srcs[0])), el.nE, el.weights,
                 el.src, el.dst)
    for l, s in enumerate(srcs):
        eng.upload_vertex_data(initial_vertex_data("sssp", el.nV, int(s)))
        eng.setActive(0, el.nV)
        st = eng.run_schedule("auto", max_iterations=el.nV + 2)
        out = np.empty(el.nV, np.int32)
        eng.download_vertex_data(out)
        np.testing.assert_array_equal(res.dist[:, l], out)
        assert res.stats.sssp_lane_iterations[l] == st.iterations, f"lane {l}"
    assert res.stats.sssp_iterations == max(res.stats.sssp_lane_iterations[l] for l in range(8))
    eng.close()
    b.close()


def test_all_three_kinds_in_one_launch(wbatch):
    b, gw = wbatch
    gs = [el for el, _ in gw]
    bs, ss, ps = _lanes(gs, 8, 31), _lanes(gs, 8, 32), _lanes(gs, 4, 33)
    res = b.run(bfs_sources=bs, sssp_sources=ss, ppr_seeds=ps, tol=PPR_TOL)
    assert res.stats.graph_launches == 1
    _check_sssp(b, gw, res.dist, ss)
    _check_ppr(b, gs, res.rank, ps)
    for g, el in enumerate(gs):
        d = b.slice(res.depth, g)
        for l in range(8):
            s = int(bs[g, l])
            if s >= 0:
                ref, _ = oracle.bfs(el.nV, el.src, el.dst, s)
                np.testing.assert_array_equal(d[:, l], ref)


def test_sssp_direct_launch_mode_identical(wbatch):
    b, gw = wbatch
    ss = _lanes([el for el, _ in gw], 8, 41)
    g = b.run(sssp_sources=ss)
    os.environ["GAS_HOST_LOOP"] = "1"
    try:
        d = b.run(sssp_sources=ss)
    finally:
        del os.environ["GAS_HOST_LOOP"]
    assert d.stats.graph_launches == 0
    np.testing.assert_array_equal(g.dist, d.dist)
    assert g.stats.sssp_iterations == d.stats.sssp_iterations
    assert list(g.stats.sssp_lane_iterations) == list(d.stats.sssp_lane_iterations)


def test_sssp_cap_and_device_output(wbatch):
    torch = pytest.importorskip("torch")
    b, gw = wbatch
    ss = _lanes([el for el, _ in gw], 8, 51)
    with pytest.raises(GasError) as ei:
        b.run(sssp_sources=ss, max_sssp_iterations=1)
    assert ei.value.status == 4
    dd = torch.empty((b.num_vertices, 8), dtype=torch.int32, device="cuda")
    b.run(sssp_sources=ss, dist_out=dd.data_ptr())
    host = b.run(sssp_sources=ss)
    np.testing.assert_array_equal(dd.cpu().numpy(), host.dist)
    _check_sssp(b, gw, host.dist, ss)


def test_profiled_pushes_same_results(wbatch):
    b, gw = wbatch
    gs = [el for el, _ in gw]
    bs, ss = _lanes(gs, 8, 61), _lanes(gs, 8, 62)
    ref = b.run(bfs_sources=bs, sssp_sources=ss)
    b.set_profiling(True)
    try:
        b.profile(reset=True)
        got = b.run(bfs_sources=bs, sssp_sources=ss)
        p = b.profile()
    finally:
        b.set_profiling(False)
    np.testing.assert_array_equal(got.depth, ref.depth)
    np.testing.assert_array_equal(got.dist, ref.dist)
    # at most one push per BFS level and per SSSP iteration, none when off
    it = got.stats.bfs_iterations + got.stats.sssp_iterations
    assert 0 < p.push_launches <= it + 2
    assert p.push_ms > 0 and p.push_bytes > 0
    b.run(bfs_sources=bs)
    assert b.profile().push_launches == 0
