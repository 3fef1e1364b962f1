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


@pytest.mark.parametrize("L", [1, 5, 16, 32])
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
