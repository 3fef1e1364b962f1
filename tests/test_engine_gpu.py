"""Parity of the CUDA engine (through the C ABI) with the reference's outputs
and the oracle.  Integer programs: bit-exact, iteration counts included.
PageRank (reference form): the ordered-fold schedule is bit-exact with the
oracle; the load-balanced gather differs only in float summation order and
is held to checkPageRank.py's rule and rtol 1e-5.  Precision-form PageRank:
L1 error <= 1e-6 against the FP64 oracle."""
import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden
from graphreduce_gb300 import GASEngineGPU, GasError, run_program
from graphreduce_gb300.engine import initial_vertex_data
from graphreduce_gb300.graph import EdgeList
from test_oracle import pr_histogram_ok

pytestmark = pytest.mark.gpu

CASES = golden_names()
INT_PROGRAMS = ["bfs", "sssp", "cc"]
KEY = {"bfs": ("bfs_depth", "bfs_iters"), "sssp": ("sssp_dist", "sssp_iters"),
       "cc": ("cc_label", "cc_iters")}


@pytest.fixture(scope="module", autouse=True)
def _built(libgas):
    return libgas


def golden_el(g):
    return EdgeList(int(g["nV"]), g["src"], g["dst"], g["w"])


@pytest.mark.parametrize("schedule", ["step", "generic", "ordered", "auto", "push", "pull"])
@pytest.mark.parametrize("program", INT_PROGRAMS)
@pytest.mark.parametrize("name", CASES)
def test_integer_programs_match_reference(name, program, schedule):
    g = load_golden(name)
    vd, it = run_program(program, golden_el(g), int(g["source"]), schedule)
    out, iters = KEY[program]
    np.testing.assert_array_equal(vd, g[out])
    assert it == g[iters]


@pytest.mark.parametrize("name", CASES)
def test_pagerank_ordered_is_bitexact_with_oracle(name):
    g = load_golden(name)
    el = golden_el(g)
    vd, it = run_program("pagerank", el, 0, "ordered")
    rank, oit = oracle.pagerank(el.nV, el.src, el.dst)
    np.testing.assert_array_equal(vd["rank"], rank)
    assert it == oit
    assert pr_histogram_ok(vd["rank"], g["pr_rank"])


@pytest.mark.parametrize("schedule", ["step", "generic"])
@pytest.mark.parametrize("name", CASES)
def test_pagerank_load_balanced_within_tolerance(name, schedule):
    g = load_golden(name)
    vd, it = run_program("pagerank", golden_el(g), 0, schedule)
    assert pr_histogram_ok(vd["rank"], g["pr_rank"])
    np.testing.assert_allclose(vd["rank"], g["pr_rank"], rtol=1e-5, atol=1e-5)
    assert abs(it - int(g["pr_iters"])) <= 1


@pytest.mark.parametrize("scale,ef,seed", [(14, 16, 41), (16, 16, 42), (15, 4, 43)])
def test_random_rmat_against_oracle(scale, ef, seed):
    el = EdgeList.rmat(scale, ef, seed=seed).with_uniform_weights(1, 64, 3)
    s = int(el.sample_sources(1, seed)[0])
    for program in INT_PROGRAMS:
        if program == "bfs":
            ref, rit = oracle.bfs(el.nV, el.src, el.dst, s)
        elif program == "sssp":
            ref, rit = oracle.sssp(el.nV, el.src, el.dst, el.weights, s)
        else:
            ref, rit = oracle.cc(el.nV, el.src, el.dst)
        for schedule in ("step", "generic", "auto", "push", "pull"):
            vd, it = run_program(program, el, s, schedule)
            np.testing.assert_array_equal(vd, ref, err_msg=f"{program}/{schedule}")
            assert it == rit, (program, schedule)


def test_cc_with_grid_islands_against_oracle():
    el = EdgeList.rmat(12, 16, seed=2).with_grid_islands(16, 32)
    ref, rit = oracle.cc(el.nV, el.src, el.dst)
    for schedule in ("generic", "auto", "push", "pull"):
        vd, it = run_program("cc", el, 0, schedule)
        np.testing.assert_array_equal(vd, ref)
        assert it == rit and it >= 62      # a 32x32 grid needs 62 label hops


def test_fast_schedules_at_scale_against_oracle():
    """Thousands of compaction blocks (R-MAT scale 19 plus 512 grid islands,
    1M vertices), blocks whose changes come and go between iterations, and
    the same engine run again: CC and SSSP under the learned and the fixed
    schedule, bit-exact with the oracle."""
    from graphreduce_gb300.learn import DATA, MLP
    model = MLP.load(DATA / "schedule_head.npz")
    base = EdgeList.rmat(19, 16, seed=7)
    cases = [("cc", base.with_grid_islands(512, 32), 0)]
    w = base.with_uniform_weights(1, 64, 8)
    cases.append(("sssp", w, int(w.sample_sources(1, 9)[0])))
    for program, el, s in cases:
        if program == "cc":
            ref, rit = oracle.cc(el.nV, el.src, el.dst)
        else:
            ref, rit = oracle.sssp(el.nV, el.src, el.dst, el.weights, s)
        eng = GASEngineGPU(program)
        eng.setGraph(el.nV, initial_vertex_data(program, el.nV, s), el.nE,
                     el.weights if program == "sssp" else None, el.src, el.dst)
        eng.set_schedule_model(model)
        for schedule in ("learned", "auto", "learned"):
            eng.upload_vertex_data(initial_vertex_data(program, el.nV, s))
            eng.setActive(0, el.nV)
            st = eng.run_schedule(schedule, max_iterations=el.nV + 2)
            out = np.empty(el.nV, np.int32)
            eng.download_vertex_data(out)
            np.testing.assert_array_equal(out, ref, err_msg=f"{program}/{schedule}")
            assert st.iterations == rit, (program, schedule)
        eng.close()


def test_bfs_bottom_up_levels_at_scale():
    """BFS from a source in the R-MAT part of a 1M-vertex graph (scale 19 +
    512 grid islands the source cannot reach): top-down only, bottom-up
    only, and the direction rule (AUTO, and LEARNED, which takes the same
    rule for BFS) give the oracle's depths and level count; the rule
    switches to bottom-up for the heavy levels and back."""
    el = EdgeList.rmat(19, 16, seed=7).with_grid_islands(512, 32)
    s = int(EdgeList.rmat(19, 16, seed=7).sample_sources(1, 9)[0])
    ref, rit = oracle.bfs(el.nV, el.src, el.dst, s)
    from graphreduce_gb300.learn import DATA, MLP
    eng = GASEngineGPU("bfs")
    eng.setGraph(el.nV, initial_vertex_data("bfs", el.nV), el.nE, None, el.src, el.dst)
    eng.set_schedule_model(MLP.load(DATA / "schedule_head.npz"))
    for schedule in ("push", "pull", "auto", "learned"):
        eng.upload_vertex_data(initial_vertex_data("bfs", el.nV))
        eng.setActive(s, s + 1)
        st = eng.run_schedule(schedule, max_iterations=el.nV + 2)
        out = np.empty(el.nV, np.int32)
        eng.download_vertex_data(out)
        np.testing.assert_array_equal(out, ref, err_msg=schedule)
        assert st.iterations == rit, schedule
        if schedule in ("auto", "learned"):
            assert st.pull_iters > 0 and st.push_iters > 0, (st.push_iters, st.pull_iters)
    eng.close()


@pytest.mark.parametrize("scale,seed", [(12, 4), (14, 4)])
def test_pagerank_precision_against_fp64_oracle(scale, seed):
    el = EdgeList.rmat(scale, 16, seed=seed, symmetrize=False)
    ref, rit, rl1 = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, 1e-6)
    eng = GASEngineGPU("pagerank")
    vd = initial_vertex_data("pagerank", el.nV, 0, el.out_degree())
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    ranks, st = eng.pagerank_precision(0.85, 1e-6)
    err = np.abs(ranks.astype(np.float64) - ref)
    assert err.sum() <= 1e-6, err.sum()          # L1 error vs FP64
    assert err.max() <= 1e-7
    assert abs(st.iterations - rit) <= 1
    assert st.residual <= 1e-6


def _tile_spanning_graphs():
    """Rows that span many merge-path tiles (2,048 path items each): a hub
    with 200,000 in-edges (about 100 tiles, several 32-record fix-up rounds),
    one more at the last vertex (the path's last tile), a scattered ring,
    and thousands of rows without in-edges; a graph with no edges; one
    vertex with a self-loop."""
    nV = 300_000
    a = np.arange(1, 200_001, dtype=np.int32)
    b = np.arange(200_001, 270_001, dtype=np.int32)
    v = np.arange(0, nV, 3, dtype=np.int64)
    src = np.concatenate([a, b, v.astype(np.int32)])
    dst = np.concatenate([np.zeros_like(a), np.full_like(b, nV - 1),
                          ((v * 7 + 3) % nV).astype(np.int32)])
    return [EdgeList(nV, src, dst),
            EdgeList(1000, np.zeros(0, np.int32), np.zeros(0, np.int32)),
            EdgeList(1, np.zeros(1, np.int32), np.zeros(1, np.int32))]


@pytest.mark.parametrize("k", range(3))
def test_pagerank_precision_rows_spanning_tiles(k):
    el = _tile_spanning_graphs()[k]
    ref, rit, rl1 = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, 1e-6)
    eng = GASEngineGPU("pagerank")
    vd = initial_vertex_data("pagerank", el.nV, 0, el.out_degree())
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    for _ in range(2):   # the second run reuses the captured loop
        ranks, st = eng.pagerank_precision(0.85, 1e-6)
        err = np.abs(ranks.astype(np.float64) - ref)
        assert err.sum() <= 1e-6, err.sum()
        assert err.max() <= 1e-7
        assert abs(st.iterations - rit) <= 1
        assert st.residual <= 1e-6
    eng.close()


def test_gather_without_apply_then_scatter():
    """gather() followed by scatterActivate() without apply(): the reference
    runs the gather and keeps the previous apply flags."""
    g = load_golden("rmat8_sym")
    el = golden_el(g)
    eng = GASEngineGPU("cc")
    vd = initial_vertex_data("cc", el.nV)
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    eng.setActive(0, el.nV)
    eng.gather()
    eng.apply()
    eng.scatterActivate()
    n1 = eng.nextIter()
    eng.gather()
    eng.scatterActivate()      # no apply: stale flags, no vertex change
    eng.getResults()
    assert n1 > 0
    ref, _ = oracle.cc(el.nV, el.src, el.dst)
    assert np.all(vd >= ref)


def test_setgraph_recall_and_empty_active_set():
    g = load_golden("rmat10_sym")
    el = golden_el(g)
    s = int(g["source"])
    eng = GASEngineGPU("sssp")
    for _ in range(2):
        vd = initial_vertex_data("sssp", el.nV, s)
        eng.setGraph(el.nV, vd, el.nE, el.weights, el.src, el.dst)
        eng.setActive(0, el.nV)
        eng.run_schedule("generic")
        eng.getResults()
        np.testing.assert_array_equal(vd, g["sssp_dist"])
    eng.setActive(5, 5)
    assert eng.countActive() == 0
    assert eng.run_schedule("generic").iterations == 0


@pytest.mark.parametrize("schedule", ["generic", "auto", "push"])
def test_iteration_cap_reports_error_without_fault(schedule):
    el = EdgeList.rmat(10, 16, seed=1).with_grid_islands(2, 16)
    eng = GASEngineGPU("cc")
    vd = initial_vertex_data("cc", el.nV)
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    eng.setActive(0, el.nV)
    with pytest.raises(GasError) as ei:
        eng.run_schedule(schedule, max_iterations=3)
    assert ei.value.status == 4
    # the context stays usable and the next run converges
    vd2 = initial_vertex_data("cc", el.nV)
    eng.upload_vertex_data(vd2)
    eng.setActive(0, el.nV)
    st = eng.run_schedule(schedule, max_iterations=el.nV + 2)
    eng.getResults()
    ref, rit = oracle.cc(el.nV, el.src, el.dst)
    np.testing.assert_array_equal(vd, ref)
    assert st.iterations == rit


def test_async_download_matches_the_blocking_one():
    """gas_engine_download_vertex_data_async queues the same copy on the
    stream without waiting; after a synchronise it holds what the blocking
    download returns."""
    torch = pytest.importorskip("torch")
    el = EdgeList.rmat(12, 16, seed=3).with_uniform_weights(1, 64, 4)
    s = int(el.sample_sources(1, 3)[0])
    eng = GASEngineGPU("sssp")
    eng.setGraph(el.nV, initial_vertex_data("sssp", el.nV, s), el.nE, el.weights,
                 el.src, el.dst)
    eng.setActive(0, el.nV)
    eng.run_schedule("push", max_iterations=el.nV + 2)
    blocking = np.empty(el.nV, np.int32)
    eng.download_vertex_data(blocking)
    stream = torch.cuda.Stream()
    pinned = torch.full((el.nV,), -7, dtype=torch.int32).pin_memory()
    eng.download_vertex_data_ptr(pinned.data_ptr(), stream.cuda_stream, wait=False)
    stream.synchronize()
    np.testing.assert_array_equal(pinned.numpy(), blocking)
    np.testing.assert_array_equal(blocking, oracle.sssp(el.nV, el.src, el.dst, el.weights, s)[0])
    with pytest.raises(GasError):
        GASEngineGPU("cc").download_vertex_data_ptr(pinned.data_ptr(), wait=False)
    eng.close()


def test_invalid_arguments_raise():
    g = load_golden("path6")
    el = golden_el(g)
    eng = GASEngineGPU("bfs")
    vd = initial_vertex_data("bfs", el.nV)
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    with pytest.raises(GasError):
        eng.setActive(0, el.nV + 1)
    with pytest.raises(GasError):
        eng.setActive(3, 2)
    e2 = GASEngineGPU("sssp")
    with pytest.raises(GasError):
        e2.setGraph(el.nV, initial_vertex_data("sssp", el.nV, 0), el.nE, None, el.src, el.dst)


@pytest.mark.parametrize("schedule", ["generic", "auto", "push", "pull"])
def test_host_loop_mode_matches(schedule, monkeypatch):
    """GAS_HOST_LOOP=1 runs the same kernels as direct launches (the form
    ncu can profile); results and iteration counts must not change."""
    monkeypatch.setenv("GAS_HOST_LOOP", "1")
    el = EdgeList.rmat(12, 16, seed=7).with_uniform_weights(1, 64, 3).with_grid_islands(4, 8)
    s = int(el.sample_sources(1, 7)[0])
    for program, ref in (("sssp", oracle.sssp(el.nV, el.src, el.dst, el.weights, s)),
                         ("cc", oracle.cc(el.nV, el.src, el.dst)),
                         ("bfs", oracle.bfs(el.nV, el.src, el.dst, s))):
        vd, it = run_program(program, el, s, schedule)
        np.testing.assert_array_equal(vd, ref[0])
        assert it == ref[1]
    d = EdgeList.rmat(11, 16, seed=4, symmetrize=False)
    r64, rit, _ = oracle.pagerank_fp64(d.nV, d.src, d.dst, 0.85, 1e-6)
    eng = GASEngineGPU("pagerank")
    vd = initial_vertex_data("pagerank", d.nV, 0, d.out_degree())
    eng.setGraph(d.nV, vd, d.nE, None, d.src, d.dst)
    ranks, st = eng.pagerank_precision(0.85, 1e-6)
    assert np.abs(ranks.astype(np.float64) - r64).sum() <= 1e-6


def test_profiling_mode_counts_kernels_and_keeps_results():
    el = EdgeList.rmat(13, 16, seed=8).with_uniform_weights(1, 64, 3)
    s = int(el.sample_sources(1, 8)[0])
    ref, rit = oracle.sssp(el.nV, el.src, el.dst, el.weights, s)
    eng = GASEngineGPU("sssp")
    vd = initial_vertex_data("sssp", el.nV, s)
    eng.setGraph(el.nV, vd, el.nE, el.weights, el.src, el.dst)
    eng.set_profiling(True)
    eng.setActive(0, el.nV)
    st = eng.run_schedule("auto", max_iterations=el.nV + 2)
    eng.getResults()
    p = eng.profile()
    np.testing.assert_array_equal(vd, ref)
    assert st.iterations == rit
    assert p.push_launches + p.pull_launches == st.iterations
    assert p.push_launches == st.push_iters and p.pull_launches == st.pull_iters
    assert p.push_ms + p.pull_ms > 0 and p.push_bytes + p.pull_bytes > 0
    d = EdgeList.rmat(11, 16, seed=4, symmetrize=False)
    e2 = GASEngineGPU("pagerank")
    vd2 = initial_vertex_data("pagerank", d.nV, 0, d.out_degree())
    e2.setGraph(d.nV, vd2, d.nE, None, d.src, d.dst)
    e2.set_profiling(True)
    ranks, pst = e2.pagerank_precision(0.85, 1e-6)
    pp = e2.profile()
    assert pp.pagerank_launches == pst.iterations and pp.pagerank_ms > 0


def _bfs_run(el, schedule, start, end, small, cap=0):
    import os
    old = os.environ.get("GAS_BFS_SMALL")
    os.environ["GAS_BFS_SMALL"] = "1" if small else "0"
    try:
        eng = GASEngineGPU("bfs")
        vd = initial_vertex_data("bfs", el.nV)
        eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
        eng.setActive(start, end)
        st = eng.run_schedule(schedule, max_iterations=cap or el.nV + 2)
        eng.getResults()
        eng.close()
        return vd, st
    finally:
        if old is None:
            os.environ.pop("GAS_BFS_SMALL", None)
        else:
            os.environ["GAS_BFS_SMALL"] = old


@pytest.mark.parametrize("schedule", ["auto", "learned", "pull"])
def test_small_graph_bfs_kernel_matches_oracle_and_fast_schedule(schedule):
    """BFS on graphs up to 2^18 vertices runs as one cooperative kernel
    (every level inside, a grid barrier between levels): depths and level
    count equal the oracle's and the multi-kernel fast schedule's
    (GAS_BFS_SMALL=0) -- from one source (a hub, an ordinary vertex, one
    without out-edges) and from a range.  Forced bottom-up levels are
    counted alike; under AUTO / LEARNED the two paths take different
    direction rules (the one kernel E/16, the multi-kernel path Beamer's)."""
    graphs = [EdgeList.rmat(16, 16, seed=1),
              EdgeList.rmat(14, 8, seed=3, symmetrize=False),
              EdgeList.rmat(12, 16, seed=2).with_grid_islands(20, 9)]
    for el in graphs:
        hub, _ = el.max_out_degree_vertex()
        od = el.out_degree()
        sink = int(np.flatnonzero(od == 0)[0]) if (od == 0).any() else hub
        ordinary = int(el.sample_sources(1, 4)[0])
        for start, end in ((hub, hub + 1), (ordinary, ordinary + 1), (sink, sink + 1),
                           (5, 40)):
            a, sa = _bfs_run(el, schedule, start, end, True)
            b, sb = _bfs_run(el, schedule, start, end, False)
            np.testing.assert_array_equal(a, b)
            assert sa.iterations == sb.iterations
            if schedule == "pull":
                assert (sa.push_iters, sa.pull_iters) == (sb.push_iters, sb.pull_iters)
            if end == start + 1:
                ref, rit = oracle.bfs(el.nV, el.src, el.dst, start)
                np.testing.assert_array_equal(a, ref)
                assert sa.iterations == rit


def test_small_graph_bfs_kernel_iteration_cap():
    """A run that needs more levels than the cap returns GAS_ERR_ITER_CAP;
    the next run on a fresh engine is exact."""
    el = EdgeList.rmat(12, 16, seed=2).with_grid_islands(4, 30)
    s = el.nV - 1  # a grid corner: the run needs about 60 levels
    with pytest.raises(GasError) as ei:
        _bfs_run(el, "auto", s, s + 1, True, cap=5)
    assert ei.value.status == 4
    vd, st = _bfs_run(el, "auto", s, s + 1, True)
    ref, rit = oracle.bfs(el.nV, el.src, el.dst, s)
    np.testing.assert_array_equal(vd, ref)
    assert st.iterations == rit
