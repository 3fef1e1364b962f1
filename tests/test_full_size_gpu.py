"""Size-independent properties of the fast schedules at the headline size
(R-MAT scale 22, seed 2, symmetrised: 4.2 M vertices, 128 M directed
edges; CC adds 4,096 32x32 grid islands), checked on the device over every
edge, and every schedule's output identical.  The bench compares the same
workload with the oracle; these checks hold whatever the oracle says:

* SSSP: d[source] = 0, d[v] <= d[u] + w on every edge out of a reached u,
  and every other reached vertex has an in-edge with d[v] = d[u] + w.
* CC: labels agree across every edge, l[v] <= v, l[l[v]] = l[v], and each
  label is the smallest vertex id carrying it.
* BFS: depth[source] = 0, depth[v] <= depth[u] + 1 on every edge out of a
  reached u, and every other reached vertex has an in-neighbour one level
  up."""
import numpy as np
import pytest

from graphreduce_gb300 import GASEngineGPU
from graphreduce_gb300.engine import initial_vertex_data
from graphreduce_gb300.graph import EdgeList
from graphreduce_gb300.learn import DATA, MLP

pytestmark = pytest.mark.gpu

SSSP_INF = 2**31 - 1 - 100000


@pytest.fixture(scope="module")
def torch(libgas):
    return pytest.importorskip("torch")


@pytest.fixture(scope="module")
def base(libgas):
    return EdgeList.rmat(22, 16, seed=2, symmetrize=True)


def _runs(program, el, s, schedules):
    eng = GASEngineGPU(program)
    vd = initial_vertex_data(program, el.nV, s)
    eng.setGraph(el.nV, vd, el.nE, el.weights if program == "sssp" else None, el.src, el.dst)
    eng.set_schedule_model(MLP.load(DATA / "schedule_head.npz"))
    outs = {}
    for sched in schedules:
        eng.upload_vertex_data(initial_vertex_data(program, el.nV, s))
        eng.setActive(*((s, s + 1) if program == "bfs" else (0, el.nV)))
        st = eng.run_schedule(sched, max_iterations=el.nV + 2)
        out = np.empty(el.nV, np.int32)
        eng.download_vertex_data(out)
        outs[sched] = (out, st.iterations)
    eng.close()
    first = next(iter(outs.values()))
    for sched, (out, it) in outs.items():
        np.testing.assert_array_equal(out, first[0], err_msg=sched)
        assert it == first[1], sched
    return first[0]


def _dev(torch, el, out):
    d = torch.from_numpy(out).cuda().long()
    src = torch.from_numpy(el.src).cuda().long()
    dst = torch.from_numpy(el.dst).cuda().long()
    return d, src, dst


def test_sssp_distances_at_headline_size(torch, base):
    el = base.with_uniform_weights(1, 64, 3)
    s = int(el.sample_sources(1, 2)[0])
    out = _runs("sssp", el, s, ("push", "pull", "auto", "learned"))
    d, src, dst = _dev(torch, el, out)
    w = torch.from_numpy(el.weights).cuda().long()
    assert int(d[s]) == 0
    reached = d != SSSP_INF
    assert int(reached.sum()) > el.nV // 2
    du, dv = d[src], d[dst]
    m = du != SSSP_INF
    assert bool(torch.all(dv[m] <= du[m] + w[m]))
    tight = m & (dv == du + w)
    has_parent = torch.zeros(el.nV, dtype=torch.bool, device="cuda")
    has_parent[dst[tight]] = True
    others = reached.clone()
    others[s] = False
    assert bool(torch.all(has_parent[others]))


def test_cc_labels_at_headline_size(torch, base):
    el = base.with_grid_islands(4096, 32)
    out = _runs("cc", el, 0, ("push", "pull", "auto", "learned"))
    lab, src, dst = _dev(torch, el, out)
    v = torch.arange(el.nV, device="cuda")
    assert bool(torch.all(lab[src] == lab[dst]))
    assert bool(torch.all(lab <= v))
    assert bool(torch.all(lab[lab] == lab))
    smallest = torch.full((el.nV,), el.nV, dtype=torch.long, device="cuda")
    smallest.scatter_reduce_(0, lab, v, reduce="amin")
    used = torch.unique(lab)
    assert bool(torch.all(smallest[used] == used))
    # each island is its own component, labelled by its first vertex
    first = base.nV + 1024 * torch.arange(4096, device="cuda")
    assert bool(torch.all(lab[first] == first))


def test_bfs_depths_at_headline_size(torch, base):
    s = int(base.sample_sources(1, 2)[0])
    out = _runs("bfs", base, s, ("push", "pull", "auto"))
    d, src, dst = _dev(torch, base, out)
    assert int(d[s]) == 0
    du, dv = d[src], d[dst]
    m = du >= 0
    assert bool(torch.all((dv[m] >= 0) & (dv[m] <= du[m] + 1)))
    up = m & (dv == du + 1)
    has_parent = torch.zeros(base.nV, dtype=torch.bool, device="cuda")
    has_parent[dst[up]] = True
    others = d >= 0
    others[s] = False
    assert bool(torch.all(has_parent[others]))
    assert int(d.max()) >= 5
