"""Host-side graph layer of libgas: generators, .gr I/O, CSR construction.
CPU only (no kernel launches)."""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from graphreduce_gb300 import GasError
from graphreduce_gb300.graph import EdgeList, edge_list_to_csr


@pytest.fixture(scope="module", autouse=True)
def _built(libgas):
    return libgas


def _keys(el):
    return el.src.astype(np.int64) << 32 | el.dst.astype(np.int64)


def test_rmat_is_deterministic_sorted_simple():
    a = EdgeList.rmat(12, 16, seed=1)
    b = EdgeList.rmat(12, 16, seed=1)
    c = EdgeList.rmat(12, 16, seed=2)
    np.testing.assert_array_equal(a.src, b.src)
    np.testing.assert_array_equal(a.dst, b.dst)
    assert not (a.nE == c.nE and np.array_equal(a.dst, c.dst))
    k = _keys(a)
    assert np.all(np.diff(k) > 0)          # sorted by (src, dst), no duplicates
    assert not np.any(a.src == a.dst)      # no self loops
    assert a.nV == 4096
    assert a.src.max() < a.nV and a.dst.max() < a.nV
    # symmetric: the reverse of every edge is present
    rev = np.sort(a.dst.astype(np.int64) << 32 | a.src.astype(np.int64))
    np.testing.assert_array_equal(rev, k)


def test_rmat_skew_follows_quadrant_probabilities():
    el = EdgeList.rmat(14, 16, seed=1, symmetrize=False)
    # with a = 0.57 the low vertex ids dominate: vertex 0 is the top out-degree
    v, d = el.max_out_degree_vertex()
    assert v == 0 and d > 50 * el.nE / el.nV
    top_bit = (el.src >> 13) & 1
    frac_high = top_bit.mean()
    assert 0.2 < frac_high < 0.3           # c + d = 0.24 before dedupe


def test_erdos_renyi_uniform():
    el = EdgeList.erdos_renyi(1 << 14, 16 << 14, seed=5)
    deg = el.out_degree()
    assert abs(deg.mean() - 16) < 0.5
    assert deg.max() < 50
    assert np.all(np.diff(_keys(el)) > 0)


def test_grid_islands_structure():
    base = EdgeList.rmat(6, 4, seed=3)
    el = base.with_grid_islands(3, 4)
    assert el.nV == base.nV + 3 * 16
    extra_s, extra_d = el.src[base.nE:], el.dst[base.nE:]
    assert extra_s.shape[0] == 3 * 4 * 4 * 3
    for s, d in zip(extra_s, extra_d):
        ls, ld = s - base.nV, d - base.nV
        assert ls // 16 == ld // 16        # same island
        rs, cs, rd, cd = (ls % 16) // 4, ls % 4, (ld % 16) // 4, ld % 4
        assert abs(rs - rd) + abs(cs - cd) == 1
    assert np.all(np.diff(_keys(el)) > 0)


def test_uniform_weights_range_and_symmetry():
    el = EdgeList.rmat(10, 16, seed=1).with_uniform_weights(1, 64, 3)
    assert el.weights.min() >= 1 and el.weights.max() <= 64
    assert len(np.unique(el.weights)) == 64
    w = dict(zip(zip(el.src.tolist(), el.dst.tolist()), el.weights.tolist()))
    for (u, v), x in list(w.items())[:2000]:
        assert w[(v, u)] == x


def test_sample_sources_in_largest_component():
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    el = EdgeList.rmat(10, 4, seed=2).with_grid_islands(8, 8)
    srcs = el.sample_sources(8, seed=3)
    assert len(set(srcs.tolist())) == 8
    m = coo_matrix((np.ones(el.nE), (el.src, el.dst)), shape=(el.nV, el.nV))
    _, lab = connected_components(m, directed=True, connection="weak")
    big = np.bincount(lab).argmax()
    assert np.all(lab[srcs] == big)
    np.testing.assert_array_equal(srcs, el.sample_sources(8, seed=3))


def test_max_out_degree_vertex_first_max():
    s = np.array([2, 2, 5, 5, 1], np.int32)
    d = np.array([0, 1, 0, 1, 0], np.int32)
    assert EdgeList(6, s, d).max_out_degree_vertex() == (2, 2)


def test_csr_matches_oracle_and_reference_offsets():
    with np.load(GOLDEN / "csr_ties.npz") as z:
        nV, s, d = int(z["nV"]), z["src"], z["dst"]
        ref_off = z["ref_off"]
    off, out, perm = edge_list_to_csr(nV, s, d)
    o_off, o_out, o_perm = oracle.edge_list_to_csr(nV, s, d)
    np.testing.assert_array_equal(off, ref_off)
    np.testing.assert_array_equal(off, o_off)
    np.testing.assert_array_equal(out, o_out)
    np.testing.assert_array_equal(perm, o_perm)


def test_csr_rejects_out_of_range_keys():
    with pytest.raises(GasError) as ei:
        edge_list_to_csr(3, np.array([0, 3]), np.array([1, 1]))
    assert ei.value.status == 1


def test_gr_reads_reference_written_file():
    with np.load(GOLDEN / "csr_ties.npz") as z:
        nV, s, d, w = int(z["nV"]), z["src"], z["dst"], z["w"]
    el = EdgeList.read_gr(GOLDEN / "ref_written.gr")
    off, out, perm = edge_list_to_csr(nV, s, d)
    assert el.nV == nV
    np.testing.assert_array_equal(el.dst, out)
    np.testing.assert_array_equal(el.src, np.repeat(np.arange(nV), np.diff(off)))
    np.testing.assert_array_equal(el.weights, w[perm])


def test_gr_round_trip(tmp_path):
    el = EdgeList.rmat(9, 8, seed=4).with_uniform_weights(1, 64, 3)
    p = tmp_path / "g.gr"
    el.write_gr(p)
    back = EdgeList.read_gr(p)
    np.testing.assert_array_equal(back.src, el.src)
    np.testing.assert_array_equal(back.dst, el.dst)
    np.testing.assert_array_equal(back.weights, el.weights)


def test_gr_odd_edge_count_padding(tmp_path):
    el = EdgeList(3, np.array([0, 1, 2], np.int32), np.array([1, 2, 0], np.int32),
                  np.array([5, 6, 7], np.int32))
    p = tmp_path / "odd.gr"
    el.write_gr(p)
    assert p.stat().st_size == 32 + 3 * 8 + 4 * 4 + 3 * 4
    back = EdgeList.read_gr(p)
    np.testing.assert_array_equal(back.weights, [5, 6, 7])


@pytest.mark.skipif(not oracle.reference_available(), reason="reference not built here")
def test_gr_written_here_loads_in_reference(tmp_path):
    el = EdgeList.rmat(8, 8, seed=9).with_uniform_weights(1, 64, 3)
    p = tmp_path / "ours.gr"
    el.write_gr(p)
    nV, s, d, w = oracle.ref_load_graph(p, el.nE + 1)
    assert nV == el.nV
    np.testing.assert_array_equal(s, el.src)
    np.testing.assert_array_equal(d, el.dst)
    np.testing.assert_array_equal(w, el.weights)


def test_gr_rejects_truncated_and_missing(tmp_path):
    p = tmp_path / "bad.gr"
    p.write_bytes(b"\x01\x00\x00")
    with pytest.raises(GasError) as ei:
        EdgeList.read_gr(p)
    assert ei.value.status == 5
    with pytest.raises(GasError):
        EdgeList.read_gr(tmp_path / "missing.gr")
    full = (GOLDEN / "ref_written.gr").read_bytes()
    p.write_bytes(full[: len(full) // 2])
    with pytest.raises(GasError):
        EdgeList.read_gr(p)


def test_edge_list_create_validates_ids():
    with pytest.raises(GasError):
        EdgeList(2, np.array([0, 2], np.int32), np.array([1, 1], np.int32)).write_gr("/tmp/x")


def test_schedule_features_host_function():
    """gas_schedule_features (the function the device loop evaluates) against
    a restatement in numpy."""
    from graphreduce_gb300 import _lib as L
    from graphreduce_gb300.learn import schedule_features
    rec = L.TraceRecord()
    rec.iteration, rec.mode, rec.n_queue, rec.n_edges_out = 7, 1, 1000, 50000
    for b, v in enumerate([400, 300, 200, 50, 30, 10, 7, 3]):
        rec.hist[b] = v
    f = schedule_features(rec, 1 << 20, 32 << 20, True)
    want = [np.log2(1001) / 32, np.log2(50001) / 32, np.log2(1 + (1 << 20)) / 32,
            np.log2(1 + (32 << 20)) / 32, 50000 / (32 << 20), 1000 / (1 << 20),
            0.4, 0.3, 0.2, 0.05, 0.03, 0.01, 0.007, 0.003, 7 / 64, 1.0]
    np.testing.assert_allclose(f, want, rtol=1e-5, atol=1e-7)
