"""Generates the golden vectors under tests/golden/ from the reference itself.

Runs the reference's own CPU engine GASEngineRef (refgas.h) and graph writer
(graphio.cpp), compiled by `make -C oracle ref` into oracle/_ref/libref.so,
on small hand-made and synthetic graphs, and stores inputs and outputs as
compressed .npz files (plus one reference-written .gr file).  Needs the
reference sources (the REF_DIR environment variable names the checkout); the
fixtures it writes are committed so that tests can run without them.

    REF_DIR=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from graphreduce_gb300.build import build, build_oracle  # noqa: E402
from graphreduce_gb300.graph import EdgeList, edge_list_to_csr  # noqa: E402

OUT = Path(__file__).resolve().parent


def sym(pairs):
    s = [a for a, b in pairs] + [b for a, b in pairs]
    d = [b for a, b in pairs] + [a for a, b in pairs]
    return np.array(s, np.int32), np.array(d, np.int32)


def hand_graphs():
    g = {}
    # path 0-1-2-3-4-5, both directions
    s, d = sym([(i, i + 1) for i in range(5)])
    g["path6"] = (6, s, d)
    # star centred on 3 with 7 leaves
    s, d = sym([(3, i) for i in range(8) if i != 3])
    g["star8"] = (8, s, d)
    # two components plus an isolated vertex (6)
    s, d = sym([(0, 1), (1, 2), (3, 4), (4, 5)])
    g["two_components"] = (7, s, d)
    # self loop and duplicate edges kept in the edge list
    s = np.array([0, 0, 1, 1, 2, 2, 2, 3, 1, 0], np.int32)
    d = np.array([1, 1, 0, 2, 1, 2, 3, 2, 0, 0], np.int32)
    g["loops_dups"] = (4, s, d)
    # directed: vertex 0 has no in-edges, vertex 4 no out-edges
    s = np.array([0, 0, 1, 2, 3, 1, 3], np.int32)
    d = np.array([1, 2, 3, 3, 4, 2, 1], np.int32)
    g["directed_dag"] = (5, s, d)
    # no edges at all
    g["no_edges"] = (5, np.zeros(0, np.int32), np.zeros(0, np.int32))
    return g


def weights_for(nV, s, d, seed=3):
    el = EdgeList(nV, s, d).with_uniform_weights(1, 64, seed)
    return el.weights


def run_case(name, nV, s, d, w, source, directed_pr=True):
    rec = dict(nV=np.int64(nV), src=s, dst=d, w=w, source=np.int64(source))
    if nV > 0:
        rec["bfs_depth"], it = oracle.ref_bfs(nV, s, d, source)
        rec["bfs_iters"] = np.int64(it)
        rec["sssp_dist"], it = oracle.ref_sssp(nV, s, d, w, source)
        rec["sssp_iters"] = np.int64(it)
        rec["cc_label"], it = oracle.ref_cc(nV, s, d)
        rec["cc_iters"] = np.int64(it)
        rec["pr_rank"], it = oracle.ref_pagerank(nV, s, d)
        rec["pr_iters"] = np.int64(it)
    np.savez_compressed(OUT / f"{name}.npz", **rec)
    print(f"{name}: V={nV} E={len(s)} bfs_it={rec.get('bfs_iters')} "
          f"sssp_it={rec.get('sssp_iters')} cc_it={rec.get('cc_iters')} pr_it={rec.get('pr_iters')}")


# Small hand-made text graphs covering the loader's rules: comments, blank
# lines, the ignored size line, 1-based ids, fractional and negative values
# (truncated), self loops with and without values, and every symmetry.
TEXT_GRAPHS = {
    "general_real.mtx": (
        "%%MatrixMarket matrix coordinate real general\n"
        "% a comment\n"
        "%another one\n"
        "5 5 7\n"
        "1 2 2.7\n"
        "2 3 -1.5\n"
        "3 1 10\n"
        "\n"
        "4 5 0.25\n"
        "6 6 3.0\n"
        "5 4 64\n"
        "2 2 1.0\n"),
    "symmetric_int.mtx": (
        "%%MatrixMarket matrix coordinate integer symmetric\n"
        "4 4 4\n"
        "2 1 5\n"
        "3 1 7\n"
        "   \n"
        "4 3 9\n"
        "4 4 2\n"),
    "skew.mtx": (
        "%%MatrixMarket matrix coordinate real skew-symmetric\n"
        "3 3 2\n"
        "2 1 1.9\n"
        "3 2 -4.2\n"),
    "pattern_general.mtx": (
        "%%MatrixMarket matrix coordinate pattern general\n"
        "% self loop on the largest id still counts here\n"
        "7 7 4\n"
        "1 2\n"
        "2 3\n"
        "3 1\n"
        "7 7\n"),
    "pattern_sym.mtx": (
        "%%MatrixMarket matrix coordinate pattern symmetric\n"
        "5 5 3\n"
        "1 5\n"
        "2 5\n"
        "3 4\n"),
    "snap.edge": (
        "# GraphLab / SNAP edge list\n"
        "# FromNodeId ToNodeId\n"
        "0 1\n"
        "1 2\n"
        "2 0\n"
        "3 3\n"
        "\n"
        "2 4\n"),
}


def text_formats():
    d = OUT / "text"
    d.mkdir(exist_ok=True)
    res = {}
    for name, body in TEXT_GRAPHS.items():
        p = d / name
        p.write_text(body)
        valued = name.endswith(".mtx") and "pattern" not in name
        nV, s, t, w = oracle.ref_load_graph(p, 64, want_weights=valued)
        key = name.replace(".", "_")
        res[f"{key}_nV"] = np.int64(nV)
        res[f"{key}_src"], res[f"{key}_dst"] = s, t
        if valued:
            res[f"{key}_w"] = w
    np.savez_compressed(OUT / "text_formats.npz", **res)
    # a MatrixMarket file written by the reference's writeGraph_mtx
    el = EdgeList.rmat(6, 4, seed=31).with_uniform_weights(1, 64, 3)
    oracle.ref_write_mtx(OUT / "text" / "ref_written.mtx", el.nV, el.src, el.dst, el.weights)
    np.savez_compressed(OUT / "ref_written_mtx.npz", nV=np.int64(el.nV), src=el.src,
                        dst=el.dst, w=el.weights)
    print("text/*.mtx, text/*.edge, text_formats.npz, ref_written_mtx.npz")


def main():
    build()
    build_oracle(with_reference=True)
    if not oracle.reference_available():
        raise SystemExit("oracle/_ref/libref.so missing: the reference sources are needed")
    for name, (nV, s, d) in hand_graphs().items():
        w = weights_for(nV, s, d) if len(s) else np.zeros(0, np.int32)
        run_case(name, nV, s, d, w, source=0)
    for scale, seed in ((8, 11), (10, 12)):
        el = EdgeList.rmat(scale, 16, seed=seed).with_uniform_weights(1, 64, 3)
        src, _ = el.max_out_degree_vertex()
        run_case(f"rmat{scale}_sym", el.nV, el.src, el.dst, el.weights, source=src)
    el = EdgeList.rmat(10, 8, seed=13, symmetrize=False).with_uniform_weights(1, 64, 3)
    run_case("rmat10_directed", el.nV, el.src, el.dst, el.weights, source=0)
    el = EdgeList.erdos_renyi(1000, 4000, seed=5, symmetrize=False).with_uniform_weights(1, 64, 3)
    run_case("er1000_directed", el.nV, el.src, el.dst, el.weights, source=7)

    # edgeListToCSR of the reference on a graph with ties, and a .gr file
    # written by the reference's writeGraph_binaryCSR.
    el = EdgeList.rmat(7, 8, seed=21).with_uniform_weights(1, 64, 3)
    rng = np.random.default_rng(0)
    order = rng.permutation(el.nE)
    s, d, w = el.src[order], el.dst[order], el.weights[order]
    off, out, perm = oracle.ref_edge_list_to_csr(el.nV, s, d)
    np.savez_compressed(OUT / "csr_ties.npz", nV=np.int64(el.nV), src=s, dst=d, w=w,
                        ref_off=off, ref_out=out, ref_perm=perm)
    off_csr, dst_csr, perm_csr = edge_list_to_csr(el.nV, s, d)
    oracle.ref_write_gr(OUT / "ref_written.gr", el.nV, off_csr, dst_csr, w[perm_csr])
    print("csr_ties.npz, ref_written.gr")
    text_formats()


if __name__ == "__main__":
    main()
