"""THE ORACLE -- test infrastructure only.

ctypes access to oracle/_build/liboracle.so (gas_oracle.c, the C restatement
of the reference's CPU engine refgas.h and its four programs, and
gas_oracle_gen.c, the seeded input generators the CPU baseline builds its
workload with) and, when it was built from the reference sources,
oracle/_ref/libref.so (the reference's own refgas.h / graphio.cpp).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
package; the engine never does.  Loading it never loads the product library.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIBORACLE = HERE / "_build" / "liboracle.so"
LIBREF = HERE / "_ref" / "libref.so"

_lock = threading.Lock()
_orc = None
_ref = None

c_i32, c_i64, c_dbl, c_vp = C.c_int32, C.c_int64, C.c_double, C.c_void_p


def _oracle():
    global _orc
    with _lock:
        if _orc is None:
            if not LIBORACLE.exists():
                subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
            lib = C.CDLL(str(LIBORACLE))
            lib.orc_edge_list_to_csr.argtypes = [c_i32, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp]
            lib.orc_edge_list_to_csr.restype = C.c_int
            lib.orc_bfs.argtypes = [c_i32, c_i64, c_vp, c_vp, c_i32, c_vp]
            lib.orc_sssp.argtypes = [c_i32, c_i64, c_vp, c_vp, c_vp, c_i32, c_vp]
            lib.orc_cc.argtypes = [c_i32, c_i64, c_vp, c_vp, c_vp]
            lib.orc_pagerank.argtypes = [c_i32, c_i64, c_vp, c_vp, c_vp]
            lib.orc_pagerank_fp64.argtypes = [c_i32, c_i64, c_vp, c_vp, c_dbl, c_dbl, c_i64,
                                              c_vp, c_vp]
            lib.orc_ppr_fp64.argtypes = [c_i32, c_i64, c_vp, c_vp, c_i32, c_dbl, c_dbl, c_i64,
                                         c_vp, c_vp]
            lib.orc_pagerank_fp64_step.argtypes = [c_i32, c_i64, c_vp, c_vp, c_dbl, c_vp, c_vp]
            lib.orc_pagerank_fp64_step.restype = c_dbl
            for f in ("orc_bfs", "orc_sssp", "orc_cc", "orc_pagerank", "orc_pagerank_fp64",
                      "orc_ppr_fp64"):
                getattr(lib, f).restype = c_i64
            lib.orc_set_threads.argtypes = [c_i32]
            lib.orc_set_threads.restype = None
            lib.orc_get_threads.restype = c_i32
            lib.orc_free.argtypes = [c_vp]
            lib.orc_free.restype = None
            lib.orc_rmat.argtypes = [c_i32, c_i32, c_dbl, c_dbl, c_dbl, C.c_uint64, c_i32,
                                     C.POINTER(C.POINTER(c_i32)), C.POINTER(C.POINTER(c_i32))]
            lib.orc_rmat.restype = c_i64
            lib.orc_grid_islands.argtypes = [c_i32, c_i32, c_i32, c_vp, c_vp]
            lib.orc_grid_islands.restype = c_i64
            lib.orc_uniform_weights.argtypes = [c_i64, c_vp, c_vp, c_i32, c_i32, C.c_uint64,
                                                c_vp]
            lib.orc_uniform_weights.restype = C.c_int
            lib.orc_sample_sources.argtypes = [c_i32, c_i64, c_vp, c_vp, c_i32, C.c_uint64,
                                               c_vp]
            lib.orc_sample_sources.restype = C.c_int
            lib.orc_graph_new.argtypes = [c_i32, c_i64, c_vp, c_vp]
            lib.orc_graph_new.restype = c_vp
            lib.orc_graph_delete.argtypes = [c_vp]
            lib.orc_graph_delete.restype = None
            lib.orc_g_bfs.argtypes = [c_vp, c_i32, c_vp]
            lib.orc_g_sssp.argtypes = [c_vp, c_vp, c_i32, c_vp]
            lib.orc_g_cc.argtypes = [c_vp, c_vp]
            lib.orc_g_pagerank.argtypes = [c_vp, c_vp]
            lib.orc_g_pagerank_fp64.argtypes = [c_vp, c_dbl, c_dbl, c_i64, c_vp, c_vp]
            lib.orc_g_ppr_fp64.argtypes = [c_vp, c_i32, c_dbl, c_dbl, c_i64, c_vp, c_vp]
            for f in ("orc_g_bfs", "orc_g_sssp", "orc_g_cc", "orc_g_pagerank",
                      "orc_g_pagerank_fp64", "orc_g_ppr_fp64"):
                getattr(lib, f).restype = c_i64
            _orc = lib
    return _orc


def set_threads(n: int) -> None:
    """OpenMP threads of the oracle's loops (results do not depend on it)."""
    _oracle().orc_set_threads(int(n))


def threads() -> int:
    return int(_oracle().orc_get_threads())


# ---------------------------------------------------------------------------
# Seeded inputs (gas_oracle_gen.c): the workload graphs without the product
# library.
# ---------------------------------------------------------------------------

def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, symmetrize=True):
    """R-MAT edge list sorted by (src, dst) -> (nV, src int32, dst int32)."""
    ps, pd = C.POINTER(c_i32)(), C.POINTER(c_i32)()
    lib = _oracle()
    n = lib.orc_rmat(scale, edge_factor, a, b, c, seed, int(bool(symmetrize)), C.byref(ps),
                     C.byref(pd))
    if n < 0:
        raise RuntimeError(f"oracle rmat failed with code {n}")
    try:
        src = np.ctypeslib.as_array(ps, shape=(max(1, n),))[:n].copy()
        dst = np.ctypeslib.as_array(pd, shape=(max(1, n),))[:n].copy()
    finally:
        lib.orc_free(C.cast(ps, c_vp))
        lib.orc_free(C.cast(pd, c_vp))
    return 1 << scale, src, dst


def with_grid_islands(nV, src, dst, n_islands, side):
    """Appends the grid islands after vertex nV -> (nV', src', dst')."""
    m = n_islands * 4 * side * (side - 1)
    s2, d2 = np.empty(m, np.int32), np.empty(m, np.int32)
    n = _oracle().orc_grid_islands(nV, n_islands, side, s2.ctypes.data, d2.ctypes.data)
    if n != m:
        raise RuntimeError("oracle grid islands: bad arguments")
    return nV + n_islands * side * side, np.concatenate([src, s2]), np.concatenate([dst, d2])


def uniform_weights(src, dst, lo, hi, seed):
    s, d = _i32(src), _i32(dst)
    w = np.empty(s.shape[0], np.int32)
    if _oracle().orc_uniform_weights(s.shape[0], s.ctypes.data, d.ctypes.data, lo, hi, seed,
                                     w.ctypes.data):
        raise ValueError("uniform_weights: bad range")
    return w


def sample_sources(nV, src, dst, k, seed):
    s, d = _i32(src), _i32(dst)
    out = np.zeros(k, np.int32)
    if _oracle().orc_sample_sources(nV, s.shape[0], s.ctypes.data, d.ctypes.data, k, seed,
                                    out.ctypes.data):
        raise ValueError("sample_sources: bad arguments or component too small")
    return out


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, np.int32)


def _check(it: int, what: str) -> int:
    if it < 0:
        raise RuntimeError(f"oracle {what} failed with code {it}")
    return int(it)


class Graph:
    """The oracle engine's CSC + CSR of one edge list, built once
    (refgas.h:81-113) and shared by any number of runs."""

    def __init__(self, nV, src, dst):
        s, d = _i32(src), _i32(dst)
        self.nV, self.nE = int(nV), int(s.shape[0])
        self._h = _oracle().orc_graph_new(nV, s.shape[0], s.ctypes.data, d.ctypes.data)
        if not self._h:
            raise RuntimeError("oracle graph: bad edge list or out of memory")

    def close(self):
        if getattr(self, "_h", None):
            _oracle().orc_graph_delete(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bfs(self, source):
        out = np.zeros(self.nV, np.int32)
        return out, _check(_oracle().orc_g_bfs(self._h, int(source), out.ctypes.data), "bfs")

    def sssp(self, weights, source):
        w = _i32(weights)
        if w.shape[0] != self.nE:
            raise ValueError("one weight per edge")
        out = np.zeros(self.nV, np.int32)
        return out, _check(_oracle().orc_g_sssp(self._h, w.ctypes.data, int(source),
                                                out.ctypes.data), "sssp")

    def cc(self):
        out = np.zeros(self.nV, np.int32)
        return out, _check(_oracle().orc_g_cc(self._h, out.ctypes.data), "cc")

    def pagerank(self):
        out = np.zeros(self.nV, np.float32)
        return out, _check(_oracle().orc_g_pagerank(self._h, out.ctypes.data), "pagerank")

    def pagerank_fp64(self, damping=0.85, tol=1e-6, max_iter=1000):
        out = np.zeros(self.nV, np.float64)
        l1 = C.c_double()
        it = _oracle().orc_g_pagerank_fp64(self._h, damping, tol, max_iter, out.ctypes.data,
                                           C.byref(l1))
        return out, _check(it, "pagerank_fp64"), l1.value

    def ppr_fp64(self, seed, damping=0.85, tol=1e-12, max_iter=10000):
        out = np.zeros(self.nV, np.float64)
        l1 = C.c_double()
        it = _oracle().orc_g_ppr_fp64(self._h, int(seed), damping, tol, max_iter,
                                      out.ctypes.data, C.byref(l1))
        return out, _check(it, "ppr_fp64"), l1.value


def bfs(nV, src, dst, source):
    """bfs.cu:93-134 on refgas.h semantics -> (depth int32[nV], iterations)."""
    s, d = _i32(src), _i32(dst)
    out = np.zeros(nV, np.int32)
    it = _oracle().orc_bfs(nV, s.shape[0], s.ctypes.data, d.ctypes.data, source, out.ctypes.data)
    return out, _check(it, "bfs")


def sssp(nV, src, dst, weights, source):
    """sssp.cu:69-111 (one run) -> (dist int32[nV], iterations)."""
    s, d, w = _i32(src), _i32(dst), _i32(weights)
    out = np.zeros(nV, np.int32)
    it = _oracle().orc_sssp(nV, s.shape[0], s.ctypes.data, d.ctypes.data, w.ctypes.data,
                            source, out.ctypes.data)
    return out, _check(it, "sssp")


def cc(nV, src, dst):
    """connected_component.cu:66-81 -> (label int32[nV], iterations)."""
    s, d = _i32(src), _i32(dst)
    out = np.zeros(nV, np.int32)
    it = _oracle().orc_cc(nV, s.shape[0], s.ctypes.data, d.ctypes.data, out.ctypes.data)
    return out, _check(it, "cc")


def pagerank(nV, src, dst):
    """pagerank.cu:85-101 -> (rank float32[nV], iterations)."""
    s, d = _i32(src), _i32(dst)
    out = np.zeros(nV, np.float32)
    it = _oracle().orc_pagerank(nV, s.shape[0], s.ctypes.data, d.ctypes.data, out.ctypes.data)
    return out, _check(it, "pagerank")


def pagerank_fp64(nV, src, dst, damping=0.85, tol=1e-6, max_iter=1000):
    """Precision-form PageRank in FP64 -> (rank float64[nV], iterations, L1)."""
    s, d = _i32(src), _i32(dst)
    out = np.zeros(nV, np.float64)
    l1 = C.c_double()
    it = _oracle().orc_pagerank_fp64(nV, s.shape[0], s.ctypes.data, d.ctypes.data, damping,
                                     tol, max_iter, out.ctypes.data, C.byref(l1))
    return out, _check(it, "pagerank_fp64"), l1.value


def ppr_fp64(nV, src, dst, seed, damping=0.85, tol=1e-12, max_iter=10000):
    """Personalized PageRank of one seed in FP64 -> (rank float64[nV], iterations, L1)."""
    s, d = _i32(src), _i32(dst)
    out = np.zeros(nV, np.float64)
    l1 = C.c_double()
    it = _oracle().orc_ppr_fp64(nV, s.shape[0], s.ctypes.data, d.ctypes.data, int(seed),
                                damping, tol, max_iter, out.ctypes.data, C.byref(l1))
    return out, _check(it, "ppr_fp64"), l1.value


def pagerank_fp64_step(nV, src, dst, r, damping=0.85):
    """One FP64 precision-form step from ranks r -> (r', L1)."""
    s, d = _i32(src), _i32(dst)
    r = np.ascontiguousarray(r, np.float64)
    out = np.zeros(nV, np.float64)
    l1 = _oracle().orc_pagerank_fp64_step(nV, s.shape[0], s.ctypes.data, d.ctypes.data,
                                          damping, r.ctypes.data, out.ctypes.data)
    return out, l1


def edge_list_to_csr(nV, keys, vals):
    """util.cuh:80-111 restated (stable) -> (offsets int64, out, perm)."""
    k, v = _i32(keys), _i32(vals)
    off = np.zeros(nV + 1, np.int64)
    out = np.zeros(k.shape[0], np.int32)
    perm = np.zeros(k.shape[0], np.int32)
    rc = _oracle().orc_edge_list_to_csr(nV, k.shape[0], k.ctypes.data, v.ctypes.data,
                                        off.ctypes.data, out.ctypes.data, perm.ctypes.data)
    if rc:
        raise ValueError(f"edge_list_to_csr: code {rc}")
    return off, out, perm


# ---------------------------------------------------------------------------
# The reference itself (oracle/_ref/libref.so), when built in this container.
# ---------------------------------------------------------------------------

def reference_available() -> bool:
    return LIBREF.exists()


def _reference():
    global _ref
    with _lock:
        if _ref is None:
            lib = C.CDLL(str(LIBREF))
            lib.ref_bfs.argtypes = [c_i32, c_i32, c_vp, c_vp, c_i32, c_vp]
            lib.ref_sssp.argtypes = [c_i32, c_i32, c_vp, c_vp, c_vp, c_i32, c_vp]
            lib.ref_cc.argtypes = [c_i32, c_i32, c_vp, c_vp, c_vp]
            lib.ref_pagerank.argtypes = [c_i32, c_i32, c_vp, c_vp, c_vp]
            for f in ("ref_bfs", "ref_sssp", "ref_cc", "ref_pagerank"):
                getattr(lib, f).restype = c_i64
            lib.ref_edge_list_to_csr.argtypes = [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp]
            lib.ref_write_gr.argtypes = [C.c_char_p, c_i32, c_i32, c_vp, c_vp, c_vp]
            lib.ref_write_mtx.argtypes = [C.c_char_p, c_i32, c_i32, c_vp, c_vp, c_vp]
            lib.ref_load_graph.argtypes = [C.c_char_p, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp]
            lib.ref_load_graph.restype = c_i64
            _ref = lib
    return _ref


def ref_bfs(nV, src, dst, source):
    s, d = _i32(src), _i32(dst)
    out = np.zeros(nV, np.int32)
    it = _reference().ref_bfs(nV, s.shape[0], s.ctypes.data, d.ctypes.data, source,
                              out.ctypes.data)
    return out, int(it)


def ref_sssp(nV, src, dst, weights, source):
    s, d, w = _i32(src), _i32(dst), _i32(weights)
    out = np.zeros(nV, np.int32)
    it = _reference().ref_sssp(nV, s.shape[0], s.ctypes.data, d.ctypes.data, w.ctypes.data,
                               source, out.ctypes.data)
    return out, int(it)


def ref_cc(nV, src, dst):
    s, d = _i32(src), _i32(dst)
    out = np.zeros(nV, np.int32)
    it = _reference().ref_cc(nV, s.shape[0], s.ctypes.data, d.ctypes.data, out.ctypes.data)
    return out, int(it)


def ref_pagerank(nV, src, dst):
    s, d = _i32(src), _i32(dst)
    out = np.zeros(nV, np.float32)
    it = _reference().ref_pagerank(nV, s.shape[0], s.ctypes.data, d.ctypes.data,
                                   out.ctypes.data)
    return out, int(it)


def ref_edge_list_to_csr(nV, keys, vals):
    k, v = _i32(keys), _i32(vals)
    off = np.zeros(nV + 1, np.int32)
    out = np.zeros(k.shape[0], np.int32)
    perm = np.zeros(k.shape[0], np.int32)
    _reference().ref_edge_list_to_csr(nV, k.shape[0], k.ctypes.data, v.ctypes.data,
                                      off.ctypes.data, out.ctypes.data, perm.ctypes.data)
    return off, out, perm


def ref_write_gr(path, nV, offsets, dsts, weights):
    o, d = _i32(offsets), _i32(dsts)
    w = None if weights is None else _i32(weights)
    _reference().ref_write_gr(str(path).encode(), nV, d.shape[0], o.ctypes.data, d.ctypes.data,
                              None if w is None else w.ctypes.data)


def ref_write_mtx(path, nV, srcs, dsts, weights):
    s, d = _i32(srcs), _i32(dsts)
    w = None if weights is None else _i32(weights)
    _reference().ref_write_mtx(str(path).encode(), nV, s.shape[0], s.ctypes.data, d.ctypes.data,
                               None if w is None else w.ctypes.data)


def ref_load_graph(path, cap, want_weights=True):
    s = np.zeros(cap, np.int32)
    d = np.zeros(cap, np.int32)
    w = np.zeros(cap, np.int32)
    nV = C.c_int32()
    n = _reference().ref_load_graph(str(path).encode(), int(want_weights), cap, C.byref(nV),
                                    s.ctypes.data, d.ctypes.data, w.ctypes.data)
    if n < 0:
        raise ValueError("capacity too small")
    return nV.value, s[:n], d[:n], (w[:n] if want_weights else None)
