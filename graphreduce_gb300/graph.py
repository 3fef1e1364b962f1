"""Host edge lists: synthetic generators and ``.gr`` I/O (the reference's
graphio.cpp / util.cuh layer), backed by libgas's native host code."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L


def _arr(ptr: int | None, n: int) -> np.ndarray:
    if n == 0 or not ptr:
        return np.zeros(0, np.int32)
    buf = (C.c_int32 * n).from_address(ptr)
    return np.frombuffer(buf, dtype=np.int32, count=n).copy()


@dataclass
class EdgeList:
    """nV vertices and nE directed edges (src[i] -> dst[i]) with optional
    int32 edge data, as loadGraph returns them (graphio.h:63-67)."""

    nV: int
    src: np.ndarray
    dst: np.ndarray
    weights: np.ndarray | None = None

    @property
    def nE(self) -> int:
        return int(self.src.shape[0])

    # -- native handle round trip -------------------------------------------
    @classmethod
    def _from_handle(cls, h: int) -> "EdgeList":
        lib = L.load()
        try:
            nV = lib.gas_edge_list_num_vertices(h)
            nE = lib.gas_edge_list_num_edges(h)
            src = _arr(lib.gas_edge_list_srcs(h), nE)
            dst = _arr(lib.gas_edge_list_dsts(h), nE)
            wp = lib.gas_edge_list_weights(h)
            w = _arr(wp, nE) if wp else None
        finally:
            lib.gas_edge_list_destroy(h)
        return cls(int(nV), src, dst, w)

    def _handle(self) -> int:
        h = C.c_void_p()
        src = np.ascontiguousarray(self.src, np.int32)
        dst = np.ascontiguousarray(self.dst, np.int32)
        w = None if self.weights is None else np.ascontiguousarray(self.weights, np.int32)
        L.call("gas_edge_list_create", self.nV, self.nE, src.ctypes.data, dst.ctypes.data,
               None if w is None else w.ctypes.data, C.byref(h))
        return h.value

    # -- generators -----------------------------------------------------------
    @classmethod
    def rmat(cls, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, seed: int = 1, symmetrize: bool = True) -> "EdgeList":
        h = C.c_void_p()
        L.call("gas_rmat", scale, edge_factor, a, b, c, seed, int(symmetrize), C.byref(h))
        return cls._from_handle(h.value)

    @classmethod
    def erdos_renyi(cls, nV: int, n_samples: int, seed: int = 5,
                    symmetrize: bool = False) -> "EdgeList":
        h = C.c_void_p()
        L.call("gas_erdos_renyi", nV, n_samples, seed, int(symmetrize), C.byref(h))
        return cls._from_handle(h.value)

    def _mutate(self, fn: str, *args) -> "EdgeList":
        h = self._handle()
        try:
            L.call(fn, h, *args)
        except Exception:
            L.load().gas_edge_list_destroy(h)
            raise
        return EdgeList._from_handle(h)

    def with_grid_islands(self, n_islands: int, side: int) -> "EdgeList":
        return self._mutate("gas_edge_list_append_grid_islands", n_islands, side)

    def with_uniform_weights(self, lo: int, hi: int, seed: int) -> "EdgeList":
        return self._mutate("gas_edge_list_set_uniform_weights", lo, hi, seed)

    def max_out_degree_vertex(self) -> tuple[int, int]:
        h = self._handle()
        v, d = C.c_int32(), C.c_int32()
        try:
            L.call("gas_edge_list_max_out_degree_vertex", h, C.byref(v), C.byref(d))
        finally:
            L.load().gas_edge_list_destroy(h)
        return v.value, d.value

    def sample_sources(self, k: int, seed: int) -> np.ndarray:
        h = self._handle()
        out = np.zeros(k, np.int32)
        try:
            L.call("gas_edge_list_sample_sources", h, k, seed, out.ctypes.data)
        finally:
            L.load().gas_edge_list_destroy(h)
        return out

    # -- .gr files ------------------------------------------------------------
    def write_gr(self, path: str) -> None:
        h = self._handle()
        try:
            L.call("gas_gr_write", str(path).encode(), h)
        finally:
            L.load().gas_edge_list_destroy(h)

    @classmethod
    def read_gr(cls, path: str) -> "EdgeList":
        h = C.c_void_p()
        L.call("gas_gr_read", str(path).encode(), C.byref(h))
        return cls._from_handle(h.value)

    def write_mtx(self, path: str) -> None:
        """MatrixMarket coordinate, 1-based, "Integer general" (writeGraph_mtx)."""
        h = self._handle()
        try:
            L.call("gas_mtx_write", str(path).encode(), h)
        finally:
            L.load().gas_edge_list_destroy(h)

    @classmethod
    def read(cls, path: str) -> "EdgeList":
        """.mtx, .edge (GraphLab / SNAP) or .gr, chosen by extension (loadGraph)."""
        h = C.c_void_p()
        L.call("gas_graph_read", str(path).encode(), C.byref(h))
        return cls._from_handle(h.value)

    # -- degrees / CSR --------------------------------------------------------
    def out_degree(self) -> np.ndarray:
        return np.bincount(self.src, minlength=self.nV).astype(np.int32)

    def in_degree(self) -> np.ndarray:
        return np.bincount(self.dst, minlength=self.nV).astype(np.int32)


def edge_list_to_csr(nV: int, keys: np.ndarray, vals: np.ndarray | None):
    """edgeListToCSR (util.cuh:80-111): (offsets[nV+1], out, perm)."""
    keys = np.ascontiguousarray(keys, np.int32)
    nE = keys.shape[0]
    off = np.zeros(nV + 1, np.int32)
    perm = np.zeros(nE, np.int32)
    out = np.zeros(nE, np.int32) if vals is not None else None
    v = None if vals is None else np.ascontiguousarray(vals, np.int32)
    L.call("gas_edge_list_to_csr", nV, nE, keys.ctypes.data,
           None if v is None else v.ctypes.data, off.ctypes.data,
           None if out is None else out.ctypes.data, perm.ctypes.data)
    return off, out, perm
