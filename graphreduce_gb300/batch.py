"""Batched engine: many graphs, many BFS sources and personalized-PageRank
seeds per graph, one CUDA-graph launch (libgas ``gas_batch_*``; no reference
counterpart).

The graphs are stored as one disjoint union graph.  Results come back laid
out ``[union vertex][lane]``; :meth:`Batch.depths` and :meth:`Batch.ranks`
slice them per graph.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .engine import _stream_ptr

MAX_LANES = L.GAS_BATCH_MAX_LANES


@dataclass
class BatchResult:
    depth: np.ndarray | None   # int32 [V][bfs_lanes], -1 unreached
    rank: np.ndarray | None    # float32 [V][ppr_lanes]
    stats: L.BatchStats
    dist: np.ndarray | None = None  # int32 [V][sssp_lanes], INT_MAX - 100000 unreached


class Batch:
    """``add_graph`` every graph, ``build`` once, then ``run`` jobs."""

    def __init__(self):
        h = C.c_void_p()
        L.call("gas_batch_create", C.byref(h))
        self._h = h
        self._sizes: list[int] = []

    def close(self) -> None:
        if getattr(self, "_h", None):
            L.load().gas_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_graph(self, nV: int, srcs: np.ndarray, dsts: np.ndarray,
                  weights: np.ndarray | None = None) -> int:
        """weights: int32 per edge for the SSSP lanes (graphs added without
        weights weigh 1 per edge)."""
        s = np.ascontiguousarray(srcs, np.int32)
        d = np.ascontiguousarray(dsts, np.int32)
        if s.shape != d.shape:
            raise ValueError("srcs and dsts differ in length")
        gid = C.c_int32()
        if weights is None:
            L.call("gas_batch_add_graph", self._h, nV, s.shape[0], s.ctypes.data,
                   d.ctypes.data, C.byref(gid))
        else:
            w = np.ascontiguousarray(weights, np.int32)
            if w.shape != s.shape:
                raise ValueError("weights and srcs differ in length")
            L.call("gas_batch_add_graph_weighted", self._h, nV, s.shape[0], s.ctypes.data,
                   d.ctypes.data, w.ctypes.data, C.byref(gid))
        self._sizes.append(nV)
        return gid.value

    def build(self, stream=None) -> None:
        L.call("gas_batch_build", self._h, _stream_ptr(stream))

    @property
    def num_graphs(self) -> int:
        return L.load().gas_batch_num_graphs(self._h)

    @property
    def num_vertices(self) -> int:
        return L.load().gas_batch_num_vertices(self._h)

    @property
    def num_edges(self) -> int:
        return L.load().gas_batch_num_edges(self._h)

    def vertex_offset(self, g: int) -> int:
        return L.load().gas_batch_vertex_offset(self._h, g)

    def set_profiling(self, on: bool) -> None:
        """Kernel-level timing of the BFS and SSSP pushes of later runs
        (direct launches, CUDA events)."""
        L.call("gas_batch_set_profiling", self._h, int(on))

    def profile(self, reset: bool = True) -> L.KernelProfile:
        p = L.KernelProfile()
        L.call("gas_batch_get_profile", self._h, C.byref(p), int(reset))
        return p

    def tune(self, ppr_lanes: int, damping: float = 0.85, trials: int = 3,
             stream=None) -> tuple[int, float]:
        """Autotunes the PPR piece size -> (piece_edges, ms per iteration)."""
        p, ms = C.c_int32(), C.c_float()
        L.call("gas_batch_tune", self._h, ppr_lanes, damping, trials, C.byref(p), C.byref(ms),
               _stream_ptr(stream))
        return p.value, ms.value

    def run(self, bfs_sources: np.ndarray | None = None, ppr_seeds: np.ndarray | None = None,
            damping: float = 0.85, tol: float = 1e-6, max_bfs_levels: int = 0,
            max_ppr_iterations: int = 0, piece_edges: int = 0, depth_out=None,
            rank_out=None, stream=None, sssp_sources: np.ndarray | None = None,
            max_sssp_iterations: int = 0, dist_out=None) -> BatchResult:
        """bfs_sources / sssp_sources / ppr_seeds: int [graphs][lanes] local
        vertex ids (-1: unused lane).  depth_out / dist_out / rank_out:
        optional numpy arrays or device pointers (ints) receiving the
        results."""
        G, V = self.num_graphs, self.num_vertices
        job = L.BatchJob()
        keep = []
        if bfs_sources is not None:
            bs = np.ascontiguousarray(bfs_sources, np.int32)
            if bs.ndim != 2 or bs.shape[0] != G:
                raise ValueError("bfs_sources must be [graphs][lanes]")
            job.bfs_lanes, job.bfs_sources = bs.shape[1], bs.ctypes.data
            keep.append(bs)
        if sssp_sources is not None:
            ss = np.ascontiguousarray(sssp_sources, np.int32)
            if ss.ndim != 2 or ss.shape[0] != G:
                raise ValueError("sssp_sources must be [graphs][lanes]")
            job.sssp_lanes, job.sssp_sources = ss.shape[1], ss.ctypes.data
            job.max_sssp_iterations = max_sssp_iterations
            keep.append(ss)
        if ppr_seeds is not None:
            ps = np.ascontiguousarray(ppr_seeds, np.int32)
            if ps.ndim != 2 or ps.shape[0] != G:
                raise ValueError("ppr_seeds must be [graphs][lanes]")
            job.ppr_lanes, job.ppr_seeds = ps.shape[1], ps.ctypes.data
            keep.append(ps)
        job.damping, job.tol = damping, tol
        job.max_bfs_levels, job.max_ppr_iterations = max_bfs_levels, max_ppr_iterations
        job.piece_edges = piece_edges
        depth = rank = dist = None
        dptr = rptr = sptr = None
        if job.sssp_lanes:
            if isinstance(dist_out, int):
                sptr = dist_out
            else:
                dist = dist_out if dist_out is not None else np.empty((V, job.sssp_lanes),
                                                                      np.int32)
                sptr = dist.ctypes.data
        if job.bfs_lanes:
            if isinstance(depth_out, int):
                dptr = depth_out
            else:
                depth = depth_out if depth_out is not None else np.empty((V, job.bfs_lanes),
                                                                         np.int32)
                dptr = depth.ctypes.data
        if job.ppr_lanes:
            if isinstance(rank_out, int):
                rptr = rank_out
            else:
                rank = rank_out if rank_out is not None else np.empty((V, job.ppr_lanes),
                                                                      np.float32)
                rptr = rank.ctypes.data
        st = L.BatchStats()
        L.call("gas_batch_run", self._h, C.byref(job), dptr, sptr, rptr, C.byref(st),
               _stream_ptr(stream))
        return BatchResult(depth, rank, st, dist)

    def slice(self, arr: np.ndarray, g: int) -> np.ndarray:
        """Rows of graph g in a [union vertex][lane] result."""
        o = self.vertex_offset(g)
        return arr[o:o + self._sizes[g]]
