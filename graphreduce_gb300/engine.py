"""Python mirror of ``GASEngineGPU`` (gpugas.h:1025-1809) for the reference's
four vertex programs, over the C ABI of libgas.

Method names, argument meaning and call order follow the reference engine:
``setGraph / setActive / countActive / gather / apply / scatterActivate /
nextIter / getResults / run``.  Vertex data is a numpy structured or int32
array owned by the caller, as in the reference (the engine copies it in at
``setGraph`` and writes it back at ``getResults``).  Errors raise
:class:`GasError` where the reference prints and aborts (gpugas.h:1105-1112).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import GasError, RunStats

BFS, SSSP, CC, PAGERANK = "bfs", "sssp", "cc", "pagerank"
_PROG = {BFS: L.GAS_PROG_BFS, SSSP: L.GAS_PROG_SSSP, CC: L.GAS_PROG_CC,
         PAGERANK: L.GAS_PROG_PAGERANK}

# VertexData layouts of the reference programs (bfs.cu:33-36, sssp.cu:28,
# connected_component.cu:28, pagerank.cu:32-37).
PR_VERTEX = np.dtype([("rank", np.float32), ("numOutEdges", np.int32)])
VERTEX_DTYPE = {BFS: np.dtype(np.int32), SSSP: np.dtype(np.int32),
                CC: np.dtype(np.int32), PAGERANK: PR_VERTEX}

SCHEDULES = {"auto": L.GAS_SCHED_AUTO, "generic": L.GAS_SCHED_GENERIC,
             "push": L.GAS_SCHED_PUSH, "pull": L.GAS_SCHED_PULL,
             "ordered": L.GAS_SCHED_ORDERED, "learned": L.GAS_SCHED_LEARNED}

BFS_UNREACHED = -1                       # bfs.cu:107
SSSP_GATHER_ZERO = 2**31 - 1 - 100000    # sssp.cu:32-33


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream"))


class GASEngineGPU:
    """One engine per program, like ``GASEngineGPU<Program>``."""

    def __init__(self, program: str):
        if program not in _PROG:
            raise ValueError(f"unknown program {program!r}; expected one of {sorted(_PROG)}")
        self.program = program
        self.vertex_dtype = VERTEX_DTYPE[program]
        h = C.c_void_p()
        L.call("gas_engine_create", _PROG[program], C.byref(h))
        self._h = h.value
        self._vd = None
        self._keep = []

    def close(self) -> None:
        if getattr(self, "_h", None):
            L.load().gas_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the reference API -------------------------------------------------
    def setGraph(self, nVertices: int, vertexData: np.ndarray, nEdges: int,
                 edgeData: np.ndarray | None, srcs: np.ndarray, dsts: np.ndarray,
                 stream=None) -> None:
        vd = vertexData
        if vd.dtype != self.vertex_dtype or not vd.flags.c_contiguous:
            raise ValueError(f"vertexData must be a C-contiguous {self.vertex_dtype} array")
        if vd.shape[0] != nVertices:
            raise ValueError("vertexData must hold nVertices records")
        s = np.ascontiguousarray(srcs, np.int32)
        d = np.ascontiguousarray(dsts, np.int32)
        if s.shape[0] != nEdges or d.shape[0] != nEdges:
            raise ValueError("srcs/dsts must hold nEdges entries")
        ed = None if edgeData is None else np.ascontiguousarray(edgeData, np.int32)
        L.call("gas_engine_set_graph", self._h, nVertices, vd.ctypes.data, nEdges,
               None if ed is None else ed.ctypes.data, s.ctypes.data, d.ctypes.data,
               _stream_ptr(stream))
        self._vd = vd
        self.nVertices, self.nEdges = nVertices, nEdges

    def setActive(self, start: int, end: int, stream=None) -> None:
        L.call("gas_engine_set_active", self._h, start, end, _stream_ptr(stream))

    def countActive(self) -> int:
        n = C.c_int32()
        L.call("gas_engine_count_active", self._h, C.byref(n))
        return n.value

    def gather(self, haveGather: bool = True, stream=None) -> None:
        L.call("gas_engine_gather", self._h, int(haveGather), _stream_ptr(stream))

    def apply(self, stream=None) -> None:
        L.call("gas_engine_apply", self._h, _stream_ptr(stream))

    def scatterActivate(self, haveScatter: bool = True, stream=None) -> None:
        L.call("gas_engine_scatter_activate", self._h, int(haveScatter), _stream_ptr(stream))

    def nextIter(self, stream=None) -> int:
        n = C.c_int32()
        L.call("gas_engine_next_iter", self._h, C.byref(n), _stream_ptr(stream))
        return n.value

    def getResults(self, stream=None) -> None:
        L.call("gas_engine_get_results", self._h, _stream_ptr(stream))

    def run(self, stream=None) -> int:
        it = C.c_int32()
        L.call("gas_engine_run", self._h, C.byref(it), _stream_ptr(stream))
        return it.value

    def setIterationCount(self, level: int) -> None:
        """setIterationCount<true> of bfs.cu:83-90 for the built-in BFS."""
        L.call("gas_engine_set_iteration", self._h, level)

    # -- device-resident extensions ----------------------------------------
    def run_schedule(self, schedule: str = "auto", max_iterations: int = 0,
                     stream=None) -> RunStats:
        st = RunStats()
        L.call("gas_engine_run_schedule", self._h, SCHEDULES[schedule], max_iterations,
               C.byref(st), _stream_ptr(stream))
        return st

    def _out_ptr(self, out):
        """(host array or None, pointer) for a float32 result: out may be a
        numpy array, a device pointer (int) or None (new host array)."""
        if isinstance(out, int):
            return None, out
        ranks = out if out is not None else np.zeros(self.nVertices, np.float32)
        return ranks, ranks.ctypes.data

    def pagerank_precision(self, damping: float = 0.85, tol: float = 1e-6,
                           max_iterations: int = 1000, out=None, stream=None):
        """Normalised PageRank with FP32 compensated gather and FP64 L1
        residual; returns (ranks, RunStats), ranks None when out is a device
        pointer."""
        ranks, ptr = self._out_ptr(out)
        st = RunStats()
        L.call("gas_engine_pagerank_precision", self._h, damping, tol, max_iterations,
               ptr, C.byref(st), _stream_ptr(stream))
        return ranks, st

    def vertex_data_device(self) -> int:
        p = C.c_void_p()
        L.call("gas_engine_vertex_data_device", self._h, C.byref(p))
        return p.value

    def upload_vertex_data(self, host: np.ndarray, stream=None) -> None:
        L.call("gas_engine_upload_vertex_data", self._h, host.ctypes.data, _stream_ptr(stream))

    def download_vertex_data(self, host: np.ndarray, stream=None) -> None:
        L.call("gas_engine_download_vertex_data", self._h, host.ctypes.data,
               _stream_ptr(stream))

    def upload_vertex_data_ptr(self, ptr: int, stream=None) -> None:
        """Copies nV records from any host or device address into the
        engine's device vertex data."""
        L.call("gas_engine_upload_vertex_data", self._h, ptr, _stream_ptr(stream))

    def download_vertex_data_ptr(self, ptr: int, stream=None, wait: bool = True) -> None:
        """Copies the device vertex data to any host or device address;
        wait=True synchronises the stream, wait=False only queues the copy
        on it (the destination must stay valid until it completes)."""
        L.call("gas_engine_download_vertex_data" if wait else
               "gas_engine_download_vertex_data_async", self._h, ptr, _stream_ptr(stream))

    def set_profiling(self, on: bool) -> None:
        """Kernel-level timing of later runs (direct launches, CUDA events)."""
        L.call("gas_engine_set_profiling", self._h, int(on))

    def profile(self, reset: bool = True) -> L.KernelProfile:
        p = L.KernelProfile()
        L.call("gas_engine_get_profile", self._h, C.byref(p), int(reset))
        return p

    def set_trace(self, on: bool) -> None:
        """Per-iteration device records of later fast runs."""
        L.call("gas_engine_set_trace", self._h, int(on))

    def trace(self) -> list:
        """The last run's records (list of TraceRecord)."""
        buf = (L.TraceRecord * L.GAS_TRACE_CAP)()
        n = C.c_int32()
        L.call("gas_engine_get_trace", self._h, buf, L.GAS_TRACE_CAP, C.byref(n))
        return [buf[i] for i in range(n.value)]

    def set_schedule_model(self, mlp) -> None:
        """Schedule head for run_schedule("learned") (None removes it)."""
        L.call("gas_engine_set_schedule_model", self._h, None if mlp is None else mlp.handle)
        self._sched_model = mlp

    def pagerank_warm_start(self, mlp, damping: float = 0.85,
                            out: np.ndarray | None = None) -> np.ndarray:
        """Initial PageRank vector proposed by the warm-start head, scaled to
        the fixed point's mass for this damping."""
        init, ptr = self._out_ptr(out)
        L.call("gas_engine_pagerank_warm_start", self._h, mlp.handle, damping, ptr, None)
        return init

    def pagerank_precision_from(self, init, damping: float = 0.85, tol: float = 1e-6,
                                max_iterations: int = 1000, stream=None, out=None):
        """From a given start vector (numpy array, device pointer or None for
        the uniform 1/N) -> (ranks, RunStats)."""
        ranks, ptr = self._out_ptr(out)
        st = RunStats()
        if isinstance(init, int):
            ip, iptr = None, init
        else:
            ip = None if init is None else np.ascontiguousarray(init, np.float32)
            iptr = None if ip is None else ip.ctypes.data
        L.call("gas_engine_pagerank_precision_from", self._h, damping, tol, max_iterations,
               iptr, ptr, C.byref(st), _stream_ptr(stream))
        return ranks, st

    def ppr_precision(self, seed: int, damping: float = 0.85, tol: float = 1e-6,
                      max_iterations: int = 1000, out=None, stream=None):
        """Personalized PageRank of one seed -> (ranks, RunStats).  out: a
        float32 numpy array, a device pointer (int), or None for a new host
        array; ranks is None when out is a device pointer."""
        st = RunStats()
        if isinstance(out, int):
            ranks, ptr = None, out
        else:
            ranks = out if out is not None else np.zeros(self.nVertices, np.float32)
            ptr = ranks.ctypes.data
        L.call("gas_engine_ppr_precision", self._h, int(seed), damping, tol, max_iterations,
               ptr, C.byref(st), _stream_ptr(stream))
        return ranks, st

    def set_edge_placement(self, where: str) -> None:
        """"device" (HBM) or "host" (pinned host memory read over NVLink-C2C);
        applies from the next setGraph."""
        L.call("gas_engine_set_edge_placement", self._h, {"device": 0, "host": 1}[where])

    def graph_arrays(self) -> dict:
        """Host copies of the CSC and CSR the engine built (edge data as int32
        for the built-in programs)."""
        nV, nE = self.nVertices, self.nEdges
        out = {k: np.empty(nV + 1, np.int32) for k in ("csc_off", "csr_off")}
        out.update({k: np.empty(nE, np.int32) for k in ("csc_src", "csr_dst")})
        ptr = {k: v.ctypes.data for k, v in out.items()}
        if self.program == SSSP:
            out["csc_w"] = np.empty(nE, np.int32)
            out["csr_w"] = np.empty(nE, np.int32)
        L.call("gas_engine_download_graph", self._h, ptr["csc_off"], ptr["csc_src"],
               ptr["csr_off"], ptr["csr_dst"],
               out["csc_w"].ctypes.data if "csc_w" in out else None,
               out["csr_w"].ctypes.data if "csr_w" in out else None, None)
        return out

    def counters(self) -> L.Counters:
        c = L.Counters()
        L.call("gas_engine_read_counters", self._h, C.byref(c), None)
        return c


# -- whole-algorithm helpers shaped like the reference apps' run<> ----------

def initial_vertex_data(program: str, nV: int, source: int | None = None,
                        out_degree: np.ndarray | None = None) -> np.ndarray:
    """Vertex data exactly as the reference apps initialise it."""
    if program == BFS:
        return np.full(nV, BFS_UNREACHED, np.int32)
    if program == SSSP:
        vd = np.full(nV, SSSP_GATHER_ZERO, np.int32)
        if nV:
            vd[source] = 0
        return vd
    if program == CC:
        return np.arange(nV, dtype=np.int32)
    vd = np.zeros(nV, PR_VERTEX)
    vd["rank"] = np.float32(0.15)
    vd["numOutEdges"] = out_degree
    return vd


def run_program(program: str, el, source: int = 0, schedule: str = "step",
                stream=None):
    """Runs a reference program the way its app does (bfs.cu:93-134,
    sssp.cu:69-111, connected_component.cu:66-81, pagerank.cu:85-101);
    returns (vertex data, iterations).  schedule="step" drives the step API
    from the host; other values use run_schedule."""
    eng = GASEngineGPU(program)
    try:
        vd = initial_vertex_data(program, el.nV, source, el.out_degree())
        ed = el.weights if program == SSSP else None
        eng.setGraph(el.nV, vd, el.nE, ed, el.src, el.dst, stream)
        if program == BFS:
            eng.setActive(source, source + 1, stream)
        else:
            eng.setActive(0, el.nV, stream)
        # BFS/SSSP/CC never need more than nV + 2 iterations (Bellman-Ford
        # bound); PageRank's |delta| >= 0.01 rule converges in tens
        cap = el.nV + 2 if program != PAGERANK else 100000
        if schedule == "step":
            it = 0
            eng.setIterationCount(0)
            while eng.countActive():
                if it >= cap:
                    raise GasError(4, "run_program", f"no convergence in {cap} iterations")
                eng.gather(program != BFS, stream)
                eng.apply(stream)
                eng.scatterActivate(program != BFS, stream)
                eng.nextIter(stream)
                it += 1
                eng.setIterationCount(it)
        else:
            it = eng.run_schedule(schedule, max_iterations=cap, stream=stream).iterations
        eng.getResults(stream)
        return vd, it
    finally:
        eng.close()


__all__ = ["GASEngineGPU", "GasError", "run_program", "initial_vertex_data", "BFS", "SSSP",
           "CC", "PAGERANK", "PR_VERTEX"]
