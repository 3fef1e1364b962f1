"""The learned parts of the engine: the per-iteration schedule head and the
PageRank warm-start head (no reference counterpart).

Both are ``gas_mlp`` models (in -> 64 -> 64 -> out, BF16 weights, FP32
accumulation) trained on the GPU by libgas's own forward/backward and Adam
kernels, on data the engine records about itself:

* schedule head -- every training graph runs SSSP and CC twice, once with
  every iteration forced to push and once forced to the dense pull.  Both
  runs go through the same sequence of frontiers (the schedules are exact),
  so iteration k of the two runs differs only in the kernel that ran; the
  device trace gives each iteration's duration, the label is the faster
  mode and the sample weight the time difference.  The fixed heuristic
  (AUTO) stays the fallback and the yardstick: the learned schedule gives
  the same vertex data and iteration count by construction.
* warm-start head -- per-vertex log in/out-degree (+ graph size) ->
  log(N * rank) of the converged precision-form PageRank; a run then starts
  from the prediction and iterates to the same tolerance.

``python -m graphreduce_gb300.learn train --out DIR`` trains both heads on
200 seeded R-MAT graphs (scales 14-20, seeds 100-299, (a, b, c) jittered by
up to 0.05) and writes DIR/schedule_head.npz and DIR/warm_start_head.npz;
``... evaluate --models DIR`` compares them with the heuristic / uniform
start on held-out graphs and prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import sys
import time
from pathlib import Path

import numpy as np

from . import _lib as L
from .engine import GASEngineGPU, initial_vertex_data
from .graph import EdgeList

DATA = Path(__file__).resolve().parent / "data"


def _torch():
    import torch
    return torch


class MLP:
    """A gas_mlp model: n_in -> 64 -> 64 -> n_out (ReLU), trained on the GPU."""

    def __init__(self, n_in: int, n_out: int, seed: int = 0):
        h = C.c_void_p()
        L.call("gas_mlp_create", n_in, n_out, seed, C.byref(h))
        self._h = h.value
        self.n_in, self.n_out = n_in, n_out

    @property
    def handle(self) -> int:
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            L.load().gas_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_params(self) -> int:
        return int(L.load().gas_mlp_num_params(self._h))

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        L.call("gas_mlp_get_params", self._h, out.ctypes.data)
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.shape == (self.n_params,)
        L.call("gas_mlp_set_params", self._h, p.ctypes.data)

    @staticmethod
    def _ptr(t):
        return None if t is None else t.data_ptr()

    def gradients(self, x, y=None, t=None, w=None):
        """Loss and gradient of all parameters for a device batch."""
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        L.call("gas_mlp_gradients", self._h, x.data_ptr(), self._ptr(y), self._ptr(t),
               self._ptr(w), x.shape[0], g.ctypes.data, C.byref(loss), None)
        return g, loss.value

    def train_step(self, x, y=None, t=None, w=None, lr: float = 1e-3) -> float:
        loss = C.c_float()
        L.call("gas_mlp_train_step", self._h, x.data_ptr(), self._ptr(y), self._ptr(t),
               self._ptr(w), x.shape[0], C.c_float(lr), C.byref(loss), None)
        return loss.value

    def forward(self, x):
        torch = _torch()
        out = torch.empty((x.shape[0], self.n_out), dtype=torch.float32, device=x.device)
        L.call("gas_mlp_forward", self._h, x.data_ptr(), x.shape[0], out.data_ptr(), None)
        torch.cuda.synchronize()
        return out

    def save(self, path, **meta):
        np.savez(path, params=self.params(), n_in=self.n_in, n_out=self.n_out,
                 meta=json.dumps(meta))

    @classmethod
    def load(cls, path) -> "MLP":
        with np.load(path) as z:
            m = cls(int(z["n_in"]), int(z["n_out"]))
            m.set_params(z["params"])
        return m


# ---------------------------------------------------------------------------
# schedule head
# ---------------------------------------------------------------------------
def schedule_features(rec, nV: int, nE: int, weighted: bool) -> np.ndarray:
    """The device's feature function (gas_schedule_features) on one record."""
    out = np.zeros(L.GAS_SCHED_FEATURES, np.float32)
    L.load().gas_schedule_features(C.byref(rec), nV, nE, int(weighted), out.ctypes.data)
    return out


def training_graph(seed: int) -> EdgeList:
    """R-MAT of scale 14 + seed % 7, quadrant probabilities (0.57, 0.19, 0.19,
    0.05) jittered by U(-0.05, 0.05) each from the seed (floored at 0.01 and
    renormalised), symmetrised, weights U[1,64]."""
    rng = np.random.default_rng(seed)
    q = np.array([0.57, 0.19, 0.19, 0.05]) + rng.uniform(-0.05, 0.05, 4)
    q = np.maximum(q, 0.01)
    q /= q.sum()
    a, b, c = q[:3].tolist()
    scale = 14 + seed % 7
    el = EdgeList.rmat(scale, 16, a, b, c, seed=seed, symmetrize=True)
    return el.with_uniform_weights(1, 64, seed)


def _timed_runs(eng, program, el, source, schedule, repeats=2):
    best = None
    for _ in range(repeats):
        vd = initial_vertex_data(program, el.nV, source)
        eng.upload_vertex_data(vd)
        eng.setActive(0, el.nV)
        st = eng.run_schedule(schedule, max_iterations=el.nV + 2)
        tr = eng.trace()
        d = np.array([r.t_end_ns - r.t_start_ns for r in tr], np.float64)
        best = d if best is None else np.minimum(best, d)
    return tr, best, st


def schedule_samples(el: EdgeList, program: str, source: int):
    """(features, label pull-faster, |t_push - t_pull| ns) per iteration."""
    eng = GASEngineGPU(program)
    vd = initial_vertex_data(program, el.nV, source)
    eng.setGraph(el.nV, vd, el.nE, el.weights if program == "sssp" else None, el.src, el.dst)
    eng.set_trace(True)
    tr_push, t_push, st_push = _timed_runs(eng, program, el, source, "push")
    tr_pull, t_pull, st_pull = _timed_runs(eng, program, el, source, "pull")
    eng.close()
    if st_push.iterations != st_pull.iterations:
        raise AssertionError("push and pull runs took different iteration counts")
    X, y, w = [], [], []
    for rp, rl, a, b in zip(tr_push, tr_pull, t_push, t_pull):
        if rp.n_queue != rl.n_queue or rp.n_edges_out != rl.n_edges_out:
            raise AssertionError("push and pull runs saw different frontiers")
        X.append(schedule_features(rp, el.nV, el.nE, program == "sssp"))
        y.append(1 if b < a else 0)
        w.append(abs(a - b))
    return np.array(X, np.float32), np.array(y, np.int32), np.array(w, np.float64)


def train_classifier(X, y, w, epochs=400, lr=2e-3, batch=256, seed=0) -> MLP:
    torch = _torch()
    dev = torch.device("cuda", 0)
    w = w / max(1e-12, w.mean())
    Xd = torch.from_numpy(X).to(dev)
    yd = torch.from_numpy(y).to(dev)
    wd = torch.from_numpy(w.astype(np.float32)).to(dev)
    m = MLP(L.GAS_SCHED_FEATURES, 2, seed)
    rng = np.random.default_rng(seed)
    n = X.shape[0]
    for _ in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).to(dev)
        for i in range(0, n, batch):
            idx = perm[i:i + batch]
            m.train_step(Xd[idx].contiguous(), yd[idx].contiguous(), None,
                         wd[idx].contiguous(), lr)
    return m


def weighted_accuracy(m: MLP, X, y, w) -> float:
    torch = _torch()
    out = m.forward(torch.from_numpy(X).to("cuda")).cpu().numpy()
    pred = (out[:, 1] > out[:, 0]).astype(np.int32)
    return float((w * (pred == y)).sum() / max(1e-12, w.sum()))


# ---------------------------------------------------------------------------
# warm-start head
# ---------------------------------------------------------------------------
def warm_features(el: EdgeList) -> np.ndarray:
    indeg, outdeg = el.in_degree(), el.out_degree()
    f = np.zeros((el.nV, L.GAS_WARM_FEATURES), np.float32)
    f[:, 0] = np.log2(1.0 + indeg) / 32.0
    f[:, 1] = np.log2(1.0 + outdeg) / 32.0
    f[:, 2] = np.float32(np.log2(1.0 + el.nV) / 32.0)
    f[:, 3] = np.float32(np.log2(1.0 + el.nE / max(1, el.nV)) / 8.0)
    return f


def warm_samples(el: EdgeList, per_graph: int, seed: int):
    eng = GASEngineGPU("pagerank")
    vd = initial_vertex_data("pagerank", el.nV, 0, el.out_degree())
    eng.setGraph(el.nV, vd, el.nE, None, el.src, el.dst)
    ranks, _ = eng.pagerank_precision(0.85, 1e-6)
    eng.close()
    X = warm_features(el)
    r = np.maximum(ranks.astype(np.float64), 1e-30)
    t = np.log(r * el.nV).astype(np.float32)
    # vertices drawn in proportion to their rank: the squared log error is
    # then weighted like the vertex's share of the L1 error of the start
    p = r / r.sum()
    idx = np.random.default_rng(seed).choice(el.nV, size=per_graph, replace=True, p=p)
    return X[idx], t[idx]


def train_regressor(X, t, epochs=30, lr=1e-3, batch=512, seed=0) -> MLP:
    torch = _torch()
    dev = torch.device("cuda", 0)
    Xd = torch.from_numpy(X).to(dev)
    td = torch.from_numpy(t).to(dev)
    m = MLP(L.GAS_WARM_FEATURES, 1, seed)
    rng = np.random.default_rng(seed)
    n = X.shape[0]
    for _ in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).to(dev)
        for i in range(0, n, batch):
            idx = perm[i:i + batch]
            m.train_step(Xd[idx].contiguous(), None, td[idx].contiguous(), None, lr)
    return m


# ---------------------------------------------------------------------------
# commands
# ---------------------------------------------------------------------------
def train(out: Path, n_graphs: int = 200, log=print) -> dict:
    out.mkdir(parents=True, exist_ok=True)
    t0 = time.time()
    Xs, ys, ws, Xw, tw = [], [], [], [], []
    for k in range(n_graphs):
        seed = 100 + k
        el = training_graph(seed)
        src = int(el.sample_sources(1, seed)[0])
        for program in ("sssp", "cc"):
            X, y, w = schedule_samples(el, program, src)
            Xs.append(X), ys.append(y), ws.append(w)
        d = EdgeList.rmat(14 + seed % 7, 16, seed=seed, symmetrize=False)
        a, b = warm_samples(d, 2048, seed)
        Xw.append(a), tw.append(b)
        if k % 20 == 0:
            log(f"graph {k}: scale {14 + seed % 7}, {time.time() - t0:.0f}s")
    X, y, w = np.concatenate(Xs), np.concatenate(ys), np.concatenate(ws)
    sched = train_classifier(X, y, w)
    acc = weighted_accuracy(sched, X, y, w)
    base_pred = (X[:, 4] * 4 > 1.0).astype(np.int32)  # the AUTO rule: pull if share > 1/4
    base_acc = float((w * (base_pred == y)).sum() / w.sum())
    sched.save(out / "schedule_head.npz", samples=int(len(y)), weighted_accuracy=acc,
               heuristic_weighted_accuracy=base_acc)
    Xw, tw = np.concatenate(Xw), np.concatenate(tw)
    warm = train_regressor(Xw, tw)
    torch = _torch()
    pred = warm.forward(torch.from_numpy(Xw).to("cuda")).cpu().numpy()[:, 0]
    mse = float(np.mean((pred - tw) ** 2))
    warm.save(out / "warm_start_head.npz", samples=int(len(tw)), mse=mse,
              baseline_mse=float(np.mean(tw ** 2)))
    res = {"schedule_samples": int(len(y)), "schedule_weighted_accuracy": acc,
           "heuristic_weighted_accuracy": base_acc, "warm_samples": int(len(tw)),
           "warm_mse": mse, "uniform_mse": float(np.mean(tw ** 2)),
           "seconds": time.time() - t0}
    log(json.dumps(res))
    return res


def _time_run(eng, program, el, source, schedule, repeats=3):
    torch = _torch()
    best, st = None, None
    vd = initial_vertex_data(program, el.nV, source)
    for _ in range(repeats):
        eng.upload_vertex_data(vd)
        eng.setActive(0, el.nV)
        torch.cuda.synchronize()
        t = time.perf_counter()
        st = eng.run_schedule(schedule, max_iterations=el.nV + 2)
        dt = time.perf_counter() - t
        best = dt if best is None else min(best, dt)
    return best, st


def evaluate(models: Path, scale: int = 24, log=print) -> dict:
    sched = MLP.load(models / "schedule_head.npz")
    warm = MLP.load(models / "warm_start_head.npz")
    out = {}
    graphs = {
        f"rmat{scale}": lambda: EdgeList.rmat(scale, 16, seed=5, symmetrize=True),
        "er16M": lambda: EdgeList.erdos_renyi(1 << 24, 8 << 24, seed=5, symmetrize=True),
    }
    for name, make in graphs.items():
        el = make().with_uniform_weights(1, 64, 5)
        src = int(el.sample_sources(1, 5)[0])
        row = {"V": el.nV, "E": el.nE}
        for program in ("sssp", "cc"):
            eng = GASEngineGPU(program)
            vd = initial_vertex_data(program, el.nV, src)
            eng.setGraph(el.nV, vd, el.nE, el.weights if program == "sssp" else None,
                         el.src, el.dst)
            eng.set_schedule_model(sched)
            res = {}
            outs = {}
            for s in ("auto", "learned", "push", "pull"):
                t, st = _time_run(eng, program, el, src, s)
                host = np.empty(el.nV, np.int32)
                eng.download_vertex_data(host)
                outs[s] = host
                res[s] = {"ms": round(1e3 * t, 3), "iterations": st.iterations,
                          "pull_iters": st.pull_iters}
            res["identical_outputs"] = all(np.array_equal(outs["auto"], o) for o in outs.values())
            res["learned_speedup_vs_auto"] = round(res["auto"]["ms"] / res["learned"]["ms"], 4)
            row[program] = res
            eng.close()
        d = (EdgeList.rmat(scale, 16, seed=4, symmetrize=False) if name.startswith("rmat")
             else EdgeList.erdos_renyi(1 << 24, 16 << 24, seed=5, symmetrize=False))
        eng = GASEngineGPU("pagerank")
        vd = initial_vertex_data("pagerank", d.nV, 0, d.out_degree())
        eng.setGraph(d.nV, vd, d.nE, None, d.src, d.dst)
        r_uni, st_uni = eng.pagerank_precision_from(None)
        init = eng.pagerank_warm_start(warm)
        r_warm, st_warm = eng.pagerank_precision_from(init)
        eng.close()
        row["pagerank"] = {"uniform_iterations": st_uni.iterations,
                           "warm_iterations": st_warm.iterations,
                           "l1_between_results": float(np.abs(r_uni.astype(np.float64) -
                                                              r_warm).sum()),
                           "uniform_residual": st_uni.residual,
                           "warm_residual": st_warm.residual}
        out[name] = row
        log(json.dumps({name: row}))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m graphreduce_gb300.learn")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", type=Path, default=DATA)
    t.add_argument("--graphs", type=int, default=200)
    e = sub.add_parser("evaluate")
    e.add_argument("--models", type=Path, default=DATA)
    e.add_argument("--scale", type=int, default=24)
    a = ap.parse_args(argv)
    log = lambda *x: print(*x, file=sys.stderr, flush=True)  # noqa: E731
    if a.cmd == "train":
        print(json.dumps(train(a.out, a.graphs, log)))
    else:
        print(json.dumps(evaluate(a.models, a.scale, log)))


if __name__ == "__main__":
    main()
