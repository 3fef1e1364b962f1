"""Benchmark of the GAS hot path on the scale-22 workload.

Workload (one "step"): SSSP from 8 sources and CC on an R-MAT graph of scale
22 (4,194,304 vertices, edge factor 16, (a,b,c,d) = (0.57,0.19,0.19,0.05),
seed 2, symmetrised, self loops and duplicates removed); SSSP weights
uniform in [1,64] (seed 3, both directions equal); sources drawn uniformly
from the largest component (seed 2); CC on the same graph plus 4,096
disjoint 32x32 4-neighbour grid islands.  Synthetic data: the reference's
real-world datasets are not available.

Metric: GTEPS with the reference's definition (sssp.cu:202-211): for every
run, the sum of out-degrees of the vertices it reached, divided by time
(for CC every vertex is reached, so a run counts all its edges).

The engine under test is the learned-schedule, batched one: the 8 SSSP
sources run as the 8 lanes of one multi-source SSSP launch (per lane
bit-exact with, and as many iterations as, one run per source; checked
every time the bench starts), CC runs through the engine with the learned
schedule.  The same step with one SSSP run per source ("comparisons") and
the plain fixed-heuristic form ("plain") are timed beside it.

  value  -- device-resident: graph and initial vertex states already in HBM,
            timed with CUDA events on the engine's stream.
  e2e    -- through the public Python API with pinned host buffers: every
            input goes up (the CC labels; the SSSP source ids -- the batched
            run builds its initial distances on the device) and every result
            comes down (the [V][8] distances, the CC labels) inside the
            timed region.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SCALE = 22
EDGE_FACTOR = 16
RMAT_ABC = (0.57, 0.19, 0.19)
GRAPH_SEED, WEIGHT_SEED, SOURCE_SEED = 2, 3, 2
N_SOURCES = 8
N_ISLANDS, ISLAND_SIDE = 4096, 32
METRIC = "GTEPS (SSSP x8 + CC, R-MAT scale {scale})"
MAX_ITERS = 20000  # far above any run of this workload; bounds a device loop
# Per-launch DRAM bytes (read + write) of the dominant kernel, by (kernel,
# scale, edge placement, schedule): one-pass ncu metrics over every launch of
# that kernel in one step, captured with
#   GAS_HOST_LOOP=1 ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,\
#     dram__bytes_write.sum --clock-control none --csv --log-file launches.csv \
#     python bench.py --launch-list --no-cpu-baseline
# (k_mss_push: 11 launches, 8.95 GB in all).
PUSH_TRAFFIC = {("mss_push", 22, "device", "learned"): 814.0e6}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_workload(scale):
    from graphreduce_gb300.graph import EdgeList
    t = time.time()
    base = EdgeList.rmat(scale, EDGE_FACTOR, *RMAT_ABC, seed=GRAPH_SEED, symmetrize=True)
    ssp = base.with_uniform_weights(1, 64, WEIGHT_SEED)
    sources = ssp.sample_sources(N_SOURCES, SOURCE_SEED)
    ccg = base.with_grid_islands(N_ISLANDS, ISLAND_SIDE)
    log(f"workload: scale {scale}: V={ssp.nV} E={ssp.nE}; CC graph V={ccg.nV} E={ccg.nE}; "
        f"generated in {time.time() - t:.1f}s")
    return ssp, sources, ccg


def max_over_ranks(ms, world, device):
    """The step time of the slowest rank (replicas: every rank times its own
    copy of the workload); a barrier after it keeps the ranks in step."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def whole_job_value(units_per_rank, world, ms_per_step):
    """GTEPS of the whole job: every rank processes units_per_rank edges per
    step, all within the slowest rank's step time."""
    return world * units_per_rank / (ms_per_step * 1e-3) / 1e9


def edges_visited(el_outdeg, vd, unreached):
    return int(el_outdeg[vd != unreached].sum(dtype=np.int64))


def config_dict(scale, extra=None):
    d = {"workload": f"sssp8+cc rmat-s{scale}-ef{EDGE_FACTOR}-sym+{N_ISLANDS}x{ISLAND_SIDE}^2-islands",
         "graph": {"scale": scale, "edge_factor": EDGE_FACTOR, "abcd": [*RMAT_ABC, 0.05],
                   "seed": GRAPH_SEED, "symmetrized": True, "weights": "uniform[1,64] seed 3",
                   "sources": f"{N_SOURCES} uniform from the largest component, seed {SOURCE_SEED}",
                   "cc_islands": f"{N_ISLANDS} x {ISLAND_SIDE}x{ISLAND_SIDE} grids"},
         "l2": "inputs larger than L2 (CSR+CSC+weights > 2 GB vs 129 MB L2)",
         "parallelism": "replicas"}
    if extra:
        d.update(extra)
    return d


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=self.file, stderr=subprocess.DEVNULL)
            # nvidia-smi takes a while to start: let its first sample land
            # before the timed region begins
            t0 = time.time()
            while time.time() - t0 < 3.0 and self.proc.poll() is None:
                self.file.flush()
                if Path(self.file.name).stat().st_size > 0:
                    break
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.file:
            return None
        try:
            rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
            os.unlink(self.file.name)
        except Exception:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch

    import graphreduce_gb300 as gg
    from graphreduce_gb300.engine import SSSP_GATHER_ZERO, initial_vertex_data

    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    gg.load()

    ssp, sources, ccg = make_workload(args.scale)
    out_sssp = ssp.out_degree()
    out_cc = ccg.out_degree()
    batched = args.sssp == "batched"

    model = None
    if args.schedule == "learned":
        from graphreduce_gb300.learn import DATA, MLP
        model = MLP.load(DATA / "schedule_head.npz")  # trained schedule head (required)

    t = time.time()
    e_s = gg.GASEngineGPU("sssp")
    e_c = gg.GASEngineGPU("cc")
    for e in (e_s, e_c):
        e.set_edge_placement(args.edges)
    vd_s = initial_vertex_data("sssp", ssp.nV, int(sources[0]))
    e_s.setGraph(ssp.nV, vd_s, ssp.nE, ssp.weights, ssp.src, ssp.dst, sp)
    vd_c = initial_vertex_data("cc", ccg.nV)
    e_c.setGraph(ccg.nV, vd_c, ccg.nE, None, ccg.src, ccg.dst, sp)
    bat = None
    if batched:
        # the 8 sources as the 8 lanes of one multi-source SSSP run
        bat = gg.Batch()
        bat.add_graph(ssp.nV, ssp.src, ssp.dst, ssp.weights)
        bat.build(sp)
    log(f"setGraph (CSR/CSC build + upload) {time.time() - t:.1f}s")
    if model is not None:
        e_s.set_schedule_model(model)
        e_c.set_schedule_model(model)

    # initial vertex states resident in HBM (value) and in pinned host memory (e2e)
    init_s = [torch.from_numpy(initial_vertex_data("sssp", ssp.nV, int(s))) for s in sources]
    init_c = torch.from_numpy(initial_vertex_data("cc", ccg.nV))
    dev_s = [x.to(dev) for x in init_s]
    dev_c = init_c.to(dev)
    pin_s = [x.pin_memory() for x in init_s]
    pin_c = init_c.pin_memory()
    res_s = [torch.empty(ssp.nV, dtype=torch.int32).pin_memory() for _ in sources]
    res_c = torch.empty(ccg.nV, dtype=torch.int32).pin_memory()
    lane_src = np.asarray(sources, np.int32)[None, :]
    dist_dev = torch.empty((ssp.nV, len(sources)), dtype=torch.int32, device=dev)
    dist_pin = torch.empty((ssp.nV, len(sources)), dtype=torch.int32).pin_memory()
    torch.cuda.synchronize()

    launches = [0]
    iters = {"sssp": [], "cc": 0}

    def sssp_batched(e2e):
        r = bat.run(sssp_sources=lane_src, max_sssp_iterations=MAX_ITERS,
                    dist_out=(dist_pin if e2e else dist_dev).data_ptr(), stream=sp)
        iters["sssp"] = [int(r.stats.sssp_lane_iterations[k]) for k in range(len(sources))]
        launches[0] += r.stats.kernel_launches

    def sssp_sequential(e2e, schedule):
        iters["sssp"] = []
        for k in range(len(sources)):
            e_s.upload_vertex_data_ptr(pin_s[k].data_ptr() if e2e else dev_s[k].data_ptr(), sp)
            e_s.setActive(0, ssp.nV, sp)
            st = e_s.run_schedule(schedule, max_iterations=MAX_ITERS, stream=sp)
            iters["sssp"].append(st.iterations)
            launches[0] += st.kernel_launches + 1
            if e2e:
                e_s.download_vertex_data_ptr(res_s[k].data_ptr(), sp)

    # end to end with batched lanes, copies overlap compute on a second
    # stream: the CC labels go up while the SSSP lanes run, the distances
    # come down while CC runs; the step ends when both streams are done
    cstream = torch.cuda.Stream(device=dev)
    csp = cstream.cuda_stream
    prev_done = torch.cuda.Event()

    def one_step(e2e, schedule=args.schedule, use_batch=batched):
        launches[0] = 0
        if e2e and use_batch:
            cstream.wait_event(prev_done)   # the previous step's results are down
            e_c.upload_vertex_data_ptr(pin_c.data_ptr(), csp)
            up = torch.cuda.Event()
            up.record(cstream)
            sssp_batched(False)
            lanes_done = torch.cuda.Event()
            lanes_done.record(stream)
            cstream.wait_event(lanes_done)
            with torch.cuda.stream(cstream):
                dist_pin.copy_(dist_dev, non_blocking=True)
            down = torch.cuda.Event()
            down.record(cstream)
            stream.wait_event(up)
        elif use_batch:
            sssp_batched(e2e)
        else:
            sssp_sequential(e2e, schedule)
        if not (e2e and use_batch):
            e_c.upload_vertex_data_ptr(pin_c.data_ptr() if e2e else dev_c.data_ptr(), sp)
        e_c.setActive(0, ccg.nV, sp)
        st = e_c.run_schedule(schedule, max_iterations=MAX_ITERS, stream=sp)
        iters["cc"] = st.iterations
        launches[0] += st.kernel_launches + 1
        if e2e:
            e_c.download_vertex_data_ptr(res_c.data_ptr(), sp)
        if e2e and use_batch:
            stream.wait_event(down)
            prev_done.record(stream)

    if args.launch_list:
        # one device-resident step and nothing else (for an ncu launch list)
        one_step(e2e=False)
        torch.cuda.synchronize()
        return {"launch_list": True, "gpu_launches": launches[0]}, None

    # correctness of this exact workload + units per step
    one_step(e2e=True)
    torch.cuda.synchronize()
    if batched:
        for k in range(len(sources)):
            res_s[k].copy_(dist_pin[:, k])
    ev_units = 0
    for k in range(len(sources)):
        ev_units += edges_visited(out_sssp, res_s[k].numpy(), SSSP_GATHER_ZERO)
    ev_units += edges_visited(out_cc, res_c.numpy(), -12345)  # every CC vertex is reached
    first_sssp = res_s[0].numpy().copy()
    if batched:
        # the lanes equal one SSSP per source through the engine (bit-exact)
        one_step(e2e=True, use_batch=False)
        torch.cuda.synchronize()
        for k in range(len(sources)):
            if not np.array_equal(res_s[k].numpy(), dist_pin[:, k].numpy()):
                raise SystemExit(f"batched SSSP lane {k} differs from the single-source run")

    def timed(e2e, steps, warmup, schedule=args.schedule, use_batch=batched):
        for _ in range(warmup):
            one_step(e2e, schedule, use_batch)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        start.record(stream)
        for _ in range(steps):
            one_step(e2e, schedule, use_batch)
        end.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        ms = start.elapsed_time(end)
        ms = max_over_ranks(ms, world, dev)
        return ms / steps, wall / steps

    with ClockSampler(torch.cuda.current_device()) as clk:
        ms_step, _ = timed(False, args.steps, args.warmup)
    clocks = clk.summary()
    launches_per_step = launches[0]
    iters_step = {"sssp": list(iters["sssp"]), "cc": iters["cc"]}
    ms_e2e, _ = timed(True, max(1, args.steps), 1)
    comparisons = {}
    # the same step with one SSSP run per source (learned schedule), and the
    # plain form: one run per source under the fixed heuristic (AUTO)
    if batched:
        ms_seq, _ = timed(False, args.steps, args.warmup, args.schedule, False)
        comparisons["sequential_sources"] = {
            "schedule": args.schedule, "ms_per_step": round(ms_seq, 3),
            "value": round(world * ev_units / (ms_seq * 1e-3) / 1e9, 4),
            "speedup_of_headline": round(ms_seq / ms_step, 4)}
    ms_plain, _ = timed(False, args.steps, args.warmup, "auto", False)
    plain = {"schedule": "auto (fixed heuristic), one SSSP run per source",
             "ms_per_step": round(ms_plain, 3),
             "value": round(world * ev_units / (ms_plain * 1e-3) / 1e9, 4),
             "speedup_of_headline": round(ms_plain / ms_step, 4)}

    value = whole_job_value(ev_units, world, ms_step)
    e2e = whole_job_value(ev_units, world, ms_e2e)
    if batched:  # sources in, the [V][8] distances and the CC labels out
        h2d = len(sources) * 4 + ccg.nV * 4
        d2h = (len(sources) * ssp.nV + ccg.nV) * 4
    else:
        h2d = (len(sources) * ssp.nV + ccg.nV) * 4
        d2h = h2d

    # per-algorithm split and the dominant kernel's roofline (untimed pass)
    split = per_algo_split(e_s, e_c, bat, dev_s, dev_c, ssp, ccg, out_sssp, sources,
                           lane_src, dist_dev, args.schedule, sp, stream)
    roof = kernel_roofline(e_s, e_c, bat, dev_s, dev_c, ssp, ccg, lane_src, dist_dev,
                           args.schedule, sp)
    traffic = PUSH_TRAFFIC.get((roof["kernel_key"], args.scale, args.edges, args.schedule))
    if traffic:
        roof["traffic"] = traffic
        roof["traffic_source"] = "ncu dram bytes per launch of this kernel, same workload"
    del roof["kernel_key"]
    peak, peak_kind = measured_peaks()
    roof["peak"] = peak
    roof["frac"] = roof["achieved"] / peak
    roof["peak_source"] = peak_kind

    result = {
        "metric": METRIC.format(scale=args.scale), "value": round(value, 4), "unit": "GTEPS",
        "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded R-MAT + grid islands; reference datasets unavailable)",
        "config": config_dict(args.scale, {"schedule": args.schedule, "edges": args.edges,
                                           "sssp": ("8 sources as 8 lanes of one batched "
                                                    "multi-source run" if batched else
                                                    "one run per source"),
                                           "edges_visited_per_step": ev_units,
                                           "iterations": iters_step}),
        "e2e": {"value": round(e2e, 4), "unit": "GTEPS", "ms_per_step": round(ms_e2e, 3),
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "copies": ("pinned host buffers; CC labels up while the SSSP lanes run and "
                           "distances down while CC runs (second stream)" if batched else
                           "pinned host buffers, on the compute stream")},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roof,
        "algos": split,
        "plain": plain,
        "comparisons": comparisons,
        "clocks": clocks,
    }
    return result, (ssp, sources, out_sssp, first_sssp)


def per_algo_split(e_s, e_c, bat, dev_s, dev_c, ssp, ccg, out_sssp, sources, lane_src,
                   dist_dev, schedule, sp, stream):
    import torch
    out = {}
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    host = np.empty(ssp.nV, np.int32)
    ev = 0
    for k in range(len(sources)):
        e_s.upload_vertex_data_ptr(dev_s[k].data_ptr(), sp)
        e_s.setActive(0, ssp.nV, sp)
        e_s.run_schedule(schedule, max_iterations=MAX_ITERS, stream=sp)
        e_s.download_vertex_data(host, sp)
        ev += edges_visited(out_sssp, host, 2**31 - 1 - 100000)
    torch.cuda.synchronize()
    a.record(stream)
    its = []
    for k in range(len(sources)):
        e_s.upload_vertex_data_ptr(dev_s[k].data_ptr(), sp)
        e_s.setActive(0, ssp.nV, sp)
        its.append(e_s.run_schedule(schedule, max_iterations=MAX_ITERS, stream=sp).iterations)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    out["sssp_sequential"] = {"ms_per_source": round(ms / len(sources), 3),
                              "gteps": round(ev / (ms * 1e-3) / 1e9, 4), "iterations": its}
    if bat is not None:
        a.record(stream)
        r = bat.run(sssp_sources=lane_src, max_sssp_iterations=MAX_ITERS,
                    dist_out=dist_dev.data_ptr(), stream=sp)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        out["sssp_batched"] = {"ms_8_sources": round(ms, 3),
                               "gteps": round(ev / (ms * 1e-3) / 1e9, 4),
                               "iterations": r.stats.sssp_iterations,
                               "union_edges_pushed": int(r.stats.sssp_edges)}
    a.record(stream)
    e_c.upload_vertex_data_ptr(dev_c.data_ptr(), sp)
    e_c.setActive(0, ccg.nV, sp)
    it = e_c.run_schedule(schedule, max_iterations=MAX_ITERS, stream=sp).iterations
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    out["cc"] = {"ms": round(ms, 3), "gteps": round(ccg.nE / (ms * 1e-3) / 1e9, 4),
                 "iterations": it}
    return out


def kernel_roofline(e_s, e_c, bat, dev_s, dev_c, ssp, ccg, lane_src, dist_dev, schedule, sp):
    """One extra pass of the step's runs with kernel profiling on: the
    engines bracket every push / dense-pull launch (and the batch every
    multi-source SSSP push) with CUDA events on the run's stream and
    accumulate its algorithmic bytes (per edge: index, weight for SSSP, and
    the state, row or membership word it reads; per frontier entry or row:
    its offsets and state).  The dominant kernel is the one with the largest
    total time."""
    import torch
    kinds = {}

    def add(key, p, name):
        ms, by, n = (getattr(p, f"{name}_ms"), getattr(p, f"{name}_bytes"),
                     getattr(p, f"{name}_launches"))
        k = kinds.setdefault(key, {"ms": 0.0, "bytes": 0, "launches": 0})
        k["ms"] += ms
        k["bytes"] += by
        k["launches"] += n

    if bat is None:  # one SSSP run per source through the engine
        e_s.set_profiling(True)
        e_s.profile(reset=True)
        for k in range(len(dev_s)):
            e_s.upload_vertex_data_ptr(dev_s[k].data_ptr(), sp)
            e_s.setActive(0, ssp.nV, sp)
            e_s.run_schedule(schedule, max_iterations=MAX_ITERS, stream=sp)
        torch.cuda.synchronize()
        ps = e_s.profile()
        e_s.set_profiling(False)
        add("push", ps, "push")
        add("pull", ps, "pull")
    e_c.set_profiling(True)
    e_c.profile(reset=True)
    e_c.upload_vertex_data_ptr(dev_c.data_ptr(), sp)
    e_c.setActive(0, ccg.nV, sp)
    e_c.run_schedule(schedule, max_iterations=MAX_ITERS, stream=sp)
    torch.cuda.synchronize()
    pc = e_c.profile()
    e_c.set_profiling(False)
    add("push", pc, "push")
    add("pull", pc, "pull")
    if bat is not None:
        bat.set_profiling(True)
        bat.profile(reset=True)
        bat.run(sssp_sources=lane_src, max_sssp_iterations=MAX_ITERS,
                dist_out=dist_dev.data_ptr(), stream=sp)
        torch.cuda.synchronize()
        add("mss_push", bat.profile(), "push")
        bat.set_profiling(False)
    for k in kinds.values():
        k["achieved_gbs"] = (k["bytes"] / (k["ms"] * 1e-3) / 1e9) if k["ms"] > 0 else 0.0
    dom = max(kinds, key=lambda k: kinds[k]["ms"])
    d = kinds[dom]
    return {"kernel": {"pull": "k_pull (CC dense pull, warp-slab)",
                       "push": "k_push (frontier push, warp-slab)",
                       "mss_push": "k_mss_push (8-lane multi-source SSSP push, warp-slab)"}[dom],
            "kernel_key": dom,
            "bound": "hbm", "achieved": round(d["achieved_gbs"], 1), "unit": "GB/s",
            "traffic": None, "launches": d["launches"],
            "algorithmic_bytes_per_launch": int(d["bytes"] / max(1, d["launches"])),
            "avg_launch_ms": round(d["ms"] / max(1, d["launches"]), 4),
            "by_kernel": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv)
                              for kk, vv in v.items()} for k, v in kinds.items()}}


# ---------------------------------------------------------------------------
# batched lanes on one scale-24 graph: 16 BFS sources, 16 PPR seeds
# ---------------------------------------------------------------------------
LANES24 = 16


def run_lanes24(args):
    """The batched engine on single R-MAT scale-24 graphs: multi-source BFS
    (16 sources, the symmetrised graph of the headline at scale 24, seed 2)
    and multi-seed personalized PageRank (16 seeds, the directed graph of the
    PageRank workload, seed 4), each against the same instances run one by
    one on the single-graph engine.  Roofline: BFS from the profiled pushes
    (per union edge index + visited + next words, per queue entry 12 B); PPR
    from the autotuner's per-iteration time (per edge index + 16 lanes of the
    source's contribution, per vertex offsets, seed mask, old and new rank and
    new contribution)."""
    import torch

    import graphreduce_gb300 as gg
    from graphreduce_gb300.engine import initial_vertex_data
    from graphreduce_gb300.graph import EdgeList
    from graphreduce_gb300.learn import DATA, MLP

    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    scale, L = args.pr_scale, LANES24
    peak, peak_kind = measured_peaks()
    model = MLP.load(DATA / "schedule_head.npz")

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        z = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        z.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(z) / steps

    out = {"metric": f"GTEPS (batched lanes on one R-MAT scale-{scale} graph: "
                     f"{L} BFS sources, {L} PPR seeds)", "unit": "GTEPS", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "dtype": "int32 (BFS), f32 two-sum + f64 residual (PPR)", "data": "synthetic"}

    # --- BFS ---------------------------------------------------------------
    el = EdgeList.rmat(scale, EDGE_FACTOR, *RMAT_ABC, seed=GRAPH_SEED, symmetrize=True)
    srcs = el.sample_sources(L, SOURCE_SEED).astype(np.int32)
    b = gg.Batch()
    b.add_graph(el.nV, el.src, el.dst)
    b.build(sp)
    depth_d = torch.empty((el.nV, L), dtype=torch.int32, device=dev)
    run_b = lambda: b.run(bfs_sources=srcs[None, :], depth_out=depth_d.data_ptr(), stream=sp)
    if args.launch_list:
        # one batched BFS run, then the first two sources one by one on the
        # single-graph engine (learned: the direction rule), and nothing else
        # (for an ncu launch list / capture)
        r = run_b()
        e = gg.GASEngineGPU("bfs")
        e.setGraph(el.nV, initial_vertex_data("bfs", el.nV), el.nE, None, el.src, el.dst, sp)
        e.set_schedule_model(model)
        init = torch.from_numpy(initial_vertex_data("bfs", el.nV)).to(dev)
        levels = []
        for src in srcs[:2]:
            e.upload_vertex_data_ptr(init.data_ptr(), sp)
            e.setActive(int(src), int(src) + 1, sp)
            st = e.run_schedule("learned", max_iterations=el.nV + 2, stream=sp)
            levels.append([st.iterations, st.push_iters, st.pull_iters])
        torch.cuda.synchronize()
        e.close()
        return {"launch_list": True, "bfs_levels": r.stats.bfs_iterations,
                "single_source": levels}
    run_b()
    depth = depth_d.cpu().numpy()
    od = el.out_degree().astype(np.int64)
    bfs_units = int(((depth >= 0) * od[:, None]).sum())
    with ClockSampler(torch.cuda.current_device()) as clk:
        ms_b = timed(run_b, args.steps, args.warmup)
    b.set_profiling(True)
    b.profile(reset=True)
    run_b()
    torch.cuda.synchronize()
    pb = b.profile()
    b.set_profiling(False)
    e = gg.GASEngineGPU("bfs")
    e.setGraph(el.nV, initial_vertex_data("bfs", el.nV), el.nE, None, el.src, el.dst, sp)
    e.set_schedule_model(model)
    init = torch.from_numpy(initial_vertex_data("bfs", el.nV)).to(dev)
    one = torch.empty(el.nV, dtype=torch.int32)

    def plain_bfs():
        for s in srcs:
            e.upload_vertex_data_ptr(init.data_ptr(), sp)
            e.setActive(int(s), int(s) + 1, sp)
            e.run_schedule("learned", max_iterations=el.nV + 2, stream=sp)

    e.upload_vertex_data_ptr(init.data_ptr(), sp)
    e.setActive(int(srcs[0]), int(srcs[0]) + 1, sp)
    e.run_schedule("learned", max_iterations=el.nV + 2, stream=sp)
    e.download_vertex_data(one.numpy(), sp)
    same = bool(np.array_equal(one.numpy(), depth[:, 0]))
    ms_plain_b = timed(plain_bfs, 1, 1)
    # the single-source engine's push roofline over the same 16 runs
    e.set_profiling(True)
    e.profile(reset=True)
    plain_bfs()
    torch.cuda.synchronize()
    pe = e.profile()
    e.set_profiling(False)
    e.close()
    b.close()
    ach1 = pe.push_bytes / (pe.push_ms * 1e-3) / 1e9 if pe.push_ms > 0 else 0.0
    ach = pb.push_bytes / (pb.push_ms * 1e-3) / 1e9 if pb.push_ms > 0 else 0.0
    out["bfs"] = {"graph": f"rmat-s{scale}-ef{EDGE_FACTOR}-sym seed {GRAPH_SEED}",
                  "V": el.nV, "E": el.nE, "lanes": L, "ms": round(ms_b, 3),
                  "gteps": round(bfs_units / (ms_b * 1e-3) / 1e9, 4),
                  "plain_one_by_one_ms": round(ms_plain_b, 3),
                  "speedup_vs_plain": round(ms_plain_b / ms_b, 3),
                  "lane0_equals_single_source_run": same,
                  "plain_push_roofline": {"kernel": "k_push (single-source BFS, learned)",
                                          "achieved": round(ach1, 1), "unit": "GB/s",
                                          "frac": round(ach1 / peak, 4),
                                          "launches": pe.push_launches,
                                          "pull_launches": pe.pull_launches},
                  "roofline": {"kernel": "k_ms_push (16-lane BFS push)", "bound": "hbm",
                               "achieved": round(ach, 1), "unit": "GB/s", "peak": peak,
                               "frac": round(ach / peak, 4), "peak_source": peak_kind,
                               "launches": pb.push_launches,
                               "push_share_of_run": round(pb.push_ms / ms_b, 3)}}
    del el, depth, depth_d
    clocks_b = clk.summary()

    # --- PPR ---------------------------------------------------------------
    d = EdgeList.rmat(scale, EDGE_FACTOR, *RMAT_ABC, seed=PR_SEED, symmetrize=False)
    seeds = d.sample_sources(L, 7).astype(np.int32)
    b = gg.Batch()
    b.add_graph(d.nV, d.src, d.dst)
    b.build(sp)
    piece, ms_iter = b.tune(L, PPR_DAMPING, 5, sp)
    rank_d = torch.empty((d.nV, L), dtype=torch.float32, device=dev)
    run_p = lambda: b.run(ppr_seeds=seeds[None, :], damping=PPR_DAMPING, tol=PPR_TOL,
                          rank_out=rank_d.data_ptr(), stream=sp)
    st = run_p().stats
    ms_p = timed(run_p, args.steps, args.warmup)
    p = gg.GASEngineGPU("pagerank")
    p.setGraph(d.nV, initial_vertex_data("pagerank", d.nV, 0, d.out_degree()), d.nE, None,
               d.src, d.dst, sp)
    outp = torch.empty(d.nV, dtype=torch.float32, device=dev)
    plain_iters = [0]

    def plain_ppr():
        plain_iters[0] = 0
        for s in seeds:
            _, pst = p.ppr_precision(int(s), PPR_DAMPING, PPR_TOL, out=outp.data_ptr(),
                                     stream=sp)
            plain_iters[0] += pst.iterations

    ms_plain_p = timed(plain_ppr, 1, 0)
    p.close()
    b.close()
    ppr_units = d.nE * L * st.ppr_iterations
    ppr_bytes = d.nE * (4 + 4 * L) + d.nV * (12 + 12 * L)
    ach = ppr_bytes / (ms_iter * 1e-3) / 1e9
    out["ppr"] = {"graph": f"rmat-s{scale}-ef{EDGE_FACTOR} directed seed {PR_SEED}",
                  "V": d.nV, "E": d.nE, "lanes": L, "iterations": st.ppr_iterations,
                  "ms": round(ms_p, 3), "gteps": round(ppr_units / (ms_p * 1e-3) / 1e9, 4),
                  "plain_one_by_one_ms": round(ms_plain_p, 3),
                  "plain_iterations": plain_iters[0],
                  "speedup_vs_plain": round(ms_plain_p / ms_p, 3),
                  "residual": st.ppr_residual,
                  "roofline": {"kernel": "PPR iteration (k_ppr_pieces + k_ppr_fix + k_ppr_finish)",
                               "bound": "hbm", "achieved": round(ach, 1), "unit": "GB/s",
                               "peak": peak, "frac": round(ach / peak, 4),
                               "peak_source": peak_kind, "piece_edges": piece,
                               "ms_per_iteration": round(ms_iter, 4),
                               "algorithmic_bytes_per_iteration": int(ppr_bytes)}}
    total_units = bfs_units + ppr_units
    out["value"] = round(total_units / ((ms_b + ms_p) * 1e-3) / 1e9, 4)
    out["ms_per_step"] = round(ms_b + ms_p, 3)
    out["clocks"] = clocks_b
    return out


# ---------------------------------------------------------------------------
# batched workload: 64 graphs x (16 BFS sources + 16 PPR seeds)
# ---------------------------------------------------------------------------
BATCH_GRAPHS, BATCH_LANES, BATCH_SEED = 64, 16, 6
BATCH_METRIC = "GTEPS (batched: 64 R-MAT graphs x (16 BFS + 16 PPR))"
PPR_DAMPING, PPR_TOL = 0.85, 1e-6
# DRAM bytes (read + write) of one PPR iteration of this workload (64 graphs,
# 16 lanes): one-pass ncu metrics over all 31 k_ppr_pieces and k_ppr_fix
# launches of a run (9.50 GB + 0.80 GB per iteration), captured with
#   GAS_HOST_LOOP=1 ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,\
#     dram__bytes_write.sum --clock-control none -k regex:"k_ppr_pieces|k_ppr_fix" \
#     python bench.py --workload batched --launch-list
PPR_TRAFFIC_64 = 10.30e9


def make_batched_workload(n_graphs=BATCH_GRAPHS):
    """Scale U[12,20], edge factor U[8,32] per graph (seed 6), symmetrised
    R-MAT; 16 BFS sources and 16 PPR seeds per graph, uniform over the
    graph's largest component (seeded per graph)."""
    from graphreduce_gb300.graph import EdgeList
    rng = np.random.default_rng(BATCH_SEED)
    scales = rng.integers(12, 21, n_graphs)
    efs = rng.integers(8, 33, n_graphs)
    t = time.time()
    graphs, srcs, seeds = [], [], []
    for g in range(n_graphs):
        el = EdgeList.rmat(int(scales[g]), int(efs[g]), *RMAT_ABC, seed=1000 + g,
                           symmetrize=True)
        graphs.append(el)
        srcs.append(el.sample_sources(BATCH_LANES, 2000 + g))
        seeds.append(el.sample_sources(BATCH_LANES, 3000 + g))
    log(f"batched workload: {n_graphs} graphs, V={sum(x.nV for x in graphs)} "
        f"E={sum(x.nE for x in graphs)}, generated in {time.time() - t:.1f}s")
    return graphs, np.stack(srcs).astype(np.int32), np.stack(seeds).astype(np.int32), \
        scales, efs


def run_batched(args):
    import torch

    import graphreduce_gb300 as gg
    from graphreduce_gb300.engine import initial_vertex_data

    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    graphs, srcs, seeds, scales, efs = make_batched_workload(args.batch_graphs)
    G, L = len(graphs), BATCH_LANES
    b = gg.Batch()
    for el in graphs:
        b.add_graph(el.nV, el.src, el.dst)
    t = time.time()
    b.build(sp)
    V, E = b.num_vertices, b.num_edges
    if args.launch_list:
        # one batch run and nothing else (for an ncu launch list / capture)
        r = b.run(srcs, seeds, PPR_DAMPING, PPR_TOL, piece_edges=256, stream=sp)
        torch.cuda.synchronize()
        return {"launch_list": True, "gpu_launches": r.stats.kernel_launches}
    piece, ms_iter = b.tune(L, PPR_DAMPING, 5, sp)
    log(f"batch build {time.time() - t:.1f}s; tuned piece {piece} edges, "
        f"{ms_iter:.3f} ms per PPR iteration")
    depth_d = torch.empty((V, L), dtype=torch.int32, device=dev)
    rank_d = torch.empty((V, L), dtype=torch.float32, device=dev)
    depth_h = torch.empty((V, L), dtype=torch.int32).pin_memory()
    rank_h = torch.empty((V, L), dtype=torch.float32).pin_memory()

    def step(e2e):
        if e2e:
            return b.run(srcs, seeds, PPR_DAMPING, PPR_TOL, depth_out=depth_h.data_ptr(),
                         rank_out=rank_h.data_ptr(), stream=sp)
        return b.run(srcs, seeds, PPR_DAMPING, PPR_TOL, depth_out=depth_d.data_ptr(),
                     rank_out=rank_d.data_ptr(), stream=sp)

    # units: BFS per (graph, lane) the out-degrees of the reached vertices;
    # PPR per (graph, lane) E_graph x iterations
    r = step(True)
    depth = depth_h.numpy()
    bfs_units = 0
    for g, el in enumerate(graphs):
        od = el.out_degree().astype(np.int64)
        d = depth[b.vertex_offset(g):b.vertex_offset(g) + el.nV]
        bfs_units += int(((d >= 0) * od[:, None]).sum())
    ppr_iters = r.stats.ppr_iterations
    ppr_units = int(sum(el.nE for el in graphs)) * L * ppr_iters

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        z = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        z.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(z) / steps

    with ClockSampler(torch.cuda.current_device()) as clk:
        ms = timed(lambda: step(False), args.steps, args.warmup)
    clocks = clk.summary()
    ms_e2e = timed(lambda: step(True), max(1, args.steps), 1)
    st = step(False).stats

    # BFS-only and PPR-only batch times (device-resident)
    ms_bfs = timed(lambda: b.run(srcs, None, depth_out=depth_d.data_ptr(), stream=sp),
                   args.steps, 1)
    ms_ppr = timed(lambda: b.run(None, seeds, PPR_DAMPING, PPR_TOL,
                                 rank_out=rank_d.data_ptr(), stream=sp), args.steps, 1)

    # the same instances run one by one on the plain single-graph engines
    from graphreduce_gb300.learn import DATA, MLP
    model = MLP.load(DATA / "schedule_head.npz")
    eb, ep, init_b = [], [], []
    for el in graphs:
        e = gg.GASEngineGPU("bfs")
        e.setGraph(el.nV, initial_vertex_data("bfs", el.nV), el.nE, None, el.src, el.dst, sp)
        e.set_schedule_model(model)
        eb.append(e)
        p = gg.GASEngineGPU("pagerank")
        p.setGraph(el.nV, initial_vertex_data("pagerank", el.nV, 0, el.out_degree()), el.nE,
                   None, el.src, el.dst, sp)
        ep.append(p)
        init_b.append(torch.from_numpy(initial_vertex_data("bfs", el.nV)).to(dev))
    out_p = torch.empty(max(el.nV for el in graphs), dtype=torch.float32, device=dev)
    plain_ppr_iters = [0]

    def plain_bfs():
        for g, el in enumerate(graphs):
            for l in range(L):
                s = int(srcs[g, l])
                eb[g].upload_vertex_data_ptr(init_b[g].data_ptr(), sp)
                eb[g].setActive(s, s + 1, sp)
                eb[g].run_schedule("learned", max_iterations=el.nV + 2, stream=sp)

    def plain_ppr():
        plain_ppr_iters[0] = 0
        for g, el in enumerate(graphs):
            for l in range(L):
                _, pst = ep[g].ppr_precision(int(seeds[g, l]), PPR_DAMPING, PPR_TOL,
                                             out=out_p.data_ptr(), stream=sp)
                plain_ppr_iters[0] += pst.iterations

    ms_plain_bfs = timed(plain_bfs, 1, 1)
    ms_plain_ppr = timed(plain_ppr, 1, 1)
    for e in eb + ep:
        e.close()

    units = bfs_units + ppr_units
    value = units / (ms * 1e-3) / 1e9
    # roofline of the PPR iteration (pieces + fix + residual kernels), timed by
    # the autotuner with CUDA events: per edge its source index and the L
    # lanes of the source's contribution; per vertex offsets (8 B), seed mask
    # (4 B), old rank, new rank and new contribution (3 x 4L B)
    ppr_bytes = E * (4 + 4 * L) + V * (12 + 12 * L)
    peak, peak_kind = measured_peaks()
    achieved = ppr_bytes / (ms_iter * 1e-3) / 1e9
    return {
        "metric": BATCH_METRIC, "value": round(value, 4), "unit": "GTEPS", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32 (BFS) + f32 (PPR, FP64 residual)",
        "data": "synthetic (seeded R-MAT graphs)",
        "config": {"workload": f"batched {G} R-MAT graphs, scale U[12,20], edge factor "
                               f"U[8,32] (seed {BATCH_SEED}), symmetrised; {L} BFS sources + "
                               f"{L} PPR seeds each (d={PPR_DAMPING}, L1 tol {PPR_TOL})",
                   "union_V": V, "union_E": E,
                   "scales": scales.tolist(), "edge_factors": efs.tolist(),
                   "bfs_units": bfs_units, "ppr_units": ppr_units,
                   "ppr_iterations": ppr_iters, "bfs_iterations": st.bfs_iterations,
                   "piece_edges": piece,
                   "l2": "inputs larger than L2 (union CSR+CSC and [V][16] rank arrays)"},
        "e2e": {"value": round(units / (ms_e2e * 1e-3) / 1e9, 4), "unit": "GTEPS",
                "ms_per_step": round(ms_e2e, 3),
                "h2d_bytes_per_step": int(srcs.nbytes + V * 4),
                "d2h_bytes_per_step": int(V * L * 8)},
        "gpu_launches": st.kernel_launches * args.steps,
        "graph_launches_per_step": st.graph_launches,
        "split": {"bfs_ms": round(ms_bfs, 3), "ppr_ms": round(ms_ppr, 3),
                  "bfs_gteps": round(bfs_units / (ms_bfs * 1e-3) / 1e9, 4),
                  "ppr_gteps": round(ppr_units / (ms_ppr * 1e-3) / 1e9, 4)},
        "plain_sequential": {
            "bfs_ms": round(ms_plain_bfs, 3), "ppr_ms": round(ms_plain_ppr, 3),
            "ppr_iterations_total": plain_ppr_iters[0],
            "bfs_speedup_of_batch": round(ms_plain_bfs / ms_bfs, 3),
            "ppr_speedup_of_batch": round(ms_plain_ppr / ms_ppr, 3),
            "total_speedup_of_batch": round((ms_plain_bfs + ms_plain_ppr) / ms, 3)},
        "roofline": {"kernel": "PPR iteration (k_ppr_pieces + k_ppr_fix + k_ppr_finish)",
                     "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": PPR_TRAFFIC_64 if G == BATCH_GRAPHS else None,
                     "traffic_note": "DRAM bytes per iteration; the [V][16] contribution "
                                     "gathers are mostly L2 hits",
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": int(ppr_bytes),
                     "avg_launch_ms": round(ms_iter, 4)},
        "clocks": clocks,
    }


# ---------------------------------------------------------------------------
# precision-form PageRank: R-MAT scale 24, directed
# ---------------------------------------------------------------------------
PR_SCALE, PR_SEED = 24, 4
# DRAM bytes (read + write) of one iteration's gather at scale 24 (k_pr_merge
# 1.477 + 0.154 GB, k_pr_merge_fix 0.016 GB), from one full ncu capture:
#   GAS_HOST_LOOP=1 ncu --set full --clock-control none -k regex:k_pr_merge -s 6 -c 2 \
#     python bench.py --workload pagerank --launch-list
PR_TRAFFIC = {24: 1.647e9}
PR_METRIC = "GTEPS (precision PageRank, R-MAT scale {scale} directed, E x iterations / time)"


def run_pagerank(args):
    import torch

    import graphreduce_gb300 as gg
    from graphreduce_gb300.engine import initial_vertex_data
    from graphreduce_gb300.graph import EdgeList
    from graphreduce_gb300.learn import DATA, MLP

    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    scale = args.pr_scale
    t = time.time()
    el = EdgeList.rmat(scale, EDGE_FACTOR, *RMAT_ABC, seed=PR_SEED, symmetrize=False)
    log(f"pagerank workload: scale {scale}: V={el.nV} E={el.nE}, generated in "
        f"{time.time() - t:.1f}s")
    e = gg.GASEngineGPU("pagerank")
    e.setGraph(el.nV, initial_vertex_data("pagerank", el.nV, 0, el.out_degree()), el.nE,
               None, el.src, el.dst, sp)
    warm_model = MLP.load(DATA / "warm_start_head.npz")
    ranks_d = torch.empty(el.nV, dtype=torch.float32, device="cuda")
    init_d = torch.empty(el.nV, dtype=torch.float32, device="cuda")

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        z = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        z.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(z) / steps

    out = {}

    def uniform():
        out["u"] = e.pagerank_precision(0.85, 1e-6, 1000, ranks_d.data_ptr(), sp)[1]

    if args.launch_list:
        # one uniform-start run and nothing else (for an ncu launch list)
        uniform()
        torch.cuda.synchronize()
        return {"launch_list": True, "iterations": out["u"].iterations}

    with ClockSampler(torch.cuda.current_device()) as clk:
        ms = timed(uniform, args.steps, args.warmup)
    clocks = clk.summary()
    st_u = out["u"]
    r_uni = ranks_d.cpu().numpy()

    def warm():  # the head's proposal, then the same iteration from it
        e.pagerank_warm_start(warm_model, 0.85, init_d.data_ptr())
        out["w"] = e.pagerank_precision_from(init_d.data_ptr(), 0.85, 1e-6, 1000, sp,
                                             out=ranks_d.data_ptr())[1]

    ms_warm = timed(warm, args.steps, 1)
    st_w = out["w"]
    r_warm = ranks_d.cpu().numpy()
    # roofline: one profiled run (events around every iteration's slab pass)
    e.set_profiling(True)
    e.profile(reset=True)
    e.pagerank_precision(0.85, 1e-6, 1000, ranks_d.data_ptr(), sp)
    prof = e.profile()
    e.set_profiling(False)
    peak, peak_kind = measured_peaks()
    achieved = prof.pagerank_bytes / (prof.pagerank_ms * 1e-3) / 1e9 if prof.pagerank_ms else 0
    units = el.nE * st_u.iterations
    res = {
        "metric": PR_METRIC.format(scale=scale), "value": round(units / (ms * 1e-3) / 1e9, 4), "unit": "GTEPS",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (two-sum compensated gather) + f64 residual",
        "data": "synthetic (seeded R-MAT)",
        "config": {"workload": f"precision PageRank, R-MAT scale {scale}, edge factor "
                               f"{EDGE_FACTOR}, directed, seed {PR_SEED}, d=0.85, L1 tol 1e-6",
                   "V": el.nV, "E": el.nE, "iterations": st_u.iterations,
                   "residual": st_u.residual,
                   "l2": "inputs larger than L2"},
        "warm_start": {"iterations": st_w.iterations, "ms": round(ms_warm, 3),
                       "speedup": round(ms / ms_warm, 4),
                       "l1_between_results": float(np.abs(r_uni.astype(np.float64) -
                                                          r_warm).sum())},
        "roofline": {"kernel": "k_pr_merge + k_pr_merge_fix (one PageRank iteration's gather)",
                     "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": PR_TRAFFIC.get(scale),
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": int(prof.pagerank_bytes /
                                                         max(1, prof.pagerank_launches)),
                     "avg_launch_ms": round(prof.pagerank_ms / max(1, prof.pagerank_launches), 4)},
        "clocks": clocks,
    }
    if args.pr_check:
        import oracle
        t = time.time()
        r64, it64, _ = oracle.pagerank_fp64(el.nV, el.src, el.dst, 0.85, 1e-6)
        d = np.abs(r_uni.astype(np.float64) - r64)
        res["error_vs_fp64_oracle"] = {"l1": float(d.sum()), "max_abs": float(d.max()),
                                       "oracle_iterations": it64,
                                       "oracle_seconds": round(time.time() - t, 1)}
    return res


# ---------------------------------------------------------------------------
# CPU baseline (the oracle, a C port of refgas.h)
# ---------------------------------------------------------------------------
def cpu_sssp_sample(ssp, sources, out_sssp, n_threads):
    import oracle
    from graphreduce_gb300.engine import SSSP_GATHER_ZERO
    res = [None] * n_threads

    def work(i):
        t = time.perf_counter()
        d, it = oracle.sssp(ssp.nV, ssp.src, ssp.dst, ssp.weights, int(sources[i]))
        res[i] = (d, it, time.perf_counter() - t)

    t0 = time.perf_counter()
    th = [threading.Thread(target=work, args=(i,)) for i in range(n_threads)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    wall = time.perf_counter() - t0
    ev = sum(edges_visited(out_sssp, r[0], SSSP_GATHER_ZERO) for r in res)
    return ev / wall / 1e9, wall, res


def run_reference(args):
    import oracle  # noqa: F401  (the oracle port: the reference's refgas.h in C)
    ssp, sources, _ = make_workload(args.scale)
    out_sssp = ssp.out_degree()
    cores = os.cpu_count() or 1
    n = min(N_SOURCES, cores)
    for _ in range(args.warmup):
        cpu_sssp_sample(ssp, sources, out_sssp, n)
    vals, walls = [], []
    for _ in range(max(1, args.steps)):
        v, w, _ = cpu_sssp_sample(ssp, sources, out_sssp, n)
        vals.append(v)
        walls.append(w)
    value = statistics.median(vals)
    sample = (f"SSSP from {n} of the {N_SOURCES} sources, one thread each, on the scale-"
              f"{args.scale} graph (CC part of the step not sampled)")
    return {"metric": METRIC.format(scale=args.scale), "value": round(value, 5), "unit": "GTEPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * statistics.median(walls), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic", "impl": "reference",
            "config": config_dict(args.scale),
            "cpu_baseline": {"value": round(value, 5), "unit": "GTEPS", "cores": n,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 5), "unit": "GTEPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--schedule", default="learned",
                    choices=["learned", "auto", "generic", "push", "pull", "ordered"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--edges", default="device", choices=["device", "host"],
                    help="edge arrays in HBM or in pinned host memory (NVLink-C2C)")
    ap.add_argument("--workload", default="sssp-cc",
                    choices=["sssp-cc", "batched", "pagerank", "lanes24"])
    ap.add_argument("--pr-scale", type=int, default=PR_SCALE)
    ap.add_argument("--pr-check", action="store_true",
                    help="compare with the FP64 oracle (single-threaded C, slow)")
    ap.add_argument("--batch-graphs", type=int, default=BATCH_GRAPHS)
    ap.add_argument("--sssp", default="batched", choices=["batched", "sequential"],
                    help="the 8 SSSP sources as lanes of one batched run, or one run each")
    ap.add_argument("--launch-list", action="store_true",
                    help="run one device-resident step only (profiling)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)), flush=True)
        return

    if args.workload == "batched":
        if rank == 0:
            print(json.dumps(run_batched(args)), flush=True)
        return
    if args.workload == "pagerank":
        if rank == 0:
            print(json.dumps(run_pagerank(args)), flush=True)
        return
    if args.workload == "lanes24":
        if rank == 0:
            print(json.dumps(run_lanes24(args)), flush=True)
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    result, cpu_inputs = run_ours(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline and cpu_inputs is not None:
            ssp, sources, out_sssp, first_sssp = cpu_inputs
            import oracle
            from graphreduce_gb300.engine import SSSP_GATHER_ZERO
            t = time.perf_counter()
            d, it = oracle.sssp(ssp.nV, ssp.src, ssp.dst, ssp.weights, int(sources[0]))
            sec = time.perf_counter() - t
            ev = edges_visited(out_sssp, d, SSSP_GATHER_ZERO)
            result["cpu_baseline"] = {
                "value": round(ev / sec / 1e9, 5), "unit": "GTEPS", "cores": 1, "kind": "port",
                "sample": f"SSSP from source {int(sources[0])} on the scale-{args.scale} graph, "
                          f"oracle C port of refgas.h, 1 thread, {sec:.1f}s"}
            result["verified_against_oracle"] = bool(np.array_equal(d, first_sssp))
        print(json.dumps(result), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
