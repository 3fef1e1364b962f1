"""Benchmark of the GAS hot path: every configuration of the workload table.

Headline ("value", one "step"): SSSP from 8 sources and CC on an R-MAT graph
of scale 22 (4,194,304 vertices, edge factor 16, (a,b,c,d) =
(0.57,0.19,0.19,0.05), seed 2, symmetrised, self loops and duplicates
removed); SSSP weights uniform in [1,64] (seed 3, both directions equal);
sources drawn uniformly from the largest component (seed 2); CC on the same
graph plus 4,096 disjoint 32x32 4-neighbour grid islands.  Synthetic data:
the reference's real-world datasets are not available.

Metric: GTEPS with the reference's definition (sssp.cu:202-211): for every
run, the sum of out-degrees of the vertices it reached, divided by time
(for CC every vertex is reached, so a run counts all its edges).

The engine under test is the learned-schedule, batched one: the 8 SSSP
sources run as the 8 lanes of one multi-source SSSP launch, CC runs through
the engine with the learned schedule.  The plain fixed-heuristic form (one
SSSP run per source and CC, schedule AUTO) is timed beside it, device
resident and end to end.

  value  -- device-resident: graph and initial vertex states already in HBM,
            timed with CUDA events on the engine's stream.
  e2e    -- through the public Python API with pinned host buffers: every
            input goes up (the CC labels; the SSSP source ids -- the batched
            run builds its initial distances on the device) and every result
            comes down (the [V][8] distances, the CC labels) inside the
            timed region.

At one GPU the same line also carries "configs", one entry per workload
configuration, each with its GTEPS, the dominant kernel's roofline on
algorithmic bytes (and on DRAM bytes where an ncu capture of that kernel is
recorded), and a parity flag from the oracle:
  c1_bfs        BFS, R-MAT scale 16, seed 1, source = first vertex of
                maximum out-degree (bfs.cu:175-195); depths and levels
                bit-exact against the oracle
  c2_sssp_cc    the headline step: all 8 SSSP lanes and the CC labels
                bit-exact against the oracle (iterations included)
  c3_pagerank   precision PageRank, R-MAT scale 24 directed, seed 4; L1 and
                max-abs error against the FP64 oracle
  c4_learned    the schedule head and the PageRank warm start on held-out
                graphs (R-MAT scale 24 seed 5; Erdos-Renyi, 2^24 vertices,
                average degree 16, seed 5) against every fixed schedule
  c5_batched    64 R-MAT graphs x (16 BFS + 16 PPR) in one graph launch
                against the same instances one by one; a per-lane parity
                sample against the oracle

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--configs c1,c2,c3,c4,c5 | --no-configs]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
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
SSSP_UNREACHED = 2**31 - 1 - 100000  # sssp.cu:32-33 gatherZero
METRIC = "GTEPS (SSSP x8 + CC, R-MAT scale {scale})"
MAX_ITERS = 20000  # far above any run of this workload; bounds a device loop
ALL_CONFIGS = ("c1", "c2", "c3", "c4", "c5")

# DRAM bytes (read + write) per launch of a dominant kernel, from ncu
# captures recorded under profiles/ (each names its command and the bounded
# form to use for a new capture).  Keys: (kernel, workload).
DRAM_PER_LAUNCH = {
    # one-pass counters over the 11 batched-SSSP push launches of a scale-22
    # step (profiles/launches_sssp8-cc_rmat-s22_batched.md)
    ("mss_push", "rmat-s22"): 814.0e6,
    # CC push, mean over the 63 launches of the same step (same profile)
    ("push", "rmat-s22-cc"): 103.2e6,
    # k_pr_merge + k_pr_merge_fix, one iteration at scale 24
    # (profiles/k_pr_merge_pagerank_rmat-s24.md)
    ("pr_gather", "rmat-s24"): 1.647e9,
    # k_ppr_pieces + k_ppr_fix, one PPR iteration of the 64-graph batch
    # (profiles/k_ppr_pieces_batched-8graphs.md)
    ("ppr_iteration", "batched-64"): 10.30e9,
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# shared helpers
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


def edges_visited(outdeg, vd, unreached):
    return int(outdeg[vd != unreached].sum(dtype=np.int64))


def gteps(units, ms):
    return round(units / (ms * 1e-3) / 1e9, 4) if ms > 0 else 0.0


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


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# What bounds each kernel, from its ncu capture under profiles/ (bound is
# "hbm" in the line's two-valued sense: a memory-side kernel, no tensor
# work; frac counts algorithmic bytes against the HBM peak, dram_frac the
# bytes that reached DRAM).
LIMITER = {
    "mss_push": "L1 data pipe (68 % of peak) and L2 tag lookups (51 %); DRAM 15.5 %: most "
                "algorithmic bytes are L2 hits (profiles/k_mss_push_sssp8-batched_rmat-s20.md)",
    "push": "latency of dependent loads per light row with 93 % of warp slots occupied; "
            "L2 tags 36 %, DRAM 25 % (profiles/k_push_cc-islands_rmat-s20.md)",
    "pr_gather": "L1 data pipe (70 %): one wavefront per random contribution gather; DRAM "
                 "18 % (profiles/k_pr_merge_pagerank_rmat-s24.md)",
    "ppr_iteration": "latency of the 64-byte contribution-row gathers, 62 % of warp slots "
                     "occupied (profiles/k_ppr_pieces_batched-8graphs.md)",
    "bfs_small": "latency: one cooperative kernel, a few microseconds per level, the graph in "
                 "L2 (profiles/k_bfs_small_bfs_rmat-s16.md)",
}


def roofline(kernel, key, total_bytes, total_ms, launches, workload, extra=None):
    """The dominant kernel's roofline: algorithmic bytes over its measured
    time (CUDA events around its launches), and where an ncu capture of the
    kernel on this workload is recorded, its DRAM bytes over the same time
    and what its counters show bounds it."""
    peak, kind = measured_peaks()
    launches = max(1, int(launches))
    ms_l = total_ms / launches
    alg_l = total_bytes / launches
    ach = alg_l / (ms_l * 1e-3) / 1e9 if ms_l > 0 else 0.0
    dram = DRAM_PER_LAUNCH.get((key, workload))
    r = {"kernel": kernel, "bound": "hbm", "achieved": round(ach, 1), "unit": "GB/s",
         "peak": peak, "peak_source": kind, "frac": round(ach / peak, 4),
         "algorithmic_bytes_per_launch": int(alg_l), "avg_launch_ms": round(ms_l, 4),
         "launches": launches, "traffic": dram,
         "dram_achieved": round(dram / (ms_l * 1e-3) / 1e9, 1) if dram and ms_l > 0 else None,
         "dram_frac": round(dram / (ms_l * 1e-3) / 1e9 / peak, 4) if dram and ms_l > 0 else None}
    if key in LIMITER and (dram is not None or key == "bfs_small"):  # captured on this workload
        r["limiter"] = LIMITER[key]
    if extra:
        r.update(extra)
    return r


def cuda_timed(stream, fn, steps, warmup):
    """Mean ms of fn() over `steps` calls after `warmup`, CUDA events on the
    stream the work is launched on, synchronised on both sides."""
    import torch
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
    return a.elapsed_time(z) / max(1, steps)


def free_gpu():
    import gc

    import torch
    gc.collect()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def oracle_threads():
    """Every host thread for the oracle's loops (its results do not depend
    on the count)."""
    import oracle
    n = os.cpu_count() or 1
    oracle.set_threads(n)
    return n


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


# ---------------------------------------------------------------------------
# C2, the headline: SSSP x8 + CC at scale 22
# ---------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch

    import graphreduce_gb300 as gg
    from graphreduce_gb300.engine import initial_vertex_data

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
    # stream (in order, so each copy also waits for the one before it): the
    # CC labels go up while the SSSP lanes run, the distances come down
    # while CC runs, and the CC labels come down while the next step's SSSP
    # lanes run; the timed region ends when both streams are done
    cstream = torch.cuda.Stream(device=dev)
    csp = cstream.cuda_stream
    dist_free = torch.cuda.Event()   # the last distances are down: dist_dev may change
    dist_free.record(cstream)

    def one_step(e2e, schedule=args.schedule, use_batch=batched):
        launches[0] = 0
        if e2e and use_batch:
            # after the previous step's labels came down (same stream)
            e_c.upload_vertex_data_ptr(pin_c.data_ptr(), csp)
            up = torch.cuda.Event()
            up.record(cstream)
            stream.wait_event(dist_free)
            sssp_batched(False)
            lanes_done = torch.cuda.Event()
            lanes_done.record(stream)
            cstream.wait_event(lanes_done)
            with torch.cuda.stream(cstream):
                dist_pin.copy_(dist_dev, non_blocking=True)
            dist_free.record(cstream)
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
        if e2e and use_batch:
            cc_done = torch.cuda.Event()
            cc_done.record(stream)
            cstream.wait_event(cc_done)
            e_c.download_vertex_data_ptr(res_c.data_ptr(), csp, wait=False)
        elif e2e:
            e_c.download_vertex_data_ptr(res_c.data_ptr(), sp)

    if args.launch_list:
        # one device-resident step and nothing else (for an ncu launch list)
        one_step(e2e=False)
        torch.cuda.synchronize()
        return {"launch_list": True, "gpu_launches": launches[0]}, None

    # outputs of this exact workload (checked against the oracle at the end)
    one_step(e2e=True)
    torch.cuda.synchronize()
    lanes = np.array(dist_pin.numpy()) if batched else np.stack(
        [r.numpy() for r in res_s], axis=1)
    cc_labels = res_c.numpy().copy()
    out_iters = {"sssp": list(iters["sssp"]), "cc": iters["cc"]}
    ev_units = sum(edges_visited(out_sssp, lanes[:, k], SSSP_UNREACHED)
                   for k in range(len(sources)))
    ev_units += edges_visited(out_cc, cc_labels, -12345)  # every CC vertex is reached

    def timed(e2e, steps, warmup, schedule=args.schedule, use_batch=batched):
        for _ in range(warmup):
            one_step(e2e, schedule, use_batch)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        start.record(stream)
        cstream.wait_event(start)    # the copies of the first step start after it
        for _ in range(steps):
            one_step(e2e, schedule, use_batch)
        stream.wait_stream(cstream)  # and the last step's copies end before `end`
        end.record(stream)
        torch.cuda.synchronize()
        ms = start.elapsed_time(end)
        return max_over_ranks(ms, world, dev) / steps

    with ClockSampler(torch.cuda.current_device()) as clk:
        ms_step = timed(False, args.steps, args.warmup)
    clocks = clk.summary()
    launches_per_step = launches[0]
    iters_step = {"sssp": list(iters["sssp"]), "cc": iters["cc"]}
    ms_e2e = timed(True, max(1, args.steps), args.warmup)
    comparisons = {}
    # the same step with one SSSP run per source (learned schedule), and the
    # plain form: one run per source under the fixed heuristic (AUTO), both
    # device resident and end to end
    if batched:
        ms_seq = timed(False, args.steps, args.warmup, args.schedule, False)
        comparisons["sequential_sources"] = {
            "schedule": args.schedule, "ms_per_step": round(ms_seq, 3),
            "value": round(world * ev_units / (ms_seq * 1e-3) / 1e9, 4),
            "speedup_of_headline": round(ms_seq / ms_step, 4)}
    ms_plain = timed(False, args.steps, args.warmup, "auto", False)
    ms_plain_e2e = timed(True, max(1, args.steps), 1, "auto", False)
    plain = {"schedule": "auto (fixed heuristic), one SSSP run per source",
             "ms_per_step": round(ms_plain, 3),
             "value": round(world * ev_units / (ms_plain * 1e-3) / 1e9, 4),
             "speedup_of_headline": round(ms_plain / ms_step, 4),
             "e2e": {"ms_per_step": round(ms_plain_e2e, 3),
                     "value": round(world * ev_units / (ms_plain_e2e * 1e-3) / 1e9, 4),
                     "h2d_bytes_per_step": (len(sources) * ssp.nV + ccg.nV) * 4,
                     "d2h_bytes_per_step": (len(sources) * ssp.nV + ccg.nV) * 4,
                     "speedup_of_headline_e2e": round(ms_plain_e2e / ms_e2e, 4)}}

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
    roof, by_kernel = kernel_roofline(e_s, e_c, bat, dev_s, dev_c, ssp, ccg, lane_src,
                                      dist_dev, args.schedule, sp, args.scale, args.edges)

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
                "copies": ("pinned host buffers; CC labels up while the SSSP lanes run, "
                           "distances down while CC runs, CC labels down while the next "
                           "step's SSSP lanes run (second stream; every step's copies "
                           "inside the timed region)" if batched else
                           "pinned host buffers, on the compute stream")},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roof,
        "by_kernel": by_kernel,
        "algos": split,
        "plain": plain,
        "comparisons": comparisons,
        "clocks": clocks,
    }
    for e in (e_s, e_c):
        e.close()
    if bat is not None:
        bat.close()
    outputs = {"ssp": ssp, "ccg": ccg, "sources": sources, "lanes": lanes,
               "cc_labels": cc_labels, "iters": out_iters, "ev_units": ev_units}
    return result, outputs


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
        ev += edges_visited(out_sssp, host, SSSP_UNREACHED)
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
                              "gteps": gteps(ev, ms), "iterations": its}
    if bat is not None:
        a.record(stream)
        r = bat.run(sssp_sources=lane_src, max_sssp_iterations=MAX_ITERS,
                    dist_out=dist_dev.data_ptr(), stream=sp)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        out["sssp_batched"] = {"ms_8_sources": round(ms, 3), "gteps": gteps(ev, ms),
                               "iterations": r.stats.sssp_iterations,
                               "union_edges_pushed": int(r.stats.sssp_edges)}
    a.record(stream)
    e_c.upload_vertex_data_ptr(dev_c.data_ptr(), sp)
    e_c.setActive(0, ccg.nV, sp)
    it = e_c.run_schedule(schedule, max_iterations=MAX_ITERS, stream=sp).iterations
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    out["cc"] = {"ms": round(ms, 3), "gteps": gteps(ccg.nE, ms), "iterations": it}
    return out


def kernel_roofline(e_s, e_c, bat, dev_s, dev_c, ssp, ccg, lane_src, dist_dev, schedule, sp,
                    scale, edges):
    """One extra pass of the step's runs with kernel profiling on: the
    engines bracket every push / dense-pull launch (and the batch every
    multi-source SSSP push) with CUDA events on the run's stream and
    accumulate its algorithmic bytes (per edge: index, weight for SSSP, and
    the state, row or membership word it reads; per frontier entry or row:
    its offsets and state).  The dominant kernel is the one with the largest
    total time; every kernel's roofline is returned beside it."""
    import torch
    kinds = {}

    def add(key, p, name):
        k = kinds.setdefault(key, {"ms": 0.0, "bytes": 0, "launches": 0})
        k["ms"] += getattr(p, f"{name}_ms")
        k["bytes"] += getattr(p, f"{name}_bytes")
        k["launches"] += getattr(p, f"{name}_launches")

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
        add("sssp_push", ps, "push")
        add("sssp_pull", ps, "pull")
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
    names = {"pull": "k_pull (CC dense pull, warp-slab)",
             "push": "k_push (CC frontier push, warp-slab)",
             "sssp_push": "k_push (SSSP frontier push, warp-slab)",
             "sssp_pull": "k_pull (SSSP dense pull, warp-slab)",
             "mss_push": "k_mss_push (8-lane multi-source SSSP push, warp-slab)"}
    wl = {"push": f"rmat-s{scale}-cc", "pull": f"rmat-s{scale}-cc",
          "sssp_push": f"rmat-s{scale}", "sssp_pull": f"rmat-s{scale}",
          "mss_push": f"rmat-s{scale}"}
    placement = "" if edges == "device" else "-host-edges"
    rows = {k: roofline(names[k], k.replace("sssp_", ""), v["bytes"], v["ms"], v["launches"],
                        wl[k] + placement, {"total_ms": round(v["ms"], 3)})
            for k, v in kinds.items() if v["launches"]}
    dom = max(rows, key=lambda k: kinds[k]["ms"])
    return rows[dom], rows


# ---------------------------------------------------------------------------
# the drop-in path: user programs through include/gpugas.h
# ---------------------------------------------------------------------------
def _write_graph_bin(path, nV, src, dst, w, sources):
    with open(path, "wb") as f:
        np.array([nV, len(src), len(sources)], np.int32).tofile(f)
        np.ascontiguousarray(src, np.int32).tofile(f)
        np.ascontiguousarray(dst, np.int32).tofile(f)
        (np.ones(len(src), np.int32) if w is None else np.ascontiguousarray(w, np.int32)).tofile(f)
        np.ascontiguousarray(sources, np.int32).tofile(f)


def user_program_path(el, sources, cc_el=None, reps=1):
    """Runs graphreduce_gb300/_lib/bench_user_programs: the reference apps'
    BFS, SSSP and CC programs written as user programs and compiled through
    include/gpugas.h (BFS and SSSP driven through the step API like bfs.cu
    and sssp.cu, CC through run(), one CUDA-graph launch).  Returns its
    timings and outputs (BFS depths from sources[0], SSSP distances per
    source, CC labels)."""
    from graphreduce_gb300.build import OUT_DIR
    exe = OUT_DIR / "bench_user_programs"
    with tempfile.TemporaryDirectory() as d:
        g = Path(d) / "g.bin"
        _write_graph_bin(g, el.nV, el.src, el.dst, el.weights, sources)
        cmd = [str(exe), str(g), str(reps), str(Path(d) / "out.bin")]
        if cc_el is not None:
            _write_graph_bin(Path(d) / "cc.bin", cc_el.nV, cc_el.src, cc_el.dst, None, [])
            cmd.append(str(Path(d) / "cc.bin"))
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
        if r.returncode != 0:
            raise RuntimeError(f"bench_user_programs failed ({r.returncode}): {r.stderr[-500:]}")
        res = json.loads(r.stdout.strip().splitlines()[-1])
        raw = np.fromfile(Path(d) / "out.bin", np.int32)
    nV, k = el.nV, len(sources)
    res["bfs_depth"] = raw[:nV]
    res["sssp_dist"] = raw[nV:nV * (1 + k)].reshape(k, nV)
    res["cc_label"] = raw[nV * (1 + k):]
    return res


# ---------------------------------------------------------------------------
# C2 parity and the CPU baseline: the oracle on the whole step
# ---------------------------------------------------------------------------
def c2_oracle_check(out):
    """The oracle (a C restatement of refgas.h, all host threads) runs the
    headline step once: SSSP from each of the 8 sources and CC on the islands
    graph.  Its outputs must equal the GPU's bit for bit (iterations
    included); its run times (graph builds excluded, as the GPU's are) are
    the CPU baseline."""
    import oracle
    n_threads = oracle_threads()
    ssp, ccg, sources = out["ssp"], out["ccg"], out["sources"]
    t = time.perf_counter()
    g = oracle.Graph(ssp.nV, ssp.src, ssp.dst)
    build_s = time.perf_counter() - t
    run_s, units = 0.0, 0
    outdeg = ssp.out_degree()
    lane_ok, iter_ok = [], []
    for k, s in enumerate(sources):
        t = time.perf_counter()
        d, it = g.sssp(ssp.weights, int(s))
        run_s += time.perf_counter() - t
        units += edges_visited(outdeg, d, SSSP_UNREACHED)
        lane_ok.append(bool(np.array_equal(d, out["lanes"][:, k])))
        iter_ok.append(it == out["iters"]["sssp"][k])
    g.close()
    t = time.perf_counter()
    gc = oracle.Graph(ccg.nV, ccg.src, ccg.dst)
    build_s += time.perf_counter() - t
    t = time.perf_counter()
    lab, it_cc = gc.cc()
    run_s += time.perf_counter() - t
    gc.close()
    units += ccg.nE
    cc_ok = bool(np.array_equal(lab, out["cc_labels"]))
    parity = {"parity": all(lane_ok) and all(iter_ok) and cc_ok and it_cc == out["iters"]["cc"],
              "sssp_lanes_bit_exact": lane_ok, "sssp_iterations_equal": iter_ok,
              "cc_labels_bit_exact": cc_ok, "cc_iterations": [it_cc, out["iters"]["cc"]],
              "oracle": "oracle/gas_oracle.c (refgas.h restated), all host threads"}
    cpu = {"value": round(units / run_s / 1e9, 5), "unit": "GTEPS", "cores": n_threads,
           "kind": "port",
           "sample": (f"the whole step once (SSSP from the 8 sources + CC) through the oracle "
                      f"port of refgas.h on {n_threads} threads, {run_s:.1f}s of runs "
                      f"(graph builds {build_s:.1f}s excluded)")}
    return parity, cpu


def c2_user_programs(out):
    """The headline step through the drop-in path: SSSP from the 8 sources
    (sssp.cu's step loop, one run per source) and CC (connected_component.cu's
    run()), as user programs compiled through include/gpugas.h; outputs
    bit-exact with the built-in engine's (which the oracle checked)."""
    ssp, ccg, sources = out["ssp"], out["ccg"], out["sources"]
    up = user_program_path(ssp, sources, ccg, reps=1)
    outdeg = ssp.out_degree()
    sssp_units = sum(edges_visited(outdeg, up["sssp_dist"][k], SSSP_UNREACHED)
                     for k in range(len(sources)))
    ms_sssp = up["sssp_ms_per_source"] * len(sources)
    ms = ms_sssp + up["cc_ms"]
    same = all(np.array_equal(up["sssp_dist"][k], out["lanes"][:, k])
               for k in range(len(sources))) and np.array_equal(up["cc_label"], out["cc_labels"])
    return {"path": "user programs through include/gpugas.h: SSSP by the step API per source, "
                    "CC by run() (one CUDA-graph launch)",
            "ms_per_step": round(ms, 3), "gteps": gteps(sssp_units + ccg.nE, ms),
            "sssp_ms_per_source": up["sssp_ms_per_source"], "sssp_iterations": up["sssp_iterations"],
            "cc_ms": up["cc_ms"], "cc_iterations": up["cc_iterations"],
            "cc_graph_launches": up["cc_graph_launches"],
            "identical_to_builtin": bool(same) and up["sssp_iterations"] == out["iters"]["sssp"]
            and up["cc_iterations"] == out["iters"]["cc"]}


# ---------------------------------------------------------------------------
# C1: BFS, R-MAT scale 16, seed 1, highest-degree source
# ---------------------------------------------------------------------------
C1_SCALE, C1_SEED = 16, 1


def run_c1(args, model):
    import torch

    import graphreduce_gb300 as gg
    import oracle
    from graphreduce_gb300.engine import initial_vertex_data
    from graphreduce_gb300.graph import EdgeList

    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    el = EdgeList.rmat(C1_SCALE, EDGE_FACTOR, *RMAT_ABC, seed=C1_SEED, symmetrize=True)
    src, deg = el.max_out_degree_vertex()   # first vertex of maximum out-degree
    e = gg.GASEngineGPU("bfs")
    e.setGraph(el.nV, initial_vertex_data("bfs", el.nV), el.nE, None, el.src, el.dst, sp)
    e.set_schedule_model(model)
    init = torch.from_numpy(initial_vertex_data("bfs", el.nV))
    init_d, init_p = init.to("cuda"), init.pin_memory()
    out_p = torch.empty(el.nV, dtype=torch.int32).pin_memory()
    last = {}

    def run(schedule, e2e=False):
        e.upload_vertex_data_ptr((init_p if e2e else init_d).data_ptr(), sp)
        e.setActive(src, src + 1, sp)
        last[schedule] = e.run_schedule(schedule, max_iterations=el.nV + 2, stream=sp)
        if e2e:
            e.download_vertex_data_ptr(out_p.data_ptr(), sp)

    run("learned", e2e=True)
    depth = out_p.numpy().copy()
    ref, rit = oracle.bfs(el.nV, el.src, el.dst, src)
    units = edges_visited(el.out_degree(), depth, -1)
    times = {}
    for s in ("learned", "push", "pull", "generic"):
        times[s] = cuda_timed(stream, lambda s=s: run(s), args.steps, args.warmup)
    ms_e2e = cuda_timed(stream, lambda: run("learned", True), args.steps, 1)
    same = {}
    for s in ("push", "pull", "generic"):
        run(s, e2e=True)
        same[s] = bool(np.array_equal(out_p.numpy(), depth)) and \
            last[s].iterations == last["learned"].iterations
    e.set_profiling(True)
    e.profile(reset=True)
    run("learned")
    torch.cuda.synchronize()
    p = e.profile()
    e.set_profiling(False)
    e.close()
    # the drop-in path: bfs.cu's BFS program and step loop through gpugas.h
    up = user_program_path(el, [src], None, reps=max(1, min(args.steps, 5)))
    user = {"path": "user program through include/gpugas.h, bfs.cu's step loop",
            "ms": up["bfs_ms"], "gteps": gteps(units, up["bfs_ms"]),
            "levels": up["bfs_levels"],
            "identical_to_builtin": bool(np.array_equal(up["bfs_depth"], depth))
            and up["bfs_levels"] == last["learned"].iterations}
    if p.pull_launches == 0 and p.push_launches == 1:  # graphs of up to 2^18 vertices
        roof = roofline("k_bfs_small (every level in one cooperative kernel)", "bfs_small",
                        p.push_bytes, p.push_ms, 1, "rmat-s16",
                        {"timed_with_byte_counting": True})
    elif p.push_ms >= p.pull_ms:
        roof = roofline("k_bfs_push (top-down levels)", "bfs_push", p.push_bytes, p.push_ms,
                        p.push_launches, "rmat-s16")
    else:
        roof = roofline("k_bfs_pull (bottom-up levels)", "bfs_pull", p.pull_bytes, p.pull_ms,
                        p.pull_launches, "rmat-s16")
    roof["note"] = ("65,536 vertices: the whole graph (7.6 MB) sits in L2 and a level is a few "
                    "microseconds of work, so the run is bound by latency (grid barriers, "
                    "L2 round trips), not by DRAM bandwidth")
    return {
        "workload": f"BFS rmat-s{C1_SCALE}-ef{EDGE_FACTOR}-sym seed {C1_SEED}, source = first "
                    f"vertex of maximum out-degree ({src}, degree {deg})",
        "V": el.nV, "E": el.nE, "levels": last["learned"].iterations,
        "schedule": "learned (direction rule: bottom-up while the frontier's out-edges > E/16)",
        "ms": round(times["learned"], 4), "gteps": gteps(units, times["learned"]),
        "e2e": {"ms": round(ms_e2e, 4), "gteps": gteps(units, ms_e2e),
                "h2d_bytes": el.nV * 4, "d2h_bytes": el.nV * 4},
        "fixed_schedules": {s: {"ms": round(times[s], 4), "gteps": gteps(units, times[s]),
                                "identical_output": same[s]}
                            for s in ("push", "pull", "generic")},
        "user_program": user,
        "parity": bool(np.array_equal(depth, ref)) and rit == last["learned"].iterations
        and all(same.values()) and user["identical_to_builtin"],
        "parity_detail": "depths and level count bit-exact against the oracle BFS",
        "roofline": roof,
    }


# ---------------------------------------------------------------------------
# C3: precision-form PageRank, R-MAT scale 24 directed
# ---------------------------------------------------------------------------
PR_SCALE, PR_SEED = 24, 4
PR_METRIC = "GTEPS (precision PageRank, R-MAT scale {scale} directed, E x iterations / time)"
PR_DAMPING, PR_TOL = 0.85, 1e-6


def run_pagerank(args, check=True):
    """Uniform start (timed), the warm start (timed), the gather's roofline
    from one profiled run, and the FP64 oracle on the same graph."""
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
    ranks_p = torch.empty(el.nV, dtype=torch.float32).pin_memory()
    out = {}

    def uniform(e2e=False):
        out["u"] = e.pagerank_precision(PR_DAMPING, PR_TOL, 1000,
                                        (ranks_p if e2e else ranks_d).data_ptr(), sp)[1]

    if args.launch_list:
        # one uniform-start run and nothing else (for an ncu launch list)
        uniform()
        torch.cuda.synchronize()
        e.close()
        return {"launch_list": True, "iterations": out["u"].iterations}

    with ClockSampler(torch.cuda.current_device()) as clk:
        ms = cuda_timed(stream, uniform, args.steps, args.warmup)
    clocks = clk.summary()
    ms_e2e = cuda_timed(stream, lambda: uniform(True), max(1, args.steps), 1)
    st_u = out["u"]
    r_uni = ranks_d.cpu().numpy()

    def warm():  # the head's proposal, then the same iteration from it
        e.pagerank_warm_start(warm_model, PR_DAMPING, init_d.data_ptr())
        out["w"] = e.pagerank_precision_from(init_d.data_ptr(), PR_DAMPING, PR_TOL, 1000, sp,
                                             out=ranks_d.data_ptr())[1]

    ms_warm = cuda_timed(stream, warm, args.steps, 1)
    st_w = out["w"]
    r_warm = ranks_d.cpu().numpy()
    # roofline: one profiled run (events around every iteration's gather)
    e.set_profiling(True)
    e.profile(reset=True)
    e.pagerank_precision(PR_DAMPING, PR_TOL, 1000, ranks_d.data_ptr(), sp)
    prof = e.profile()
    e.set_profiling(False)
    e.close()
    units = el.nE * st_u.iterations
    roof = roofline("k_pr_merge + k_pr_merge_fix (one PageRank iteration's gather)",
                    "pr_gather", prof.pagerank_bytes, prof.pagerank_ms,
                    prof.pagerank_launches, f"rmat-s{scale}")
    res = {
        "metric": PR_METRIC.format(scale=scale), "value": gteps(units, ms), "unit": "GTEPS",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (two-sum compensated gather) + f64 residual",
        "data": "synthetic (seeded R-MAT)",
        "config": {"workload": f"precision PageRank, R-MAT scale {scale}, edge factor "
                               f"{EDGE_FACTOR}, directed, seed {PR_SEED}, d={PR_DAMPING}, "
                               f"L1 tol {PR_TOL}",
                   "V": el.nV, "E": el.nE, "iterations": st_u.iterations,
                   "residual": st_u.residual, "l2": "inputs larger than L2"},
        "e2e": {"value": gteps(units, ms_e2e), "unit": "GTEPS", "ms_per_step": round(ms_e2e, 3),
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": el.nV * 4,
                "copies": "graph resident; the ranks come down to pinned host memory"},
        "warm_start": {"iterations": st_w.iterations, "uniform_iterations": st_u.iterations,
                       "ms": round(ms_warm, 3), "speedup": round(ms / ms_warm, 4),
                       "l1_between_results": float(np.abs(r_uni.astype(np.float64) -
                                                          r_warm).sum())},
        "roofline": roof,
        "clocks": clocks,
    }
    if check:
        import oracle
        n = oracle_threads()
        t = time.time()
        r64, it64, _ = oracle.pagerank_fp64(el.nV, el.src, el.dst, PR_DAMPING, PR_TOL)
        d = np.abs(r_uni.astype(np.float64) - r64)
        l1, mx = float(d.sum()), float(d.max())
        res["error_vs_fp64_oracle"] = {"l1": l1, "max_abs": mx, "oracle_iterations": it64,
                                       "oracle_seconds": round(time.time() - t, 1),
                                       "oracle_threads": n}
        res["parity"] = l1 <= 1e-6
        res["parity_detail"] = ("L1 error of the FP32 ranks against the FP64 oracle's <= 1e-6 "
                                "(same damping and residual tolerance)")
    return res


# ---------------------------------------------------------------------------
# C4: learned schedule and warm start on held-out graphs
# ---------------------------------------------------------------------------
C4_SEED = 5
C4_SCHEDULES = ("auto", "push", "pull", "learned")


def run_c4(args, model, pr_warm):
    """BFS, SSSP and CC under every schedule on graphs the heads never saw;
    the learned schedule against the fixed heuristic (AUTO) and against the
    best fixed schedule; outputs identical across schedules (BFS has no
    learned head: LEARNED runs its AUTO direction rule).  The PageRank warm
    start against the uniform start (iterations to the same tolerance)."""
    import torch

    import graphreduce_gb300 as gg
    from graphreduce_gb300.engine import initial_vertex_data
    from graphreduce_gb300.graph import EdgeList
    from graphreduce_gb300.learn import DATA, MLP

    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    scale = args.pr_scale
    graphs = {
        f"rmat{scale}": lambda: EdgeList.rmat(scale, EDGE_FACTOR, *RMAT_ABC, seed=C4_SEED,
                                              symmetrize=True),
        "er2^24": lambda: EdgeList.erdos_renyi(1 << scale, 8 << scale, seed=C4_SEED,
                                               symmetrize=True),
    }
    res = {}
    all_ok = True
    for name, make in graphs.items():
        t = time.time()
        el = make().with_uniform_weights(1, 64, C4_SEED)
        src = int(el.sample_sources(1, C4_SEED)[0])
        log(f"c4 {name}: V={el.nV} E={el.nE}, generated in {time.time() - t:.1f}s")
        row = {"V": el.nV, "E": el.nE}
        for program in ("bfs", "sssp", "cc"):
            e = gg.GASEngineGPU(program)
            vd = initial_vertex_data(program, el.nV, src)
            e.setGraph(el.nV, vd, el.nE, el.weights if program == "sssp" else None,
                       el.src, el.dst, sp)
            e.set_schedule_model(model)
            init_d = torch.from_numpy(vd).to("cuda")
            host = np.empty(el.nV, np.int32)
            lo, hi = (src, src + 1) if program == "bfs" else (0, el.nV)
            outs, r = {}, {}
            for s in C4_SCHEDULES:
                st = {}

                def run(s=s, st=st, lo=lo, hi=hi):
                    e.upload_vertex_data_ptr(init_d.data_ptr(), sp)
                    e.setActive(lo, hi, sp)
                    st["s"] = e.run_schedule(s, max_iterations=el.nV + 2, stream=sp)

                ms = cuda_timed(stream, run, max(2, min(args.steps, 5)), 1)
                e.download_vertex_data(host, sp)
                outs[s] = host.copy()
                r[s] = {"ms": round(ms, 3), "iterations": st["s"].iterations,
                        "pull_iters": st["s"].pull_iters}
            e.close()
            same = all(np.array_equal(outs["auto"], o) for o in outs.values()) and \
                len({v["iterations"] for v in r.values()}) == 1
            best_fixed = min(("auto", "push", "pull"), key=lambda s: r[s]["ms"])
            r["identical_outputs"] = same
            r["learned_speedup_vs_auto"] = round(r["auto"]["ms"] / r["learned"]["ms"], 4)
            r["best_fixed"] = best_fixed
            r["learned_vs_best_fixed"] = round(r[best_fixed]["ms"] / r["learned"]["ms"], 4)
            if program == "bfs":  # the BFS head is the per-level direction rule
                r["learned_runs_as"] = "auto"
            all_ok &= same
            row[program] = r
        del el
        res[name] = row
        free_gpu()
    # warm start on the held-out ER graph (the R-MAT one is C3's graph)
    d = EdgeList.erdos_renyi(1 << scale, 16 << scale, seed=C4_SEED, symmetrize=False)
    warm_model = MLP.load(DATA / "warm_start_head.npz")
    e = gg.GASEngineGPU("pagerank")
    e.setGraph(d.nV, initial_vertex_data("pagerank", d.nV, 0, d.out_degree()), d.nE, None,
               d.src, d.dst, sp)
    r_uni, st_uni = e.pagerank_precision_from(None, PR_DAMPING, PR_TOL, 1000, sp)
    init = e.pagerank_warm_start(warm_model, PR_DAMPING)
    r_warm, st_warm = e.pagerank_precision_from(init, PR_DAMPING, PR_TOL, 1000, sp)
    e.close()
    res["pagerank_warm_start"] = {
        f"rmat{scale}_directed_seed{PR_SEED}": pr_warm,
        "er2^24_directed": {"uniform_iterations": st_uni.iterations,
                            "warm_iterations": st_warm.iterations,
                            "l1_between_results": float(np.abs(r_uni.astype(np.float64) -
                                                               r_warm).sum())}}
    res["parity"] = all_ok
    res["parity_detail"] = ("BFS depths, SSSP distances and CC labels identical under auto, "
                            "push, pull and learned, with equal iteration counts (the oracle pins the "
                            "schedules on C1/C2 and in the GPU tests)")
    return res


# ---------------------------------------------------------------------------
# C5: 64 graphs x (16 BFS sources + 16 PPR seeds) in one graph launch
# ---------------------------------------------------------------------------
BATCH_GRAPHS, BATCH_LANES, BATCH_SEED = 64, 16, 6
BATCH_METRIC = "GTEPS (batched: 64 R-MAT graphs x (16 BFS + 16 PPR))"
PPR_DAMPING, PPR_TOL = 0.85, 1e-6
# A PPR lane stops when its L1 step <= tol; PPR is a d-contraction in L1, so
# the lane is within d/(1-d) * tol of its fixed point (5.67e-6), plus FP32
# rounding of ranks that sum to at most 1.
PPR_L1_BOUND = 8e-6


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


def run_batched(args, check=True):
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
        b.close()
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
    depth = depth_h.numpy().copy()
    rank = rank_h.numpy().copy()
    bfs_units = 0
    for g, el in enumerate(graphs):
        od = el.out_degree().astype(np.int64)
        d = depth[b.vertex_offset(g):b.vertex_offset(g) + el.nV]
        bfs_units += int(((d >= 0) * od[:, None]).sum())
    ppr_iters = r.stats.ppr_iterations
    ppr_units = int(sum(el.nE for el in graphs)) * L * ppr_iters

    with ClockSampler(torch.cuda.current_device()) as clk:
        ms = cuda_timed(stream, lambda: step(False), args.steps, args.warmup)
    clocks = clk.summary()
    ms_e2e = cuda_timed(stream, lambda: step(True), max(1, args.steps), 1)
    st = step(False).stats

    # BFS-only and PPR-only batch times (device-resident)
    ms_bfs = cuda_timed(stream, lambda: b.run(srcs, None, depth_out=depth_d.data_ptr(),
                                              stream=sp), args.steps, 1)
    ms_ppr = cuda_timed(stream, lambda: b.run(None, seeds, PPR_DAMPING, PPR_TOL,
                                              rank_out=rank_d.data_ptr(), stream=sp),
                        args.steps, 1)

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

    ms_plain_bfs = cuda_timed(stream, plain_bfs, 1, 1)
    ms_plain_ppr = cuda_timed(stream, plain_ppr, 1, 1)
    for e in eb + ep:
        e.close()
    offsets = [b.vertex_offset(g) for g in range(G)]
    b.close()

    units = bfs_units + ppr_units
    value = units / (ms * 1e-3) / 1e9
    # roofline of the PPR iteration (pieces + fix + residual kernels), timed by
    # the autotuner with CUDA events: per edge its source index and the L
    # lanes of the source's contribution; per vertex offsets (8 B), seed mask
    # (4 B), old rank, new rank and new contribution (3 x 4L B)
    ppr_bytes = E * (4 + 4 * L) + V * (12 + 12 * L)
    roof = roofline("PPR iteration (k_ppr_pieces + k_ppr_fix + k_ppr_finish)",
                    "ppr_iteration", ppr_bytes, ms_iter, 1,
                    "batched-64" if G == BATCH_GRAPHS else f"batched-{G}",
                    {"traffic_note": "DRAM bytes per iteration; the [V][16] contribution "
                                     "gathers are mostly L2 hits", "piece_edges": piece})
    res = {
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
                "h2d_bytes_per_step": int(srcs.nbytes + V * 4),  # sources + PPR seed mask
                "d2h_bytes_per_step": int(V * L * 8)},
        "gpu_launches": st.kernel_launches * args.steps,
        "graph_launches_per_step": st.graph_launches,
        "split": {"bfs_ms": round(ms_bfs, 3), "ppr_ms": round(ms_ppr, 3),
                  "bfs_gteps": gteps(bfs_units, ms_bfs), "ppr_gteps": gteps(ppr_units, ms_ppr)},
        "plain_sequential": {
            "bfs_ms": round(ms_plain_bfs, 3), "ppr_ms": round(ms_plain_ppr, 3),
            "ppr_iterations_total": plain_ppr_iters[0],
            "bfs_speedup_of_batch": round(ms_plain_bfs / ms_bfs, 3),
            "ppr_speedup_of_batch": round(ms_plain_ppr / ms_ppr, 3),
            "total_speedup_of_batch": round((ms_plain_bfs + ms_plain_ppr) / ms, 3),
            "per_instance_ms_batched": round(ms / (G * L * 2), 5),
            "per_instance_ms_plain": round((ms_plain_bfs + ms_plain_ppr) / (G * L * 2), 5)},
        "roofline": roof,
        "clocks": clocks,
    }
    if check:
        res.update(batched_parity_sample(graphs, srcs, seeds, depth, rank, offsets))
    return res


def batched_parity_sample(graphs, srcs, seeds, depth, rank, offsets):
    """A per-lane sample of the batched results against the oracle: BFS lanes
    0 and 15 of four graphs (the smallest, the largest and two between)
    bit-exact; PPR lanes 0 and 15 of two graphs within the stated L1 bound
    of the FP64 oracle."""
    import oracle
    oracle_threads()
    order = np.argsort([el.nV for el in graphs], kind="stable")
    pick = [int(order[0]), int(order[len(order) // 3]), int(order[2 * len(order) // 3]),
            int(order[-1])]
    bfs_ok, ppr_err = [], []
    for g in pick:
        el = graphs[g]
        og = oracle.Graph(el.nV, el.src, el.dst)
        sl = slice(offsets[g], offsets[g] + el.nV)
        for lane in (0, BATCH_LANES - 1):
            ref, _ = og.bfs(int(srcs[g, lane]))
            bfs_ok.append(bool(np.array_equal(depth[sl, lane], ref)))
        if g in pick[:2]:
            for lane in (0, BATCH_LANES - 1):
                r64, _, _ = og.ppr_fp64(int(seeds[g, lane]), PPR_DAMPING, 1e-12)
                ppr_err.append(float(np.abs(rank[sl, lane].astype(np.float64) - r64).sum()))
        og.close()
    return {"parity": all(bfs_ok) and max(ppr_err) <= PPR_L1_BOUND,
            "parity_detail": {"graphs": pick, "bfs_lanes_bit_exact": bfs_ok,
                              "ppr_lane_l1_vs_fp64": ppr_err, "ppr_l1_bound": PPR_L1_BOUND}}


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
    model = MLP.load(DATA / "schedule_head.npz")
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
        ms_b = cuda_timed(stream, run_b, args.steps, args.warmup)
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
    ms_plain_b = cuda_timed(stream, plain_bfs, 1, 1)
    # the single-source engine's push roofline over the same 16 runs
    e.set_profiling(True)
    e.profile(reset=True)
    plain_bfs()
    torch.cuda.synchronize()
    pe = e.profile()
    e.set_profiling(False)
    e.close()
    b.close()
    out["bfs"] = {"graph": f"rmat-s{scale}-ef{EDGE_FACTOR}-sym seed {GRAPH_SEED}",
                  "V": el.nV, "E": el.nE, "lanes": L, "ms": round(ms_b, 3),
                  "gteps": gteps(bfs_units, ms_b),
                  "plain_one_by_one_ms": round(ms_plain_b, 3),
                  "speedup_vs_plain": round(ms_plain_b / ms_b, 3),
                  "lane0_equals_single_source_run": same,
                  "plain_push_roofline": roofline("k_push (single-source BFS, learned)",
                                                  "bfs_push", pe.push_bytes, pe.push_ms,
                                                  pe.push_launches, f"rmat-s{scale}",
                                                  {"pull_launches": pe.pull_launches}),
                  "roofline": roofline("k_ms_push (16-lane BFS push)", "ms_push",
                                       pb.push_bytes, pb.push_ms, pb.push_launches,
                                       f"rmat-s{scale}",
                                       {"push_share_of_run": round(pb.push_ms / ms_b, 3)})}
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
    ms_p = cuda_timed(stream, run_p, args.steps, args.warmup)
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

    ms_plain_p = cuda_timed(stream, plain_ppr, 1, 0)
    p.close()
    b.close()
    ppr_units = d.nE * L * st.ppr_iterations
    ppr_bytes = d.nE * (4 + 4 * L) + d.nV * (12 + 12 * L)
    out["ppr"] = {"graph": f"rmat-s{scale}-ef{EDGE_FACTOR} directed seed {PR_SEED}",
                  "V": d.nV, "E": d.nE, "lanes": L, "iterations": st.ppr_iterations,
                  "ms": round(ms_p, 3), "gteps": gteps(ppr_units, ms_p),
                  "plain_one_by_one_ms": round(ms_plain_p, 3),
                  "plain_iterations": plain_iters[0],
                  "speedup_vs_plain": round(ms_plain_p / ms_p, 3),
                  "residual": st.ppr_residual,
                  "roofline": roofline("PPR iteration (k_ppr_pieces + k_ppr_fix + "
                                       "k_ppr_finish)", "ppr_iteration", ppr_bytes, ms_iter, 1,
                                       f"rmat-s{scale}-16-seeds", {"piece_edges": piece})}
    total_units = bfs_units + ppr_units
    out["value"] = gteps(total_units, ms_b + ms_p)
    out["ms_per_step"] = round(ms_b + ms_p, 3)
    out["clocks"] = clocks_b
    return out


# ---------------------------------------------------------------------------
# the reference arm: the oracle port of refgas.h on the host cores
# ---------------------------------------------------------------------------
def run_reference(args):
    """The reference's CPU engine (refgas.h, as restated by the oracle port:
    the reference's own build needs moderngpu and a GPU path it cannot have
    here) on the headline step: the same graphs, weights, sources and runs
    as our arm, built by the oracle's own generators so that the product
    library is never loaded.  Each step is a bounded sample of the headline
    step: one of its nine runs (SSSP from source k, k = 0..7, then CC) in
    rotation, on every host thread; the value is the edges of all timed runs
    over their total time, so K >= 9 steps cover the whole step."""
    import oracle
    n_threads = oracle_threads()
    t = time.time()
    nV, s, d = oracle.rmat(args.scale, EDGE_FACTOR, *RMAT_ABC, seed=GRAPH_SEED,
                           symmetrize=True)
    w = oracle.uniform_weights(s, d, 1, 64, WEIGHT_SEED)
    sources = oracle.sample_sources(nV, s, d, N_SOURCES, SOURCE_SEED)
    nVc, sc, dc = oracle.with_grid_islands(nV, s, d, N_ISLANDS, ISLAND_SIDE)
    g = oracle.Graph(nV, s, d)
    gc = oracle.Graph(nVc, sc, dc)
    outdeg = np.bincount(s, minlength=nV)
    log(f"reference arm: scale {args.scale}: V={nV} E={len(s)}; CC graph V={nVc} E={len(sc)}; "
        f"inputs and graph builds {time.time() - t:.1f}s, {n_threads} threads")
    runs = [("sssp", k) for k in range(N_SOURCES)] + [("cc", None)]

    def one(i):
        kind, k = runs[i % len(runs)]
        t0 = time.perf_counter()
        if kind == "sssp":
            dist, _ = g.sssp(w, int(sources[k]))
            sec = time.perf_counter() - t0
            return sec, edges_visited(outdeg, dist, SSSP_UNREACHED)
        gc.cc()
        return time.perf_counter() - t0, len(sc)

    for i in range(args.warmup):
        one(i)
    secs, units = [], 0
    for i in range(max(1, args.steps)):
        sec, u = one(i)
        secs.append(sec)
        units += u
    g.close()
    gc.close()
    value = units / sum(secs) / 1e9
    covered = sorted({runs[i % len(runs)][0] + ("" if runs[i % len(runs)][1] is None else
                                                str(runs[i % len(runs)][1]))
                      for i in range(max(1, args.steps))})
    sample = (f"one run of the step per timed step, in rotation (SSSP from source 0..7, then "
              f"CC), oracle port of refgas.h on {n_threads} threads; runs timed: "
              f"{', '.join(covered)}")
    return {"metric": METRIC.format(scale=args.scale), "value": round(value, 5), "unit": "GTEPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * sum(secs) / len(secs), 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic", "impl": "reference",
            "config": config_dict(args.scale),
            "cpu_baseline": {"value": round(value, 5), "unit": "GTEPS", "cores": n_threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 5), "unit": "GTEPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
def run_configs(args, headline_outputs):
    """The configuration entries of the one-GPU line (each leg frees its
    graphs before the next)."""
    from graphreduce_gb300.learn import DATA, MLP
    want = set(args.configs.split(",")) if args.configs else set()
    model = MLP.load(DATA / "schedule_head.npz")
    out = {}
    t0 = time.time()
    if "c2" in want and headline_outputs is not None:
        par, cpu = c2_oracle_check(headline_outputs)
        out["c2_sssp_cc"] = par
        out["_cpu_baseline"] = cpu
        log(f"c2 oracle check {time.time() - t0:.1f}s")
        t = time.time()
        out["c2_sssp_cc"]["user_programs"] = c2_user_programs(headline_outputs)
        log(f"c2 user programs {time.time() - t:.1f}s")
    if "c1" in want:
        t = time.time()
        out["c1_bfs"] = run_c1(args, model)
        free_gpu()
        log(f"c1 {time.time() - t:.1f}s")
    pr_warm = None
    if "c3" in want:
        t = time.time()
        r = run_pagerank(args, check=True)
        pr_warm = r["warm_start"]
        out["c3_pagerank"] = {k: r[k] for k in (
            "value", "unit", "ms_per_step", "e2e", "config", "roofline", "warm_start",
            "error_vs_fp64_oracle", "parity", "parity_detail")}
        out["c3_pagerank"]["gteps"] = r["value"]
        free_gpu()
        log(f"c3 {time.time() - t:.1f}s")
    if "c4" in want:
        t = time.time()
        out["c4_learned"] = run_c4(args, model, pr_warm)
        free_gpu()
        log(f"c4 {time.time() - t:.1f}s")
    if "c5" in want:
        t = time.time()
        r = run_batched(args, check=True)
        out["c5_batched"] = {k: r[k] for k in (
            "value", "unit", "ms_per_step", "e2e", "config", "split", "plain_sequential",
            "roofline", "graph_launches_per_step", "parity", "parity_detail")}
        out["c5_batched"]["gteps"] = r["value"]
        free_gpu()
        log(f"c5 {time.time() - t:.1f}s")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--schedule", default="learned",
                    choices=["learned", "auto", "generic", "push", "pull", "ordered"])
    ap.add_argument("--configs", default=",".join(ALL_CONFIGS),
                    help="configuration entries added at one GPU (comma list of c1..c5)")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--edges", default="device", choices=["device", "host"],
                    help="edge arrays in HBM or in pinned host memory (NVLink-C2C)")
    ap.add_argument("--workload", default="sssp-cc",
                    choices=["sssp-cc", "batched", "pagerank", "lanes24", "bfs16"])
    ap.add_argument("--pr-scale", type=int, default=PR_SCALE)
    ap.add_argument("--pr-check", action="store_true",
                    help="--workload pagerank: compare with the FP64 oracle")
    ap.add_argument("--batch-graphs", type=int, default=BATCH_GRAPHS)
    ap.add_argument("--sssp", default="batched", choices=["batched", "sequential"],
                    help="the 8 SSSP sources as lanes of one batched run, or one run each")
    ap.add_argument("--launch-list", action="store_true",
                    help="run one device-resident step only (profiling)")
    args = ap.parse_args()
    if args.no_configs:
        args.configs = ""

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)), flush=True)
        return

    if args.workload != "sssp-cc":
        if rank == 0:
            if args.workload == "batched":
                r = run_batched(args, check=not args.launch_list)
            elif args.workload == "pagerank":
                r = run_pagerank(args, check=args.pr_check)
            elif args.workload == "bfs16":
                from graphreduce_gb300.learn import DATA, MLP
                r = run_c1(args, MLP.load(DATA / "schedule_head.npz"))
            else:
                r = run_lanes24(args)
            print(json.dumps(r), flush=True)
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    result, outputs = run_ours(args, rank, world)
    if rank == 0 and outputs is not None:
        if world == 1 and args.configs:
            configs = run_configs(args, outputs)
            cpu = configs.pop("_cpu_baseline", None)
            if cpu is not None and not args.no_cpu_baseline:
                result["cpu_baseline"] = cpu
            if "c2_sssp_cc" in configs:
                c2 = configs["c2_sssp_cc"]
                c2.update({"gteps": result["value"], "e2e_gteps": result["e2e"]["value"],
                           "roofline": result["roofline"],
                           "plain_gteps": result["plain"]["value"],
                           "plain_e2e_gteps": result["plain"]["e2e"]["value"]})
                result["verified_against_oracle"] = c2["parity"]
            result["configs"] = configs
        elif not args.no_cpu_baseline:
            # replicas: the oracle on lane 0 only, on rank 0
            import oracle
            n = oracle_threads()
            ssp, s0 = outputs["ssp"], int(outputs["sources"][0])
            g = oracle.Graph(ssp.nV, ssp.src, ssp.dst)
            t = time.perf_counter()
            d, _ = g.sssp(ssp.weights, s0)
            sec = time.perf_counter() - t
            g.close()
            ev = edges_visited(ssp.out_degree(), d, SSSP_UNREACHED)
            result["cpu_baseline"] = {
                "value": round(ev / sec / 1e9, 5), "unit": "GTEPS", "cores": n, "kind": "port",
                "sample": f"SSSP from source {s0} on the scale-{args.scale} graph, oracle port "
                          f"of refgas.h on {n} threads, {sec:.1f}s"}
            result["verified_against_oracle"] = bool(np.array_equal(d, outputs["lanes"][:, 0]))
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
