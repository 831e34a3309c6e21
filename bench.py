"""Throughput benchmark of the GB300 coarsening path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload rmat22]

One step = one full multilevel coarsening (cuMetis_coarsen's loop: matching,
coarse map, contraction per level, reference stop rule) of the workload.
Metric: coarsened edges/s = sum over levels of the level's directed entries m,
divided by the time.  `value` is measured with the input resident in HBM;
`e2e` goes through the public C-ABI call with pinned host buffers: host->device
copy of the input, coarsening, device->host copy of the coarsest graph.

--impl reference times the reference's CPU coarsening (cuMetis_cpu_match +
cuMetis_cpu_create_cgraph, cuMetis.cu:737-918, as restated in the oracle; the
reference tree is not available where the benchmark runs) on the same
workload, same metric.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
REF_BUDGET_S = 100.0

WORKLOADS = {
    # name: (generator, nparts, description)
    "rmat22": (lambda cm: cm.gen_rmat(22, 16, 0.57, 0.19, 0.19, 1, 1, 100), 256,
               "R-MAT scale 22, edge factor 16, (a,b,c,d)=(.57,.19,.19,.05), weights U[1,100], k=256"),
    "rmat20": (lambda cm: cm.gen_rmat(20, 16, 0.57, 0.19, 0.19, 1, 1, 100), 256,
               "R-MAT scale 20, edge factor 16, (a,b,c,d)=(.57,.19,.19,.05), weights U[1,100], k=256 "
               "(profiling case)"),
    "grid725": (lambda cm: cm.gen_grid2d(725, 725), 64, "2D 5-point grid 725x725, unit weights, k=64"),
    "tri69": (lambda cm: cm.gen_tri_grid(69, 69), 8, "2D triangulated grid 69x69, unit weights, k=8"),
}
# The same workloads built by the oracle's restated generators (identical
# graphs, tests/test_oracle.py), so that the CPU reference arm never loads the
# product library.
REF_WORKLOADS = {
    "rmat22": lambda O: O.gen_rmat(22, 16, 0.57, 0.19, 0.19, 1, 1, 100),
    "rmat20": lambda O: O.gen_rmat(20, 16, 0.57, 0.19, 0.19, 1, 1, 100),
    "grid725": lambda O: O.gen_grid2d(725, 725),
    "tri69": lambda O: O.gen_tri_grid(69, 69),
}


def coarsen_threshold(nvtxs, nparts):
    """k-way Coarsen_threshold = max(n / (20 log2 k), 30 k), cuMetis.cu:3634."""
    lg, k = 0, nparts
    while k > 1:
        lg, k = lg + 1, k >> 1
    return max(nvtxs // (20 * lg) if lg > 0 else nvtxs, 30 * nparts)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def level_bytes(sizes):
    """Algorithmic HBM bytes of each coarsening level (int32 arrays, each
    touched once): matching 4(2m+3n+1), coarse map 4(2n), contraction
    4(3m+3n+1) + 4(2m'+2n'+1)."""
    out = []
    for (n, m), (cn, cm_) in zip(sizes[:-1], sizes[1:]):
        out.append(4 * (5 * m + 2 * cm_ + 8 * n + 2 * cn + 3))
    return out


def dist_setup(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if os.environ.get("CM_BENCH_BACKEND") != "gloo" else "gloo")
    return ws, rank, local


def allreduce_max(x, ws, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, ws, rank):
    """CPU baseline arm: the reference's CPU coarsening (restated) on the host."""
    if rank != 0:
        return
    from oracle import oracle as O
    _, k, desc = WORKLOADS[args.workload]
    og = REF_WORKLOADS[args.workload](O)
    thr = args.coarsen_to or coarsen_threshold(og.n, k)
    mv = O.maxvwgt_rule(int(og.vwgt.sum()), thr)

    def step():
        O.srand(1)
        cur, units = og, 0
        while True:
            cg, _, _ = O.ref_cpu_coarsen_level(cur, mv)
            units += cur.m
            prev, cur = cur, cg
            if not (cur.n > thr and cur.n < 0.75 * prev.n and cur.m > cur.n // 2):
                break
        return units

    # The reference's coarsening is single-threaded host code (one level of
    # R-MAT s22 takes seconds), so the warm-up is one step and the timed
    # region stops after --steps steps or REF_BUDGET_S seconds, whichever
    # comes first; the metric is a rate, so the step count does not bias it.
    step()
    t0 = time.perf_counter()
    units, done = 0, 0
    while done < args.steps:
        units += step()
        done += 1
        if time.perf_counter() - t0 > REF_BUDGET_S:
            break
    dt = time.perf_counter() - t0
    v = units / dt
    line = {"metric": "coarsened edges/s", "value": v, "unit": "edges/s", "n_gpus": args.gpus, "steps": done,
            "warmup": 1, "ms_per_step": dt * 1e3 / done, "steps_requested": args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": args.workload, "description": desc, "nvtxs": og.n, "nedges": og.m,
                       "nparts": k, "coarsen_threshold": thr, "maxvwgt": mv},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "edges/s", "cores": 1, "kind": "port",
                             "sample": "full multilevel coarsening of the workload per step (reference CPU "
                                       "matching + contraction, single-threaded as in the reference)"},
            "e2e": {"value": v, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(g, k, budget_s=20.0, coarsen_to=0):
    from oracle import oracle as O
    import cumetis_gb300 as cm
    og = O.CSR(g.xadj, g.adjncy, g.adjwgt, g.vwgt)
    thr = coarsen_to or cm.coarsen_threshold(g.nvtxs, k)
    mv = O.maxvwgt_rule(int(g.vwgt.sum()), thr)
    O.srand(1)
    t0 = time.perf_counter()
    units, reps = 0, 0
    while time.perf_counter() - t0 < budget_s or reps == 0:
        cg, _, _ = O.ref_cpu_coarsen_level(og, mv)
        units += og.m
        reps += 1
    dt = time.perf_counter() - t0
    return {"value": units / dt, "unit": "edges/s", "cores": 1, "kind": "port",
            "sample": "%d x level 0 of the workload (reference CPU matching + contraction, restated; %.1f s)" %
                      (reps, dt)}


def batch_graphs(count, seed=1):
    """The batched workload: `count` random geometric graphs in the unit
    square, n log-uniform in [1k, 200k], r = sqrt(8/(pi n)) (mean degree 8),
    k uniform in {2, 4, ..., 64}; seeded."""
    import cumetis_gb300 as cm
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(1000), np.log(200000), count)).astype(np.int64)
    ks = 2 * rng.integers(1, 33, count)
    return [cm.gen_rgg(int(n), 8.0, seed=seed * 100003 + i) for i, n in enumerate(ns)], [int(k) for k in ks]


def run_batch(args):
    """Batched partitioning (cm_part_batch): partitions/s over the whole batch."""
    import cumetis_gb300 as cm
    t0 = time.perf_counter()
    graphs, ks = batch_graphs(args.batch_graphs)
    gen_s = time.perf_counter() - t0
    warm = min(len(graphs), 32)
    for _ in range(max(1, args.warmup // 3)):
        cm.part_batch(graphs[:warm], ks[:warm], workers=args.workers)
    clocks = ClockSampler(0)
    clocks.start()
    t1 = time.perf_counter()
    _, cuts, st = cm.part_batch(graphs, ks, workers=args.workers)
    dt = time.perf_counter() - t1
    clk = clocks.stop()
    # The plain per-graph launch for comparison: one context, one graph at a
    # time (cm_part_graph), on the same graphs (every one, or a sample with
    # --plain-sample).
    import torch
    ctx1 = cm.Context(0)
    step_ = max(1, len(graphs) // args.plain_sample) if args.plain_sample > 0 else 1
    sample = list(range(0, len(graphs), step_))
    for i in sample[:4]:
        ctx1.part_graph(graphs[i], ks[i])
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    for i in sample:
        ctx1.part_graph(graphs[i], ks[i])
    plain_dt = time.perf_counter() - t2
    ctx1.close()
    plain_rate = len(sample) / plain_dt
    # the sample's share of the batch's work, to compare rates on equal work
    sample_m = sum(graphs[i].nedges for i in sample)
    n_sum = int(sum(g.nvtxs for g in graphs))
    m_sum = int(sum(g.nedges for g in graphs))
    imb = [float(np.bincount(p, minlength=k).max() * k / g.nvtxs) for g, p, k in
           zip(graphs[:64], cm.part_batch(graphs[:64], ks[:64], workers=args.workers)[0], ks[:64])]
    line = {"metric": "partitions/s", "value": len(graphs) / dt, "unit": "partitions/s", "n_gpus": 1, "steps": 1,
            "warmup": max(1, args.warmup // 3), "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": "batch", "graphs": len(graphs), "sum_nvtxs": n_sum, "sum_nedges": m_sum,
                       "description": "random geometric graphs, n log-uniform [1k,200k], mean degree 8, "
                                      "k uniform in {2..64} even, unit weights",
                       "workers": args.workers, "generation_s": gen_s, "engine_setup_ms": st["setup_ms"],
                       "mean_phase_ms": {"coarsen_in_batch": st["sum_coarsen_ms"] / len(graphs),
                                         "initial_partition": st["sum_init_ms"] / len(graphs),
                                         "refine_project": st["sum_uncoarsen_ms"] / len(graphs)}},
            "edges_per_s": m_sum / dt, "mean_edge_cut": float(np.mean(cuts)),
            "plain_per_graph": {"partitions_per_s": plain_rate, "edges_per_s": sample_m / plain_dt,
                                "graphs": len(sample), "seconds": plain_dt,
                                "batch_speedup_partitions": (len(graphs) / dt) / plain_rate,
                                "batch_speedup_edges": (m_sum / dt) / (sample_m / plain_dt)},
            "mean_imbalance_first64": float(np.mean(imb)), "clocks": clk, "gpu_launches": None,
            "e2e": {"value": len(graphs) / dt, "unit": "partitions/s",
                    "h2d_bytes_per_step": int(4 * (2 * n_sum + len(graphs) + 2 * m_sum)),
                    "d2h_bytes_per_step": int(4 * n_sum)}}
    print(json.dumps(line), flush=True)


def serve_pool(seed=1, count=48):
    """Request graphs of the served workload: half 3D 7-point grids with side
    U[20,120], half R-MAT scale U{14..21} (edge factor 16, weights U[1,100])."""
    import cumetis_gb300 as cm
    rng = np.random.default_rng(seed)
    pool = []
    for i in range(count):
        if i % 2 == 0:
            s = int(rng.integers(20, 121))
            pool.append(("grid3d_%d" % s, cm.gen_grid3d(s, s, s)))
        else:
            sc = int(rng.integers(14, 22))
            pool.append(("rmat%d" % sc, cm.gen_rmat(sc, 16, 0.57, 0.19, 0.19, seed * 1000 + i, 1, 100)))
    return pool


def serve_once(args, pool, rate, duration, drain, seed=7):
    """One served run: Poisson arrivals at `rate` requests/s for `duration`
    seconds, each a random pool graph with k uniform in {8..256};
    submissions beyond --max-queue waiting jobs are rejected; after the window
    the engine drains for at most `drain` seconds, then drops what has not
    finished.  Returns the run's counts and latency percentiles."""
    import cumetis_gb300 as cm
    rng = np.random.default_rng(seed)
    max_n = max(g.nvtxs for _, g in pool)
    max_m = max(g.nedges for _, g in pool)
    eng = cm.Engine(0, workers=args.workers, hbm_budget_bytes=int(args.hbm_budget_gb * 2**30),
                    max_queue=args.max_queue, reserve_nvtxs=max_n, reserve_nedges=max_m)
    for _, g in pool[:4]:  # warm-up
        eng.wait(eng.submit(g, 16))
    eng.stats(reset=True)
    jobs, rejected = [], 0
    t_start = time.perf_counter()
    t_next = t_start
    while True:
        now = time.perf_counter()
        if now - t_start >= duration:
            break
        if now < t_next:
            time.sleep(min(t_next - now, 0.001))
            continue
        _, g = pool[int(rng.integers(0, len(pool)))]
        try:
            jobs.append(eng.submit(g, int(rng.integers(8, 257))))
        except cm.CMError as e:
            if e.code != cm.CM_ERR_LIMIT:
                raise
            rejected += 1
        t_next += rng.exponential(1.0 / rate)
    deadline = time.perf_counter() + drain
    lat, unfinished = [], 0
    for j in jobs:
        while not eng.poll(j) and time.perf_counter() < deadline:
            time.sleep(0.001)
        if eng.poll(j):
            lat.append(eng.wait(j)[2]["latency_ms"])
        else:
            unfinished += 1
    t_end = time.perf_counter()
    eng.close()  # drops jobs that never finished
    lat = np.sort(np.array(lat))
    done = len(lat)
    offered = len(jobs) + rejected
    return {"offered_rate": rate, "offered": offered, "rejected": rejected, "unfinished_dropped": unfinished,
            "completed": done, "failed_frac": (rejected + unfinished) / max(offered, 1),
            "partitions_per_s": done / (t_end - t_start), "seconds": t_end - t_start,
            "latency_ms": {"p50": float(np.percentile(lat, 50)) if done else None,
                           "p99": float(np.percentile(lat, 99)) if done else None,
                           "max": float(lat[-1]) if done else None}}


def run_serve(args):
    """Served partitioning (cm_engine) at --rate requests/s; with
    --serve-rates, a sweep of offered rates (ascending, stopping at the first
    rate where 1% or more of the requests were rejected or not finished),
    reporting the highest rate served within that bound and the run at
    --rate beside it."""
    t0 = time.perf_counter()
    pool = serve_pool(count=args.serve_pool)
    gen_s = time.perf_counter() - t0
    clocks = ClockSampler(0)
    clocks.start()
    sweep = []
    if args.serve_rates:
        for r in [float(x) for x in args.serve_rates.split(",")]:
            res = serve_once(args, pool, r, args.duration, args.drain)
            sweep.append(res)
            if res["failed_frac"] >= 0.01:
                break
    main_run = serve_once(args, pool, args.rate, args.duration, args.drain)
    clk = clocks.stop()
    ok = [r for r in sweep if r["failed_frac"] < 0.01]
    best = max(ok, key=lambda r: r["offered_rate"]) if ok else None
    head = best or main_run
    line = {"metric": "partitions/s", "value": head["partitions_per_s"], "unit": "partitions/s", "n_gpus": 1,
            "steps": head["completed"], "warmup": 4, "ms_per_step": head["seconds"] * 1e3 / max(head["completed"], 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": "serve", "duration_s": args.duration, "drain_s": args.drain,
                       "max_queue": args.max_queue, "pool": len(pool), "pool_generation_s": gen_s,
                       "workers": args.workers, "hbm_budget_gb": args.hbm_budget_gb,
                       "description": "Poisson arrivals; 50% 3D 7-point grids side U[20,120], 50% R-MAT "
                                      "s14-21 (ef 16, weights U[1,100]); k uniform in {8..256}"},
            "max_rate_under_1pct_failed": best["offered_rate"] if best else None,
            "at_max_rate": best, "at_offered_rate": main_run, "sweep": sweep,
            "latency_ms": head["latency_ms"], "clocks": clk, "gpu_launches": None,
            "e2e": {"value": head["partitions_per_s"], "unit": "partitions/s", "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": None}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="rmat22", choices=sorted(WORKLOADS) + ["batch", "serve"])
    ap.add_argument("--workers", type=int, default=16, help="batch/serve: worker threads (one context each)")
    ap.add_argument("--batch-graphs", type=int, default=4096)
    ap.add_argument("--plain-sample", type=int, default=0,
                    help="batch: graphs of the plain per-graph comparison (0: every graph of the batch)")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve: offered requests/s")
    ap.add_argument("--serve-rates", default="", help="serve: offered rates to sweep, e.g. 1,2,5,10,20")
    ap.add_argument("--duration", type=float, default=10.0, help="serve: arrival window in seconds")
    ap.add_argument("--serve-pool", type=int, default=48, help="serve: distinct request graphs")
    ap.add_argument("--hbm-budget-gb", type=float, default=200.0, help="serve: admission budget")
    ap.add_argument("--max-queue", type=int, default=64, help="serve: waiting jobs before submissions are rejected")
    ap.add_argument("--drain", type=float, default=10.0, help="serve: seconds to wait for admitted jobs")
    ap.add_argument("--mode", type=int, default=1,
                    help="matching tie order: 1 = edge hash (default), 0 = lower vertex id")
    ap.add_argument("--coarsen-to", type=int, default=0,
                    help="coarsening threshold in place of the reference's rule max(n/(20 log2 k), 30k)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode0-steps", type=int, default=5,
                    help="steps timed with lowest-id ties (the contract's rule) beside a --mode 1 run")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffers) measurement")
    ap.add_argument("--e2e-pipes", type=int, default=4, help="host threads (contexts) taking alternate e2e steps")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        barrier(ws)
        return
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)

    import torch
    import cumetis_gb300 as cm
    torch.cuda.set_device(local)
    dev = "cuda:%d" % local
    gen, k, desc = WORKLOADS[args.workload]
    g = gen(cm)
    thr = args.coarsen_to or cm.coarsen_threshold(g.nvtxs, k)
    ctx = cm.Context(local)
    ctx.reserve(g.nvtxs, g.nedges)
    dg = g.to_device(dev)
    stream = torch.cuda.current_stream()

    def step():
        h = ctx.coarsen(dg, thr, args.mode)
        sizes = h.sizes()
        h.close()
        return sizes

    for _ in range(args.warmup):
        sizes = step()
    units_per_step = sum(m for (_, m) in sizes[:-1])

    # ---- device-resident timed region ------------------------------------
    ctx.set_stage_timing(True)
    ctx.stage_times(reset=True)
    launches0 = ctx.launch_count()
    barrier(ws)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(ws)
    launches = ctx.launch_count() - launches0
    stages = ctx.stage_times(reset=True)
    ctx.set_stage_timing(False)
    ms = e0.elapsed_time(e1) / args.steps
    ms = allreduce_max(ms, ws, dev)
    value = units_per_step * ws / (ms / 1e3)

    # ---- roofline of the dominant stage ------------------------------------
    # The contraction (k_cmap, the row sorts of every size class on several
    # streams, the count scan and the copy; CUDA events on the caller's
    # stream bracket each stage) is the larger part of the step; the matching
    # (k_match_prep, k_match_first, the round kernel k_match, k_match_finish)
    # is reported beside it in config.stage_roofline.
    peak, peak_kind = measured_peaks()
    lb = level_bytes(sizes)
    n0, m0 = sizes[0]
    pairs = list(zip(sizes[:-1], sizes[1:]))
    group_bytes = {
        "k_match": sum(4 * (2 * m + 3 * n + 1) for (n, m), _ in pairs),
        "contraction": sum(4 * (2 * n) + 4 * (3 * m + 3 * n + 1) + 4 * (2 * cm_ + 2 * cn + 1)
                           for (n, m), (cn, cm_) in pairs),
    }
    per_step_ms = {k_: v / args.steps for k_, v in stages.items() if k_}
    group_ms = {"k_match": per_step_ms.get("k_match", 0.0),
                "contraction": sum(v for k_, v in per_step_ms.items() if k_ != "k_match")}
    stage_roofline = {}
    for g_, b_ in group_bytes.items():
        if group_ms[g_] > 0:
            a_ = b_ / (group_ms[g_] / 1e3) / 1e9
            stage_roofline[g_] = {"bytes_per_step": b_, "ms_per_step": group_ms[g_], "achieved_gbs": a_,
                                  "frac": a_ / peak}
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get(args.workload, {}).get("contraction")
    except Exception:
        pass
    dom = max(group_ms, key=lambda k_: group_ms[k_])
    roof = None
    nlev = max(len(pairs), 1)
    if group_ms[dom] > 0:
        per_launch_bytes = group_bytes[dom] / nlev
        per_launch_ms = group_ms[dom] / nlev
        ach = per_launch_bytes / (per_launch_ms / 1e3) / 1e9
        label = {"contraction": "contraction (k_cmap, k_tiny_units, k_class_rows, k_long_sort/merge/dedup, "
                                "k_count_scan, k_copy_rows, k_copy_class_rows, k_long_copy)",
                 "k_match": "k_match (with k_match_prep, k_match_first, k_match_finish)"}[dom]
        roof = {"kernel": label, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "peak_kind": peak_kind, "traffic": traffic if dom == "contraction" else None,
                "bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_ms}

    # ---- the contract's own tie rule (lowest vertex id) --------------------
    mode0_ms = None
    if args.mode != 0 and args.mode0_steps > 0:
        def step0():
            h = ctx.coarsen(dg, thr, 0)
            h.close()
        step0()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.mode0_steps):
            step0()
        f1.record(stream)
        torch.cuda.synchronize()
        mode0_ms = f0.elapsed_time(f1) / args.mode0_steps
    level_ach = sum(lb) / (ms / 1e3) / 1e9

    # ---- end to end through the C ABI with pinned host buffers --------------
    cn_, cm2 = sizes[-1]
    h2d = 4 * (2 * n0 + 1 + 2 * m0)
    d2h = 4 * (2 * cn_ + 1 + 2 * cm2)
    e2e = None
    if not args.no_e2e:
        # Every step copies its input from pinned host memory, coarsens and
        # reads the coarsest graph back, through the public API (cm_coarsen
        # on host arrays + cm_hierarchy_read_level).  args.e2e_pipes host
        # threads, each with its own context (and stream), take alternate
        # steps, so one step's copies overlap another step's kernels; the
        # host link (about 210 GB/s one way, 340 GB/s both ways at once) is
        # otherwise idle while the GPU computes.
        import threading
        pin = {a: torch.empty(getattr(g, a).shape[0], dtype=torch.int32, pin_memory=True) for a in
               ("xadj", "adjncy", "adjwgt", "vwgt")}
        for a, t in pin.items():
            t.numpy()[:] = getattr(g, a)
        hg = cm.Graph(*(pin[a].numpy() for a in ("xadj", "adjncy", "adjwgt", "vwgt")))
        pipes = max(1, args.e2e_pipes)
        ctxs = [ctx] + [cm.Context(local) for _ in range(pipes - 1)]
        for c in ctxs[1:]:
            c.reserve(g.nvtxs, g.nedges)
        strs = [torch.cuda.Stream() for _ in range(pipes)]  # non-blocking streams, one per pipeline
        outs = [{a: torch.empty(max(s, 1), dtype=torch.int32, pin_memory=True)
                 for a, s in (("xadj", cn_ + 1), ("adjncy", cm2), ("adjwgt", cm2), ("vwgt", cn_))}
                for _ in range(pipes)]

        def e2e_step(i):
            h = ctxs[i].coarsen(hg, thr, args.mode, stream=strs[i])
            last = len(h) - 1
            o = outs[i]
            h.read_level(last, o["xadj"].data_ptr(), o["adjncy"].data_ptr(), o["adjwgt"].data_ptr(),
                         o["vwgt"].data_ptr())
            h.close()

        def run(i, count):
            torch.cuda.set_device(local)
            for _ in range(count):
                e2e_step(i)

        for i in range(pipes):
            e2e_step(i)
        barrier(ws)
        torch.cuda.synchronize()
        e2e_steps = max(pipes, args.steps // pipes * pipes)
        t0 = time.perf_counter()
        ths = [threading.Thread(target=run, args=(i, e2e_steps // pipes)) for i in range(pipes)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
        e2e_ms = allreduce_max(e2e_ms, ws, dev)
        for c in ctxs[1:]:
            c.close()
        # one request alone, no overlap: the latency a single caller sees
        lat = []
        for _ in range(max(1, min(5, args.steps))):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            e2e_step(0)
            torch.cuda.synchronize()
            lat.append((time.perf_counter() - t1) * 1e3)
        e2e = {"value": units_per_step * ws / (e2e_ms / 1e3), "unit": "edges/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms, "steps": e2e_steps, "pipelines": pipes,
               "kind": "throughput of %d pipelined contexts whose steps overlap (not a per-request latency)" % pipes,
               "single_request_ms": float(np.median(lat))}

    line = {"metric": "coarsened edges/s", "value": value, "unit": "edges/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": args.workload, "description": desc, "nvtxs": n0, "nedges": m0, "nparts": k,
                       "coarsen_threshold": thr, "levels": [list(s) for s in sizes], "match_mode": args.mode,
                       "parallelism": "replicas" if ws > 1 else "single-gpu",
                       "l2": "inputs larger than L2 (%.0f MB of CSR)" % (4 * (2 * n0 + 2 * m0) / 1e6),
                       "level_roofline_frac": level_ach / peak, "level_achieved_gbs": level_ach,
                       "mode0_ms_per_step": mode0_ms,
                       "stage_ms_per_step": per_step_ms, "stage_roofline": stage_roofline},
            "roofline": roof, "clocks": clk, "gpu_launches": launches, "e2e": e2e}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(g, k, coarsen_to=args.coarsen_to)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    barrier(ws)


if __name__ == "__main__":
    main()
