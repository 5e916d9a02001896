"""Benchmark: node-days/s of the batched ParameterStudy ensemble of graph-ODE
SECIR simulations (1024 samples x 400 nodes, ~30 out-edges per node, 6 age
groups, 90 days, mobility exchange every 0.5 days).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision mixed|mixed_fp64_control|fp64|plain] [--samples S] [--nodes N] [--days D]

One step = one full solve of the ensemble (all samples, all 90 days).
`value`: inputs resident in HBM (mgpu_batch_reset, then mgpu_batch_advance),
device time from CUDA events on the library's stream. `e2e`: the public C ABI
from host buffers per step: mgpu_batch_create (H2D of every input),
mgpu_batch_advance, mgpu_batch_get_state (D2H of every node state).
--impl reference: the FP64 CPU restatement of the reference path (the
checker), all host threads, one graph per thread, on a bounded sample.
After the timed region: the oracle's final states of the CPU-baseline sample
give every precision's per-compartment error (`oracle_error`), and the other
batched precisions run the same ensemble once each (`precision_legs`).
Under torchrun every rank solves its own S samples (weak scaling, no collective).
"""
from __future__ import annotations

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

METRIC = "node-days/s, 1024x400-node SECIR ensemble vs plain GPU FP64; p50/p99 latency"
UNIT = "node-days/s"


def flops_per_attempt(G: int) -> float:
    """Algorithmic FLOPs of one Cash-Karp attempt: 6 RHS of 6G^2 + 90G + 10 flops
    (contact evaluation and G x G contraction, per-group prep, 14 linear flows,
    derivative scatter) plus 55 n for stage combinations, 5th-order sum, error
    combination and norm (n = 10 G)."""
    return 6.0 * (6 * G * G + 90 * G + 10) + 55.0 * 10 * G


def measured_peaks() -> dict:
    """HBM copy rate measured on the GB300s (MEASURED_PEAKS.json beside
    this file), else the stated fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return {"hbm_gbs": float(m["hbm_gbs"]), "source": "measured (MEASURED_PEAKS.json: STREAM-style copy)"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "source": "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_baseline_run(graphs, days, threads, repeats=1):
    """Oracle ensemble on host threads: node-days/s on the given sample."""
    from oracle import oracle as O
    best = None
    for _ in range(repeats):
        _, el, st = O.ensemble_run(graphs, 0.0, days, num_threads=threads)
        nd = sum(g.num_nodes for g in graphs) * days
        v = nd / el
        best = v if best is None else max(best, v)
    return best, st


def run_reference(args, graphs_builder):
    """--impl reference: the CPU restatement of the reference path, all host threads."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sample = max(cores, min(2 * cores, args.samples))
    graphs = graphs_builder(sample)
    for _ in range(args.warmup if args.warmup <= 1 else 1):
        cpu_baseline_run(graphs[:cores], min(args.days, 5.0), cores)
    times = []
    for _ in range(args.steps):
        from oracle import oracle as O
        _, el, _ = O.ensemble_run(graphs, 0.0, args.days, num_threads=cores)
        times.append(el)
    nd = sum(g.num_nodes for g in graphs) * args.days
    v = nd / float(np.median(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": float(np.median(times)) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": workload_config(args),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{sample} of {args.samples} samples x {args.nodes} nodes x {args.days:g} days per "
                                   f"step, one graph per thread"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args):
    return {"workload": f"ParameterStudy ensemble: {args.samples} samples x {args.nodes}-node mobility graph, "
                        f"6 age groups, ~30 out-edges/node, {args.days:g} days, exchange every 0.5 d",
            "samples": args.samples, "nodes": args.nodes, "age_groups": 6, "days": args.days,
            "integrator": "Cash-Karp 5(4), abs 1e-10, rel 1e-5, dt0 0.1",
            "precision": args.precision,
            "l2": "inputs larger than L2 (node parameters and states of the ensemble exceed 129 MB)"}


def schedule_leg(N, ctx, args, ms_step, prec):
    """Cost of the per-interval launch schedule itself: a two-node graph with one
    edge each way runs the same kernels per 0.5-day interval (phase bookkeeping,
    instance order, node solve, return, four exact-scan passes, fallback,
    cleanup, departure) with almost no work, so its time per interval is the
    launch and bookkeeping overhead that one persistent kernel could at most save."""
    from memilio_gb300 import workloads as W
    g = W.mobility_graph(seed=9, N=2, G=6, out_degree=1)
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=prec))
    b.advance(args.days)  # warm-up (captures the interval's CUDA graph)
    st0 = b.stats()
    ms = []
    for _ in range(3):
        b.reset(0.0)
        b.advance(args.days)
        ms.append(b.timing()["advance_ms"])
    st1 = b.stats()
    b.close()
    intervals = int(round(args.days / 0.5))
    launches = (st1["kernel_launches"] - st0["kernel_launches"]) / 3 / intervals
    per = min(ms) / intervals
    return {"us_per_interval": per * 1e3, "launches_per_interval": launches, "intervals_per_step": intervals,
            "ms_per_step": min(ms), "share_of_step": min(ms) / ms_step,
            "workload": "2-node graph, one edge each way, 6 age groups: the interval schedule without work"}


def uneven_leg(N, ctx, args):
    """Uneven batch: graphs with log-uniform node counts in [1, 2000], 1-6 age
    groups, horizons U[30, 180] days, out-degree U{0..50}, mixed precision, all
    in one batch (one launch per age-group count and interval)."""
    from memilio_gb300 import workloads as W
    graphs, horizons = W.uneven_batch(num_graphs=args.uneven, seed=3)
    nd = W.node_days(graphs, horizons)
    b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    tune = b.autotune()
    b.advance(0.0, horizons)  # warm-up
    ms = []
    for _ in range(2):
        b.reset(0.0)
        b.advance(0.0, horizons)
        ms.append(b.timing()["advance_ms"])
    st = b.stats()
    b.close()
    return {"value": nd / (min(ms) / 1e3), "unit": UNIT, "graphs": len(graphs),
            "nodes": int(sum(g.num_nodes for g in graphs)), "node_days": nd, "ms": min(ms),
            "sequential_exchanges": st["sequential_exchanges"], "autotune": tune,
            "workload": f"{len(graphs)} graphs, nodes logU[1,2000], groups U{{1..6}}, horizon U[30,180] d, "
                        "out-degree U{0..50}, mixed precision"}


def serving_leg(N, ctx, args):
    """Serving: requests of the uneven distribution arriving Poisson at each rate
    for a fixed window; continuous batching (mgpu_server_*); latency from
    submission to completion; throughput = completed node-days / wall time."""
    from memilio_gb300 import workloads as W
    pool, horizons = W.uneven_batch(num_graphs=512, seed=11)
    rng = np.random.default_rng(13)
    # the plain per-request FP64 path on a few requests, one after another
    pk = [i for i in range(len(pool)) if pool[i].num_nodes <= 400][:4]
    p_ms, p_nd = 0.0, 0.0
    for i in pk:
        pb = N.Batch(ctx, [pool[i]], 0.0, N.solver_opts(precision=N.PRECISION_FP64_PLAIN))
        pb.advance(float(horizons[i]))
        p_ms += pb.timing()["advance_ms"]
        p_nd += pool[i].num_nodes * horizons[i]
        pb.close()
    out = {"window_s": args.serve_seconds, "rebatch_max_graphs": args.serve_rebatch, "plain_fp64_per_request": {"value": p_nd / (p_ms / 1e3), "unit": UNIT,
                                                                       "sample": f"{len(pk)} requests"},
           "rates": []}
    for lam in args.serve_rates:
        srv = N.Server(ctx_device(ctx), N.server_opts(max_batches=16, phases_per_launch=2,
                                                      rebatch_max_graphs=args.serve_rebatch))
        t_start = time.perf_counter()
        next_t = t_start + rng.exponential(1.0 / lam)
        submitted, nd_done, lat, k = {}, 0.0, [], 0
        while True:
            now = time.perf_counter()
            while now >= next_t and now - t_start < args.serve_seconds:
                i = k % len(pool)
                k += 1
                submitted[srv.submit(pool[i], 0.0, float(horizons[i]))] = i
                next_t += rng.exponential(1.0 / lam)
            srv.step()
            while True:
                t = srv.take()
                if t is None:
                    break
                rid, _, l = t
                i = submitted.pop(rid)
                nd_done += pool[i].num_nodes * horizons[i]
                lat.append(l)
            if now - t_start >= args.serve_seconds and not submitted:
                break
            if now - t_start > args.serve_seconds + 120.0:
                break  # drain limit
        wall = time.perf_counter() - t_start
        merges = srv.num_merges()
        srv.close()
        lat_ms = np.array(lat) * 1e3
        out["rates"].append({"lambda_per_s": lam, "completed": len(lat), "unfinished": len(submitted),
                             "p50_ms": float(np.percentile(lat_ms, 50)) if len(lat) else None,
                             "p99_ms": float(np.percentile(lat_ms, 99)) if len(lat) else None,
                             "node_days_per_s": nd_done / wall, "wall_s": wall, "merges": merges})
    return out


def ctx_device(ctx) -> int:
    import torch
    return torch.cuda.current_device()


def h2d_bytes(graphs) -> int:
    """Bytes mgpu_batch_create copies to the device: every input array once
    (arrays shared by several graphs of the batch are uploaded once)."""
    seen, total = set(), 0
    for g in graphs:
        arrs = [g.params, g.contact_baseline, g.contact_minimum, g.damping_times, g.damping_values, g.init_state,
                g.edge_src, g.edge_dst, g.edge_coeff_baseline, g.edge_damping_times, g.edge_damping_values]
        if g.edge_coeff_minimum is not None:
            arrs.append(g.edge_coeff_minimum)
        for a in arrs:
            key = (a.__array_interface__["data"][0], a.nbytes)
            if a.nbytes and key not in seen:
                seen.add(key)
                total += a.nbytes
    return int(total)


# Algorithmic bytes per active (node, age group) item and launch of the mixed
# exchange passes (float-float states: 80 B per state row read or written):
#   return: state read + next-state write 160, own snapshot 40, factors 8,
#           return-time rates 48  (snapshot rows of the sources and the
#           ensemble-shared coefficients are counted once, as the own rows)
#   depart: state read + write 160, departure state write 80, snapshot 40, factors 8
#   (the node pass, return-time rates and departure snapshot, runs inside the
#   mixed node kernel)
BYTES_PER_ITEM = {"return": 256, "depart": 288, "exact": 256}
# DRAM bytes (read + write) per (node, group) item of one launch, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of a 256-sample x
# 400-node ensemble (per-graph passes): 209.7 MB (return, with the pre-return
# copy for the exact path) and 154.9 MB (departure) for 614,400 items. The
# traffic grows in proportion to the items, so it scales to the full launch.
NCU_BYTES_PER_ITEM = {"return": (158.565376e6 + 51.165696e6) / 614400, "depart": (106.436608e6 + 48.486144e6) / 614400}
# the same for the mixed node kernel, per node instance of one interval
# (225.3 MB for 102,400 instances)
NCU_ODE_BYTES_PER_INSTANCE = (178.253824e6 + 47.016960e6) / 102400


# --precision names, the ABI's precision constants and the arithmetic each computes in
PRECISION_NAMES = {"mixed": "PRECISION_MIXED", "mixed_fp64_control": "PRECISION_MIXED_FP64_CONTROL",
                   "fp64": "PRECISION_FP64", "plain": "PRECISION_FP64_PLAIN"}
DTYPES = {"mixed": "f32 (float-float state)", "mixed_fp64_control": "f32 (f64 state, error norm, controller)",
          "fp64": "f64", "plain": "f64"}
ERROR_FLOOR = 1e-6  # absolute floor of the per-compartment error, a fraction of the age group's population


def precision_error(O, got, ref, graphs) -> dict:
    """Per-compartment relative error of final states against the oracle's:
    max and percentiles over every compartment of every sampled graph, with the
    floor stated; and the largest error relative to the age group's population."""
    errs = [O.compartment_error(a, r, g.num_groups, ERROR_FLOOR) for a, r, g in zip(got, ref, graphs)]
    grp = max(float(O.compartment_error(a, r, g.num_groups, 1.0).max()) for a, r, g in zip(got, ref, graphs))
    return dict(O.error_summary(errs), floor=ERROR_FLOOR, max_group_scaled=grp,
                measure="|gpu - oracle| / max(|oracle|, floor * N_group), final states",
                sample=f"{len(graphs)} samples x {graphs[0].num_nodes} nodes, every compartment of every node")


def precision_legs(N, ctx, graphs, days, prec_main, O, ref_final, sample) -> dict:
    """The batched precisions other than the headline's on the first samples of
    the same ensemble, one advance each: node-days/s (device time) and the error
    of the oracle-checked samples."""
    out = {}
    for name in ("fp64", "mixed_fp64_control", "mixed"):
        p = getattr(N, PRECISION_NAMES[name])
        if p == prec_main:
            continue
        b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=p))
        b.advance(0.5)  # warm-up (the interval's CUDA graph is captured here)
        b.reset(0.0)
        b.advance(days)
        ms = b.timing()["advance_ms"]
        st = b.stats()
        got = b.states()[:len(sample)]
        b.close()
        out[name] = {"value": sum(g.num_nodes for g in graphs) * days / (ms / 1e3), "unit": UNIT,
                     "ms": ms, "samples": len(graphs), "dtype": DTYPES[name],
                     "attempts_per_node_day": (st["accepted_steps"] + st["rejected_steps"]) /
                                              (sum(g.num_nodes for g in graphs) * days),
                     "oracle_error": precision_error(O, got, ref_final, sample)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=list(PRECISION_NAMES))
    ap.add_argument("--samples", type=int, default=1024)
    ap.add_argument("--nodes", type=int, default=400)
    ap.add_argument("--days", type=float, default=90.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--uneven", type=int, default=4096, help="graphs of the uneven-batch leg (0 = skip)")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="arrival window per rate (0 = skip)")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[50.0, 200.0, 800.0])
    ap.add_argument("--serve-rebatch", type=int, default=0,
                    help="re-batching: merge running batches of at most this many requests (0 = off)")
    ap.add_argument("--legs-samples", type=int, default=256,
                    help="samples of the ensemble the other batched precisions run once each (0 = skip)")
    args = ap.parse_args()

    from memilio_gb300 import replicas as R
    from memilio_gb300 import workloads as W

    base = W.mobility_graph(seed=1, N=args.nodes)

    def graphs_builder(count):
        # every rank its own samples (rank 0: the single-GPU ensemble)
        return R.ensemble_for_rank(count, dist_info()[0], base=base)

    if args.impl == "reference":
        run_reference(args, graphs_builder)
        return

    rank, world, local = dist_info()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    from memilio_gb300 import _native as N
    from memilio_gb300 import build as B
    B.build()
    prec = getattr(N, PRECISION_NAMES[args.precision])
    graphs = graphs_builder(args.samples)
    nd_step = sum(g.num_nodes for g in graphs) * args.days
    ctx = N.Context(local)
    batch = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=prec))

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        batch.reset(0.0)
        batch.advance(args.days)
    st0 = batch.stats()
    dev_ms = []
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            batch.reset(0.0)
            batch.advance(args.days)
            dev_ms.append(batch.timing()["advance_ms"])
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    barrier()
    st1 = batch.stats()
    launches = (st1["kernel_launches"] - st0["kernel_launches"])
    exchange_stats = {k: (st1[k] - st0[k]) // args.steps for k in ("underflow_fixes", "sequential_exchanges", "scan_items")}
    ms_step = float(np.sum(dev_ms)) / args.steps
    ms_max = R.max_over_ranks(ms_step, device="cuda")
    value = R.job_throughput(nd_step, ms_max / 1e3, world)
    final = batch.state_flat()
    attempts_step = (st1["accepted_steps"] + st1["rejected_steps"] - st0["accepted_steps"] - st0["rejected_steps"]) \
        / args.steps

    # per-kernel device times (profile mode: events around the node solves and the exchange passes)
    prof = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=prec, profile=True))
    prof.advance(args.days)
    tm = prof.timing()
    dev_bytes = prof.device_bytes()
    prof.close()
    ode_ms_launch = tm["ode_ms"] / max(tm["ode_launches"], 1)
    flops_launch = tm["attempts"] * flops_per_attempt(6) / max(tm["ode_launches"], 1)
    clocks = clk.summary()
    f_sm = clocks["sm_mhz"] or 1965.0
    num_sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = num_sms * 128 * 2 * f_sm * 1e6 / 1e12  # TFLOP/s at the sampled clock
    achieved = flops_launch / (ode_ms_launch / 1e3) / 1e12
    mixed = prec in (N.PRECISION_MIXED, N.PRECISION_MIXED_FP64_CONTROL)
    roofline = {"bound": "fp32" if mixed else "fp64",
                "kernel": {N.PRECISION_MIXED: "k_ode_mixed<6,false>", N.PRECISION_MIXED_FP64_CONTROL:
                           "k_ode_mixed<6,true>", N.PRECISION_FP64: "k_ode_batched<6>"}.get(prec, "k_ode_plain"),
                "achieved": achieved, "unit": "TFLOP/s",
                "peak": fp32_peak if mixed else 1.25,
                "peak_source": (f"nominal FP32 FMA rate ({num_sms} SMs x 128 lanes x 2) at the sampled median SM "
                                "clock; MEASURED_PEAKS.json holds no FP32 figure") if mixed else
                               "nominal GB300 FP64 rate",
                "frac": None,
                "traffic": (NCU_ODE_BYTES_PER_INSTANCE * sum(g.num_nodes for g in graphs)
                            if prec == N.PRECISION_MIXED else None),
                "traffic_source": "ncu DRAM bytes per node instance of a 256-sample capture, times the instances",
                "ode_share_of_step": tm["ode_ms"] / max(tm["advance_ms"], 1e-9),
                "exchange_ms_per_step": tm["exchange_ms"], "ode_ms_per_step": tm["ode_ms"],
                "algorithmic_flops_per_launch": flops_launch, "avg_launch_ms": ode_ms_launch}
    roofline["frac"] = roofline["achieved"] / roofline["peak"]
    parts = {"ode": tm["ode_ms"], "prep": tm["prep_ms"], "return": tm["return_ms"], "exact": tm["exact_ms"],
             "depart": tm["depart_ms"]}
    roofline["parts_ms_per_step"] = parts
    dominant = max(parts, key=parts.get)
    if mixed and dominant in ("return", "depart", "exact"):
        # the exchange pass that dominates the step, against the measured HBM copy rate
        peaks = measured_peaks()
        items = sum(g.num_nodes * g.num_groups for g in graphs)
        launches_active = args.days / 0.5 / 2  # one return and one departure per day
        if dominant == "exact":
            items = exchange_stats["scan_items"] / launches_active  # scanned (node, group) items per return
        bytes_launch = items * BYTES_PER_ITEM[dominant]
        ms_launch = parts[dominant] / launches_active
        ach = bytes_launch / (ms_launch / 1e3) / 1e9
        roofline = dict(roofline, bound="hbm", kernel={"return": "k_xs_return / k_xf_return",
                                                      "depart": "k_xs_depart / k_xf_depart",
                                                      "exact": "k_xf_scan"}[dominant],
                        achieved=ach, unit="GB/s", peak=peaks["hbm_gbs"], peak_source=peaks["source"],
                        frac=ach / peaks["hbm_gbs"], algorithmic_bytes_per_launch=bytes_launch,
                        traffic=(items * NCU_BYTES_PER_ITEM[dominant] if dominant in NCU_BYTES_PER_ITEM else None),
                        traffic_source=("ncu dram__bytes_read.sum + dram__bytes_write.sum per item of a "
                                        "256-sample capture, times the items of this launch"),
                        avg_launch_ms=ms_launch, ode_roofline={"bound": "fp32", "achieved_tflops": achieved,
                                                               "peak_tflops": fp32_peak,
                                                               "frac": achieved / fp32_peak})
    roofline["dominant_part"] = dominant

    # end to end through the C ABI from host buffers
    e2e = None
    if not args.no_e2e:
        h2d = h2d_bytes(graphs)
        d2h = batch.total * 8
        e2e_t, parts_t = [], []
        for k in range(2):
            t0 = time.perf_counter()
            b2 = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=prec))
            t1 = time.perf_counter()
            b2.advance(args.days)
            t2 = time.perf_counter()
            out = b2.state_flat()
            t3 = time.perf_counter()
            b2.close()
            e2e_t.append(time.perf_counter() - t0)
            parts_t.append({"create_s": t1 - t0, "advance_s": t2 - t1, "d2h_s": t3 - t2})
        best = int(np.argmin(e2e_t))
        e2e = {"value": world * nd_step / min(e2e_t), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "parts": parts_t[best]}
        assert np.array_equal(out, final)
    batch.close()

    # the plain per-graph FP64 drop-in on a sample of the same ensemble (graphs
    # run one after another, so its rate does not depend on the sample size)
    plain = None
    if rank == 0 and not args.no_plain and prec != N.PRECISION_FP64_PLAIN:
        k = min(2, len(graphs))
        pb = N.Batch(ctx, graphs[:k], 0.0, N.solver_opts(precision=N.PRECISION_FP64_PLAIN))
        pb.advance(args.days)
        p_ms = pb.timing()["advance_ms"]
        pb.close()
        p_val = k * args.nodes * args.days / (p_ms / 1e3)
        plain = {"value": p_val, "unit": UNIT, "sample": f"{k} samples x {args.nodes} nodes x {args.days:g} days",
                 "speedup_of_value": value / world / p_val}

    schedule = schedule_leg(N, ctx, args, ms_step, prec) if rank == 0 and prec != N.PRECISION_FP64_PLAIN else None
    uneven = uneven_leg(N, ctx, args) if rank == 0 and args.uneven > 0 else None
    serving = serving_leg(N, ctx, args) if rank == 0 and args.serve_seconds > 0 else None

    cpu, oracle_error, legs = None, None, None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        cores = os.cpu_count() or 1
        sample = graphs[:cores]
        ref_final, el, _ = O.ensemble_run(sample, 0.0, args.days, num_threads=cores)
        v = sum(g.num_nodes for g in sample) * args.days / el
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{len(sample)} samples x {args.nodes} nodes x {args.days:g} days, one graph per thread"}
        # the same runs are the checker: every precision's final states against them
        got = np.split(final[:sum(g.num_nodes * g.n for g in sample)], np.cumsum([g.num_nodes * g.n for g in sample])[:-1])
        oracle_error = dict(precision_error(O, got, ref_final, sample), precision=args.precision)
        if args.legs_samples > 0 and prec != N.PRECISION_FP64_PLAIN:
            legs = precision_legs(N, ctx, graphs[:max(args.legs_samples, len(sample))], args.days, prec, O,
                                  ref_final, sample)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPES[args.precision],
            "data": "synthetic (seeded)", "config": workload_config(args), "clocks": clocks,
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu,
            "attempts_per_node_day": attempts_step / nd_step, "wall_s_timed": t_wall,
            "exchange_per_step": exchange_stats, "plain_fp64": plain, "device_bytes": dev_bytes,
            "uneven_batch": uneven, "serving": serving, "oracle_error": oracle_error, "precision_legs": legs,
            "schedule_overhead": schedule,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
