#!/usr/bin/env python
"""CCD queries per second of the GB300 C2A conservative-advancement path.

Workload (one step = one batch): 65,536 seeded CCD queries between two
procedural (2,3) torus-knot tubes of 40,000 triangles each (400 x 50), object
A fixed, object B starting at a random pose with a gap of U[0.05, 1] diag,
translating U[0.5, 3] diag towards A inside a cone and turning by U[0, pi]
about a random axis; th_ca = 1e-4 diag (tolerance_d and m_toc_delta),
t_delta = 1e-4, contacts within 2 d + 0.001 enumerated at every TOC, the
reference's traversal order and seeds (triangle 0 of each model).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config2|config4] [--mode reference|canonical|learned]

Before timing: the autotuner picks the launch on a strided sample of the
batch, and a cost model (the seeding network trained on other batches'
measured query costs) orders the batch costliest first.  Each timed step is
the network's inference, the library's ordering kernels and a CUDA-graph
replay of the ordered solve.
value: queries/s with the queries already in HBM (CUDA events on the
launching stream, L2 flushed between steps).
e2e: the same pipeline from host buffers (pose features computed on the host,
queries H2D, results and dense contacts D2H inside the timed region).
roofline: the algorithm's FP64 flops per launch (per-unit counts from the
oracle's own arithmetic) against the FP64 peak measured in the same run.
cpu_baseline: the oracle port on all host cores over a strided sample,
compared with the GPU's results field by field and contact by contact.
--impl reference: the CPU oracle port of the reference (bit-identical to
the reference's own code) on all host cores, on a bounded sample, plus the
same code on one core, one call per query, over a smaller sample
(cpu_baseline.single_core: queries/s, latency mean/p50/p99/max, mean
numCA and work counters per query).
Under torchrun each rank runs its own replica batch (queries are independent).
"""
from __future__ import annotations

import argparse
import json
import os
import signal
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from c2a_gb300 import workloads  # noqa: E402
from c2a_gb300.dist import env_rank  # noqa: E402

METRIC = "CCD queries/s on 1 GB300: learned+batched vs plain GPU CA at equal TOC (≤1e-6 rel)"
UNIT = "queries/s"
NODE_BYTES = 208   # FP64 node fields a BV test reads (R, Tr, l, r, angularRadius, R_loc, first_child)
TRI_BYTES = 144    # two triangles (9 doubles each) per triangle test
# FP64 flops (add/sub, mul, div, sqrt) of the reference's algorithm per unit of work, counted by
# oracle/flop_count.cpp over 1,024 evenly strided queries of this batch: a node-pair test (half an
# expansion: child transform, RSS distance, both motion bounds, descent test) and a leaf triangle
# test (its triangle-level CA iterations included); tests/test_flop_count.py re-counts them
F_BV = 233.6
F_TRI = 353.4
CONTACT_SLOTS = 64
REFERENCE_SAMPLE = 16384  # queries per step of the CPU arms (evenly strided over the batch)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--queries", type=int, default=65536)
    p.add_argument("--cpu-sample", type=int, default=0, help="queries in the CPU-baseline sample (0: auto)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--mode", choices=["reference", "canonical", "learned"], default="reference",
                   help="reference: the reference's results bit for bit; canonical: closest-pair-seeded steps; "
                        "learned: train the seeding network on the uneven pool, then hinted vs plain "
                        "CANONICAL batches on held-out queries")
    p.add_argument("--train", type=int, default=262144, help="--mode learned: training queries")
    p.add_argument("--epochs", type=int, default=6, help="--mode learned: training epochs")
    p.add_argument("--engine", choices=["auto", "warp", "thread", "batched", "spec"], default="auto")
    p.add_argument("--order", choices=["learned", "geometric"], default="learned",
                   help="REFERENCE mode: the work-queue order; learned: a cost model trained on other seeds' "
                        "batches (--order-seeds; costs measured by the library) starts the costliest queries "
                        "first; geometric: "
                        "queries whose bounding spheres approach first.  Results are identical either way.")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--heavy", type=int, default=0,
                   help="--order learned: the costliest queries at the head of the order that get an SM "
                        "sub-partition of their own (c2a_params.heavy_prefix)")
    p.add_argument("--order-seeds", type=int, default=3,
                   help="--order learned: batches of other seeds whose measured costs train the cost model")
    p.add_argument("--workload", choices=["config2", "config4"], default="config2",
                   help="config4: config 2 plus --near grazing near-contact queries (gap log-uniform [1e-6, 1e-3] "
                        "diag, velocity within 5 degrees of the tangent plane); reports the exact distance at "
                        "every near-contact TOC against th_ca")
    p.add_argument("--near", type=int, default=16384, help="--workload config4: near-contact queries")
    return p.parse_args()


class Clocks:
    """nvidia-smi sampling during the timed region (200 ms period)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="c2a_clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.send_signal(signal.SIGTERM)
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": float(max(power))}


def measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def strided(n: int, sample: int) -> np.ndarray:
    """``sample`` query indices spread evenly over a batch of ``n``."""
    sample = max(1, min(sample, n))
    return np.unique(np.linspace(0, n - 1, sample).astype(np.int64))


def cpu_baseline(wl, idx, threads: int):
    """The oracle port (the reference's algorithm, bit-identical) on host threads,
    over the queries ``idx`` of ``wl``."""
    from oracle.oracle import Port, build

    build(ref=False)
    port = Port()
    models = port.models(wl.meshes)
    sub = wl.subset(idx)
    t0 = time.perf_counter()
    res, con = port.solve_batch(models, sub.qint, sub.poses, sub.params, threads=threads,
                                contacts_per_query=CONTACT_SLOTS)
    dt = time.perf_counter() - t0
    return sub.n / dt, dt, res, con


def cpu_latency(wl, idx):
    """The oracle port on one core, each query of ``idx`` its own call: per-query
    times (s) and results."""
    from oracle.oracle import Port, build

    build(ref=False)
    port = Port()
    models = port.models(wl.meshes)
    sub = wl.subset(idx)
    times = np.empty(sub.n)
    parts = []
    for k in range(sub.n):
        t0 = time.perf_counter()
        r, _ = port.solve_batch(models, sub.qint[k:k + 1], sub.poses[k:k + 1], sub.params, threads=1,
                                contacts_per_query=CONTACT_SLOTS)
        times[k] = time.perf_counter() - t0
        parts.append(r)
    return times, np.concatenate(parts)


def run_reference(args, rank, world):
    """--impl reference: the CPU oracle port of the reference on all host
    cores, over an evenly strided sample of the same batch (placed on the host)."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    idx = strided(args.queries, args.cpu_sample or REFERENCE_SAMPLE)
    wl = workloads.config2(n=args.queries, seed=2, device="cpu", indices=idx)
    all_idx = np.arange(wl.n)
    rates, times = [], []
    for _ in range(args.warmup):
        cpu_baseline(wl, all_idx[:min(256, wl.n)], threads)
    for _ in range(args.steps):
        r, dt, _, _ = cpu_baseline(wl, all_idx, threads)
        rates.append(r)
        times.append(dt)
    value = float(wl.n * len(times) / sum(times))
    sample = f"{wl.n} of the {args.queries} queries, evenly strided, every step"
    # the same code on one core, one call per query, over every 16th query of that sample
    one_idx = all_idx[::16]
    lat, lres = cpu_latency(wl, one_idx)
    single_core = {"value": float(len(lat) / lat.sum()), "unit": UNIT, "cores": 1,
                   "sample": f"{len(one_idx)} of the {args.queries} queries, evenly strided, one call each "
                             f"({lat.sum():.1f} s)",
                   "latency_ms": {"mean": 1e3 * float(lat.mean()), "p50": 1e3 * float(np.percentile(lat, 50)),
                                  "p99": 1e3 * float(np.percentile(lat, 99)), "max": 1e3 * float(lat.max())},
                   "per_query_mean": {"numCA": float(lres["numCA"].mean()),
                                      "num_bv_tests": float(lres["num_bv_tests"].mean()),
                                      "num_tri_tests": float(lres["num_tri_tests"].mean())}}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic: seeded procedural torus knots (the reference publishes no scenes)",
            "config": config_dict(wl, args, queries=args.queries), "implementation": implementation_dict(args),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "single_core": single_core},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


ENGINES = {"auto": 0, "warp": 1, "batched": 2, "thread": 3, "spec": 4}
ENGINE_OF = {"auto": "warp"}  # what ENGINE_AUTO runs in REFERENCE mode
KERNELS = {("reference", "auto"): "c2a_solve_warp_kernel", ("reference", "warp"): "c2a_solve_warp_kernel",
           ("reference", "spec"): "c2a_solve_spec_kernel",
           ("reference", "thread"): "c2a_solve_kernel", ("canonical", "auto"): "c2a_canonical_kernel",
           ("canonical", "warp"): "c2a_canonical_kernel", ("canonical", "batched"): "k_dsearch"}


def config_dict(wl, args, queries=None):
    """The workload (identical for both arms); how it runs is in implementation_dict."""
    return {"workload": wl.name, "queries": wl.n if queries is None else int(queries),
            "triangles_per_model": wl.meshes[0].num_tris, "models": "two (2,3) torus-knot tubes, 400 x 50",
            "th_ca": wl.params["th_ca"], "t_delta": wl.params["tol_t"], "qsize": wl.params["qsize"],
            "mode": args.mode,
            "seeding": "plain (triangle 0 of each model, as after EndModel); the learned seeding is measured "
                       "by --mode learned (CANONICAL mode only: REFERENCE results depend on the seed)",
            "contacts_per_query": CONTACT_SLOTS, "parallelism": f"replicas x{args.gpus}"}


def implementation_dict(args, engine=None):
    if args.impl == "reference":
        return {"what": "the CPU oracle port of the reference (bit-identical to the reference compiled here), "
                        "one query per task, all host threads"}
    traversal = {"spec": "reference order by speculative expansion and ordered replay: each warp round tests up to "
                         "16 node pairs the order is about to need (two lanes each, certified FP32 with FP64 where "
                         "undecided), then replays the reference's decisions (FP64, bit-identical)",
                 "warp": "reference order (FP64, bit-identical to the reference); one warp per query, each "
                         "node-pair test split across the lanes",
                 "thread": "reference order, one thread per query"}
    return {"engine": args.engine, "order": args.order if args.mode == "reference" else "geometric",
            "learned_part": "the work-queue order: the seeding network trained as a cost model on measured query "
                            "costs (64 log-cost buckets), queries taken costliest first; the seeding use of the "
                            "network (CANONICAL hints) is measured by --mode learned"
            if args.mode == "reference" and args.order == "learned" else None,
            "launch": "CUDA graph replay of each step (tune.GraphSolve): with the learned order, the network's "
                      "inference, the ordering kernels and the ordered solve in one graph",
            "heavy_prefix": args.heavy if args.mode == "reference" and args.order == "learned" else 0,
            "traversal": traversal.get(engine or ENGINE_OF.get(args.engine, args.engine), "canonical front")
            if args.mode == "reference" else
            "canonical: each step seeded with the exact closest pair (the reference's C2A_Distance), order-free "
            "front traversal; bit-identical to that composition of the reference's functions",
            "l2": "flushed between timed steps (256 MiB write)"}


def run_learned(args, rank, world, local):
    """The learned seeding on the uneven pool (config 3's mesh pool): labels
    from the exact distance query, training on the library's own kernels,
    then held-out CANONICAL batches, plain and hinted, each timed once."""
    import torch
    from c2a_gb300 import api, build, learned

    torch.cuda.set_device(local)
    if rank == 0:
        build.build()
    if rank != 0:
        return
    t0 = time.time()
    clocks = Clocks(local)
    clocks.start()  # sampled over the whole experiment (labels, training and the timed batches)
    engine = api.ENGINE_WARP if args.engine == "warp" else api.ENGINE_BATCHED  # auto: the batched engine
    r = learned.experiment(n_train=args.train, n_eval=args.queries, epochs=args.epochs, pool=12,
                           tri_range=(1000, 200000), engine=engine, seed=3,
                           log=lambda m: print(m, file=sys.stderr, flush=True))
    clk = clocks.stop()
    ev, rp = r.pop("eval_workload"), r.pop("eval_results")
    # roofline of the hinted batch on the FP64 pipe: the reference counters' node-pair and triangle tests at the
    # per-unit flops of the REFERENCE path (the closest-pair search's node pairs are not in those counters, so
    # this understates the work)
    bv, tri = int(r["bv_tests_hinted"]), int(rp["num_tri_tests"].sum())
    fma_peak, add_peak = api.fp64_peak(local)
    achieved = (bv * F_BV + tri * F_TRI) / (r["hinted_ms"] / 1e3) / 1e9
    roofline = {"bound": "fp64", "achieved": achieved, "peak": fma_peak / 1e9, "unit": "GFLOP/s",
                "frac": achieved / (fma_peak / 1e9), "traffic": None, "peak_unfused": add_peak / 1e9,
                "peak_source": "measured in this run: c2a_probe_fp64_peak",
                "kernel": "c2a_canonical_kernel" if engine == api.ENGINE_WARP else "k_dsearch + step waves",
                "note": "counts only the step's node-pair and triangle tests (num_bv_tests, num_tri_tests); the "
                        "closest-pair search that seeds every step is not in those counters"}
    cpu = None
    if not args.no_cpu:  # the oracle port in CANONICAL mode on an evenly strided sample of the held-out batch
        idx = strided(ev.n, args.cpu_sample or 4096)
        ev.params.update(mode=api.MODE_CANONICAL)
        rate, dt, pres, _ = cpu_baseline(ev, idx, os.cpu_count() or 1)
        fields = ("collisionfree", "numCA", "toc", "distance", "mint", "num_bv_tests", "num_tri_tests",
                  "num_contact", "R_toc", "T_toc")
        cpu = {"value": rate, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{len(idx)} of the {ev.n} held-out queries, evenly strided, CANONICAL mode "
                         f"({dt:.1f} s wall)",
               "bit_identical_to_gpu": bool(all(pres[f].tobytes() == rp[f][idx].tobytes() for f in fields)),
               "compared": "every result field but the reported seed pair (among exact ties the GPU reports the "
                           "smallest pair)"}
    e2e = {"value": args.queries / r["e2e_s"], "unit": UNIT, "h2d_bytes_per_step": r["e2e_h2d_bytes"],
           "d2h_bytes_per_step": r["e2e_d2h_bytes"], "identical_results": r["e2e_identical"],
           "api": "features on the host, the network's top-k on the device, c2a_solve_batch_hinted from host "
                  "arrays (learned.solve_hinted)"}
    line = {"metric": METRIC, "value": r["hinted_qps"], "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": r["hinted_ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 CA / bf16 network", "impl": "learned",
            "data": "synthetic: seeded config-3 mesh pool (torus knots, noisy icospheres, clustered soups)",
            "config": {"workload": f"config3 pool of 12 meshes ({min(r['pool_tris'])}-{max(r['pool_tris'])} "
                                   f"triangles), {args.queries} held-out queries", "mode": "canonical",
                       "engine": "warp" if engine == api.ENGINE_WARP else "batched", "train_queries": args.train,
                       "epochs": args.epochs,
                       "network": "50->256->256->256->4096, GELU, bf16 weights, fp32 accumulation", "top_k": 8},
            "plain_qps": r["plain_qps"], "speedup_vs_plain": r["speedup"], "identical_results": r["identical"],
            "differing_fields": r["differ"], "contact_overflow_queries": r["contact_overflow_queries"],
            "true_pair_hint_qps": args.queries / r["oracle_hint_ms"] * 1e3,
            "top1": r["top1"], "top8": r["topk"], "train_loss": r["loss"], "label_s": r["label_s"],
            "train_s": r["train_s"], "wall_s": time.time() - t0, "colliding": r["colliding"],
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": r["e2e_launches"], "clocks": clk}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = env_rank()
    if args.mode == "learned" and args.impl == "ours":
        run_learned(args, rank, world, local)
        return
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo" if args.impl == "reference" else "nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    from c2a_gb300 import api, build

    torch.cuda.set_device(local)
    if rank == 0:
        build.build()
    if dist:
        dist.barrier()
    ctx = api.Context(local)
    if args.workload == "config4":  # the near-contact placement runs the library's exact distance query
        knot = workloads.config2(n=1, seed=2, device=f"cuda:{local}").meshes[0]
        wl = workloads.config4(workloads.gpu_distance_fn(ctx, ctx.model(knot)), n=args.queries, n_near=args.near,
                               seed=4 + rank, device=f"cuda:{local}")
    else:
        wl = workloads.config2(n=args.queries, seed=2 + rank, device=f"cuda:{local}")
    wl.params["mode"] = 1 if args.mode == "canonical" else 0
    wl.params["engine"] = ENGINES[args.engine]
    mid = ctx.model(wl.meshes[0])
    qint = wl.qint.copy()
    qint[:, :2] = mid
    qs = api.make_queries(qint, wl.poses)
    n = wl.n
    d_q = torch.from_numpy(qs.view(np.uint8).copy()).cuda()
    d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(n * CONTACT_SLOTS * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()

    from c2a_gb300 import tune

    tuned = None
    if args.engine == "auto":  # the autotuner's launch for this kind of batch (never changes a result)
        t_tune = time.time()
        tuned = tune.Tuner(ctx, sample=4096, repeats=1).choose(d_q, n, wl.params, CONTACT_SLOTS, stream=stream)
        wl.params.update(engine=tuned["params"]["engine"], warps_per_sm=tuned["params"]["warps_per_sm"])
        tuned = {"choice": tuned["record"]["choice"]["name"], "sample_ms": tuned["record"]["ms"],
                 "sample_queries": tuned["record"]["sample_queries"], "cached": tuned["record"]["cached"],
                 "tune_s": time.time() - t_tune}
    run_engine = tuned["choice"].split("/")[0] if tuned else args.engine
    # every timed step replays a CUDA graph of the solve's launches on fixed buffers
    plain_graph = tune.GraphSolve(ctx, d_q, n, wl.params, d_r, d_c, CONTACT_SLOTS, stream=stream)

    def plain_step():
        plain_graph.replay()

    learned_info = None
    step = plain_step
    if args.mode == "reference" and args.order == "learned":
        from c2a_gb300 import learned

        t_setup = time.time()
        diag = wl.meshes[0].bbox_diag()
        costs, feats = [], []
        for k in range(args.order_seeds):  # training batches of other seeds; their costs measured by the library
            wl_tr = workloads.config2(n=args.queries, seed=1000 + 100 * k + rank, device=f"cuda:{local}")
            q_tr = wl_tr.qint.copy()
            q_tr[:, :2] = mid
            res_tr, _ = ctx.solve(q_tr, wl_tr.poses, wl.params, contacts_per_query=0)
            costs.append(learned.query_cost(res_tr))
            feats.append(learned.features(wl_tr.poses, np.full(wl_tr.n, diag), np.full(wl_tr.n, diag)))
        cost_tr, f_tr = np.concatenate(costs), np.concatenate(feats)
        n_tr = len(cost_tr)
        cut = (n_tr * 4 // 5) // 1024 * 1024  # 80 % to train on, the rest held out
        cost_model = learned.CostOrder(1, seed=rank)
        zeros_tr = np.zeros(n_tr, dtype=np.int32)
        epochs = max(30, -(-1536 // max(cut // 1024, 1)))  # about 1,500 optimizer steps whatever the batch size
        hist = cost_model.fit(f_tr[:cut], zeros_tr[:cut], zeros_tr[:cut], cost_tr[:cut], epochs=epochs)
        held = cost_model.expected(torch.tensor(f_tr[cut:], device="cuda"), torch.tensor(zeros_tr[cut:], device="cuda"),
                                   torch.tensor(zeros_tr[cut:], device="cuda")).cpu().numpy()
        rank_r = float(np.corrcoef(np.argsort(np.argsort(held)), np.argsort(np.argsort(cost_tr[cut:])))[0, 1])
        feat_dev = torch.tensor(learned.features(wl.poses, np.full(n, diag), np.full(n, diag)), device="cuda")
        zeros_dev = torch.zeros(n, dtype=torch.int32, device="cuda")
        learned_info = {"train_queries": cut, "held_out_queries": n_tr - cut, "train_seeds": args.order_seeds,
                        "epochs": epochs, "final_loss": hist[-1], "held_out_rank_correlation": rank_r,
                        "used": rank_r >= 0.6, "setup_s": time.time() - t_setup}

        d_order = torch.arange(n, dtype=torch.int32, device="cuda")
        if args.heavy and wl.params.get("engine", 0) in (ENGINES["auto"], ENGINES["warp"]):
            wl.params["heavy_prefix"] = args.heavy
        # one CUDA graph per step: the network's inference, the ordering kernels and the ordered solve
        ordered_graph = tune.GraphSolve(ctx, d_q, n, wl.params, d_r, d_c, CONTACT_SLOTS, d_order=d_order,
                                        stream=stream,
                                        prologue=lambda: d_order.copy_(cost_model.order(feat_dev, zeros_dev,
                                                                                        zeros_dev)))

        def learned_step():
            ordered_graph.replay()

        if learned_info["used"]:  # a model that does not rank held-out costs leaves the geometric order
            step = learned_step

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    launches0 = ctx.launches()
    clocks = Clocks(local)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()  # evict queries, models and results from L2 before each timed step
            starts[k].record(stream)
            step()
            ends[k].record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    # graph replays do not pass through the library's launch counter: count their kernels per replay
    launches = ctx.launches() - launches0
    if step is plain_step:
        launches += plain_graph.kernels * args.steps
    else:
        launches += ordered_graph.kernels * args.steps
    if learned_info is not None:  # the geometric order on the same batch, for the comparison
        if learned_info["used"]:
            # the network and the schedule per step: assembly, four GEMMs, expected bucket, three ordering kernels
            launches += 9 * args.steps
        res_learned = d_r.cpu().numpy().copy()
        plain_step()
        stream.synchronize()
        pm = []
        for _ in range(args.steps):
            flush.zero_()
            a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a_ev.record(stream)
            plain_step()
            b_ev.record(stream)
            stream.synchronize()
            pm.append(a_ev.elapsed_time(b_ev))
        learned_info["geometric_order_ms_per_step"] = float(np.mean(pm))
        learned_info["geometric_order_value"] = n * args.steps / (sum(pm) / 1000.0)
        learned_info["identical_results"] = bool(np.array_equal(res_learned, d_r.cpu().numpy()))
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = float(sum(step_ms))
    t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    res = d_r.cpu().numpy().view(api.RESULT_DTYPE)
    if (res["status"] & ~(api.QUERY_ITER_CAP | api.QUERY_CONTACT_OVERFLOW)).any():
        raise RuntimeError("a query reported a failure status")
    value = n * world * args.steps / (total_ms / 1000.0)

    # roofline of the CA kernel on its binding resource, the FP64 pipe: the algorithm's flops per launch
    # (per-unit counts x the launch's node-pair and triangle tests) over the launch time, against the FP64
    # peak measured now on this GPU; the HBM view beside it (the trees stay in L2)
    bv = int(res["num_bv_tests"].sum())
    tri = int(res["num_tri_tests"].sum())
    launch_s = (total_ms / args.steps) / 1000.0
    alg_flops = bv * F_BV + tri * F_TRI
    fma_peak, add_peak = api.fp64_peak(local)
    achieved = alg_flops / launch_s / 1e9
    alg_bytes = bv * NODE_BYTES + tri * TRI_BYTES
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    hbm_src = "measured (MEASURED_PEAKS.json)" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0
    roofline = {"bound": "fp64", "achieved": achieved, "peak": fma_peak / 1e9, "unit": "GFLOP/s",
                "frac": achieved / (fma_peak / 1e9), "traffic": None,
                "peak_source": "measured in this run: c2a_probe_fp64_peak (FP64 FMA chains on every SM, best of 5)",
                "peak_unfused": add_peak / 1e9, "frac_of_unfused": achieved / (add_peak / 1e9),
                "kernel": KERNELS.get((args.mode, run_engine)),
                "flops_per_bv_test": F_BV, "flops_per_tri_test": F_TRI, "algorithmic_flops_per_launch": alg_flops,
                "num_bv_tests": bv, "num_tri_tests": tri,
                "hbm": {"achieved": alg_bytes / launch_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                        "frac": alg_bytes / launch_s / 1e9 / hbm_peak, "peak_source": hbm_src,
                        "algorithmic_bytes_per_launch": alg_bytes},
                "note": "traffic: not measured in this run (ncu DRAM bytes of a small capture are in profiles/); "
                        "peak_unfused: the same pipe issuing one add per instruction, the ceiling of code "
                        "compiled without contraction as the reference's is"}

    e2e = None
    if not args.no_e2e:
        h2d_extra = 0
        if learned_info is not None and learned_info["used"]:
            # the learned pipeline from host memory: features H2D, the network's order on the device, then
            # the ordered host-buffer call (queries H2D, results and dense contacts D2H)
            h_feat = torch.empty((n, learned.IN_FEATURES), dtype=torch.float32).pin_memory()
            h2d_extra = h_feat.numel() * 4

            def e2e_call():
                # the features from the host poses, inside the timed region like the queries' copy
                h_feat.copy_(torch.from_numpy(learned.features(wl.poses, np.full(n, diag), np.full(n, diag))))
                with torch.cuda.stream(stream):
                    feat_dev.copy_(h_feat, non_blocking=True)
                    order = cost_model.order(feat_dev, zeros_dev, zeros_dev)
                stream.synchronize()
                return ctx.solve_ordered_host(qint, wl.poses, wl.params, order.data_ptr(),
                                              contacts_per_query=CONTACT_SLOTS)
        else:
            def e2e_call():
                return ctx.solve(qint, wl.poses, wl.params, contacts_per_query=CONTACT_SLOTS)

        rr, cc = e2e_call()  # warm the host path
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        totals = []
        for _ in range(args.steps):
            rr, cc = e2e_call()
            totals.append(cc.total())
        e2e_s = time.perf_counter() - t0
        te = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
        if dist:
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
        e2e_s = float(te.item())
        e2e = {"value": n * world * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": n * api.QUERY_DTYPE.itemsize + h2d_extra,
               "d2h_bytes_per_step": int(n * api.RESULT_DTYPE.itemsize + np.mean(totals) * api.CONTACT_DTYPE.itemsize
                                         + 4),
               "api": ("c2a_solve_batch_ordered_host (host buffers; the order from the network on the device)"
                       if h2d_extra else "c2a_solve_batch (host buffers)")}

    near_info = None
    if args.workload == "config4":
        # the near-contact part: bit-identical to the reference (the CPU sample below covers it), so no TOC is
        # later than the reference's; and where the CA loop reached tolerance_d (numCA >= 2), the exact distance
        # at the returned TOC poses must be within th_ca
        nr = res[args.queries:]
        hit = (nr["collisionfree"] == 0) & (nr["distance"] <= wl.params["tol_d"]) & (nr["numCA"] >= 2) & \
              (nr["distance"] > 0)
        P = np.zeros((int(hit.sum()), workloads.POSE_WIDTH))
        P[:, 0:9] = nr["R_toc"][hit, 0]
        P[:, 9:12] = nr["T_toc"][hit, 0]
        P[:, 24:33] = nr["R_toc"][hit, 1]
        P[:, 33:36] = nr["T_toc"][hit, 1]
        dq = qint[args.queries:][hit].copy()
        dq[:, 2] = nr["seed_a"][hit]
        dq[:, 3] = nr["seed_b"][hit]
        exact = ctx.distance(dq, P)["distance"] if len(dq) else np.zeros(0)
        near_info = {"queries": int(len(nr)), "colliding": int((nr["collisionfree"] == 0).sum()),
                     "toc_checked": int(hit.sum()), "max_exact_distance_at_toc": float(exact.max()) if len(exact)
                     else None, "th_ca": wl.params["th_ca"],
                     "all_within_th_ca": bool((exact <= wl.params["th_ca"] * (1 + 1e-12)).all()),
                     "toc_error_vs_reference": "0 (bit-identical: see cpu_baseline.bit_identical_to_gpu)"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        idx = strided(n, args.cpu_sample or REFERENCE_SAMPLE)
        rate, dt, pres, pcon = cpu_baseline(wl, idx, threads)
        cont = d_c.cpu().numpy().view(api.CONTACT_DTYPE).reshape(n, CONTACT_SLOTS)
        fields = ("collisionfree", "numCA", "translation", "num_contact", "toc", "distance", "mint", "num_bv_tests",
                  "num_tri_tests", "seed_a", "seed_b", "R_toc", "T_toc")
        same = all(pres[f].tobytes() == res[f][idx].tobytes() for f in fields)
        for k, i in enumerate(idx):
            m = min(int(pres[k]["num_contact"]), CONTACT_SLOTS)
            for f in ("type_a", "type_b", "fid_a", "fid_b", "tri_a", "tri_b", "pa", "pb", "distance"):
                same = same and cont[i][:m][f].tobytes() == pcon[k][:m][f].tobytes()
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{len(idx)} of the {n} queries, evenly strided ({dt:.1f} s wall on {threads} threads)",
               "bit_identical_to_gpu": bool(same),
               "compared": "every result field (flags, TOC, iterations, distance, mint, counters, seeds, TOC poses) "
                           "and every contact in its slots"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic: seeded procedural torus knots (the reference publishes no scenes)",
                "config": config_dict(wl, args), "implementation": implementation_dict(args, run_engine), "clocks": clk,
                "gpu_launches": launches, "e2e": e2e,
                "roofline": roofline, "cpu_baseline": cpu,
                "learned_order": learned_info, "tuned_launch": tuned, "near_contact": near_info,
                "collision_fraction": float(1 - res["collisionfree"].mean()),
                "mean_numCA": float(res["numCA"].mean()), "step_ms": step_ms}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
