"""Launch autotuner and CUDA-graph replay for batched solves.

How a batch is launched never changes a result: the engine (one warp per
query, one thread per query, speculative expansion, the batched CANONICAL
engine) and the launch shape (resident warps per SM) only change the time.
Which launch is fastest depends on the GPU, the meshes and the batch, so the
tuner measures it:

  * a sample of the caller's own batch (evenly strided queries, the batch's
    models and parameters) is solved with every candidate launch, each timed
    with CUDA events on the launching stream after an untimed warm-up;
  * launch shapes (warps per SM) are candidates only where the sample is the
    whole batch: a sample's time is set by its heaviest queries, which favour
    fewer warps per SM, while a whole batch favours full occupancy;
  * every candidate's results and contacts must equal the first candidate's
    bit for bit (a launch choice that changed a result would be a defect, and
    the tuner raises);
  * the first candidate is the library's default launch, and another
    replaces it only when it is at least 5 % faster on the sample (a
    sample's time is set by its heaviest queries, so small differences do
    not carry over to the whole batch);
  * the chosen candidate is kept per workload signature (GPU, SM count,
    mode, contact enumeration, triangle counts of the models used, batch size
    to a power of two) in a JSON cache, so later batches of the same kind
    launch without tuning.

GraphSolve captures one solve launch sequence (the work counter's reset, the
schedule kernel, the solve kernel) for fixed device buffers as a CUDA graph;
replay() re-runs it on whatever the buffers hold, for loops that solve a
batch of the same shape every frame.
"""
from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from . import api

CACHE = os.environ.get("C2A_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "c2a_gb300",
                                                           "tune.json")

# (engine, warps per SM; 0 = the most that fit)
REFERENCE_CANDIDATES = [(api.ENGINE_WARP, 0), (api.ENGINE_WARP, 4), (api.ENGINE_THREAD, 0), (api.ENGINE_SPEC, 0)]
CANONICAL_CANDIDATES = [(api.ENGINE_WARP, 0), (api.ENGINE_WARP, 8), (api.ENGINE_BATCHED, 0)]
ENGINE_NAMES = {api.ENGINE_AUTO: "auto", api.ENGINE_WARP: "warp", api.ENGINE_BATCHED: "batched",
                api.ENGINE_THREAD: "thread", api.ENGINE_SPEC: "spec"}


def _torch():
    import torch

    return torch


def signature(ctx, d_queries, n: int, params: dict, contacts_per_query: int) -> str:
    """The cache key of a batch: GPU, SM count, mode, contacts, the triangle
    counts of the models its queries use (up to four, largest first) and n to
    a power of two."""
    torch = _torch()
    q = d_queries.view(-1, api.QUERY_DTYPE.itemsize)[:n]
    ids = torch.unique(q[:, 0:8].contiguous().view(torch.int32).reshape(-1)).cpu().numpy()
    tris = sorted((ctx.model_info(int(i))[0] for i in ids if i >= 0), reverse=True)[:4]
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    mode = "canonical" if params.get("mode", 0) == api.MODE_CANONICAL else "reference"
    return (f"{props.name}|sm{props.multi_processor_count}|{mode}|contacts{int(params.get('with_contacts', 1))}"
            f"x{contacts_per_query}|tris{'-'.join(map(str, tris))}|n2^{max(0, math.ceil(math.log2(max(n, 1))))}")


def _load(path: str) -> dict:
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store(path: str, table: dict):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


class Tuner:
    """Picks the fastest launch for a kind of batch (see the module notes)."""

    def __init__(self, ctx, cache: str | None = CACHE, sample: int = 4096, repeats: int = 2, margin: float = 0.05):
        self.ctx, self.cache, self.sample, self.repeats, self.margin = ctx, cache, sample, repeats, margin

    def candidates(self, params: dict):
        return CANONICAL_CANDIDATES if params.get("mode", 0) == api.MODE_CANONICAL else REFERENCE_CANDIDATES

    def choose(self, d_queries, n: int, params: dict, contacts_per_query: int = 64, stream=None,
               retune: bool = False) -> dict:
        """The tuned parameters for this batch (params with engine and
        warps_per_sm set) and how they were found: {"params", "record"}.
        d_queries: the batch as a device uint8 tensor of n query records."""
        key = signature(self.ctx, d_queries, n, params, contacts_per_query)
        table = _load(self.cache) if self.cache else {}
        rec = None if retune else table.get(key)
        if rec is None:
            rec = self.measure(d_queries, n, params, contacts_per_query, stream)
            rec["signature"] = key
            if self.cache:
                table = _load(self.cache)
                table[key] = rec
                _store(self.cache, table)
            rec = dict(rec, cached=False)
        else:
            rec = dict(rec, cached=True)
        out = dict(params, engine=rec["choice"]["engine"], warps_per_sm=rec["choice"]["warps_per_sm"])
        return {"params": out, "record": rec}

    def measure(self, d_queries, n: int, params: dict, contacts_per_query: int = 64, stream=None) -> dict:
        """Times every candidate on the sample; raises if any candidate's results differ."""
        torch = _torch()
        qs = d_queries.view(-1, api.QUERY_DTYPE.itemsize)[:n]
        k = min(self.sample, n)
        idx = np.unique(np.linspace(0, n - 1, k).astype(np.int64))
        sub = qs[torch.as_tensor(idx, device=qs.device)].contiguous()
        k = len(idx)
        slots = contacts_per_query
        d_r = torch.zeros(k * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=qs.device)
        d_c = torch.zeros(max(1, k * slots) * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device=qs.device)
        s = stream or torch.cuda.Stream()
        first = None
        times = {}
        best = math.inf
        for eng, wps in self.candidates(params):
            if wps and k < n:
                # a strided sample's time is set by its heaviest queries, which run faster with fewer warps
                # sharing an SM sub-partition, while a whole batch runs faster at full occupancy (4 warps per
                # SM: 8.6 % faster on a 4,096-query config-2 sample, 14 % slower on the 65,536-query batch);
                # launch shapes are therefore tuned only where the sample is the whole batch
                continue
            prm = dict(params, engine=eng, warps_per_sm=wps)
            name = f"{ENGINE_NAMES[eng]}/{wps or 'max'}"

            def run():
                d_r.zero_()
                d_c.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(s):
                    a.record(s)
                    self.ctx.solve_device(sub.data_ptr(), k, prm, d_r.data_ptr(), d_c.data_ptr() if slots else None,
                                          slots, stream=s.cuda_stream)
                    b.record(s)
                s.synchronize()
                return a.elapsed_time(b)

            warm = run()
            got = (d_r.cpu().numpy().tobytes(), d_c.cpu().numpy().tobytes())
            if first is None:
                first = (name, got)
            elif got != first[1]:
                raise RuntimeError(f"launch {name} changed the results of {first[0]}: a defect, not a tuning choice")
            ms = warm
            if warm < 3.0 * best:  # clearly slower candidates keep their warm-up time
                ms = min(run() for _ in range(self.repeats))
            times[name] = ms
            # the first candidate is the library's default launch; another replaces it only when it is
            # clearly faster on the sample (a sample is tail-bound, so small differences do not carry over
            # to the whole batch)
            if first[0] == name or ms < best * (1.0 - self.margin):
                best, choice = ms, {"engine": eng, "warps_per_sm": wps, "name": name}
        return {"choice": choice, "ms": times, "sample_queries": k, "batch_queries": n, "when": time.time(),
                "margin": self.margin}


class GraphSolve:
    """A batched solve captured once as a CUDA graph for fixed device buffers
    (queries, optional order, results, contacts) and replayed on whatever
    those buffers hold.  The first, uncaptured call sizes the library's
    scratch so the captured launches allocate nothing.  An optional prologue
    (a callable issuing device work on the current stream, such as the
    network that writes the order) is captured ahead of the solve.  The object keeps the
    buffers alive for as long as the graph can be replayed; the context's
    models must not change between replays (the graph holds the model table's
    address)."""

    def __init__(self, ctx, d_queries, n: int, params: dict, d_results, d_contacts, contacts_per_query: int,
                 d_order=None, stream=None, prologue=None):
        torch = _torch()
        self.ctx, self.n = ctx, n
        self._buffers = (d_queries, d_results, d_contacts, d_order)
        self.stream = stream or torch.cuda.Stream()
        ptrs = (d_queries.data_ptr(), d_results.data_ptr(), d_contacts.data_ptr() if d_contacts is not None else None)

        def call(stream_handle):
            if prologue is not None:  # device work that prepares the buffers (e.g. the order), on the same stream
                with torch.cuda.stream(self.stream):
                    prologue()
            if d_order is None:
                ctx.solve_device(ptrs[0], n, params, ptrs[1], ptrs[2], contacts_per_query, stream=stream_handle)
            else:
                ctx.solve_ordered(ptrs[0], n, params, d_order.data_ptr(), ptrs[1], ptrs[2], contacts_per_query,
                                  stream=stream_handle)

        call(self.stream.cuda_stream)
        self.stream.synchronize()
        before = ctx.launches()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream, capture_error_mode="thread_local"):
            call(self.stream.cuda_stream)
        self.kernels = ctx.launches() - before  # kernel launches per replay

    def replay(self):
        """Re-runs the captured launches on the graph's stream (asynchronous:
        synchronize self.stream, or make another stream wait on it)."""
        torch = _torch()
        with torch.cuda.stream(self.stream):
            self.graph.replay()
