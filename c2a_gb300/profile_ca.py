"""A small, self-contained run of the CA kernel for profiler captures.

    python -m c2a_gb300.profile_ca [--queries N] [--launches K] [--pick I[,J...]] [--mode canonical]

Builds the config-2 model (two 40,000-triangle (2,3) torus knots), places the
first N of the config-2 queries, then launches the solve kernel K times on
device-resident buffers and prints the mean kernel time (CUDA events).  Small
N keeps an ncu --set full capture to a few seconds per pass; --pick runs only
the listed queries (indices into the first N), e.g. one query alone to see a
single traversal's instruction mix and stalls.
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--queries", type=int, default=2048)
    ap.add_argument("--launches", type=int, default=2)
    ap.add_argument("--slots", type=int, default=64)
    ap.add_argument("--pick", type=str, default="")
    ap.add_argument("--mode", choices=["reference", "canonical"], default="reference")
    ap.add_argument("--engine", choices=["auto", "warp", "batched", "thread"], default="auto")
    args = ap.parse_args()

    import torch

    from . import api, build, workloads

    build.build()
    wl = workloads.config2(n=65536, seed=2, device="cuda", subset=args.queries)
    if args.pick:
        wl = wl.subset(np.array([int(i) for i in args.pick.split(",")]))
    if args.mode == "canonical":
        wl.params["mode"] = api.MODE_CANONICAL
    wl.params["engine"] = {"auto": api.ENGINE_AUTO, "warp": api.ENGINE_WARP, "batched": api.ENGINE_BATCHED,
                           "thread": api.ENGINE_THREAD}[args.engine]
    ctx = api.Context(0)
    mid = ctx.model(wl.meshes[0])
    q = wl.qint.copy()
    q[:, :2] = mid
    qs = api.make_queries(q, wl.poses)
    d_q = torch.from_numpy(qs.view(np.uint8).copy()).cuda()
    d_r = torch.zeros(wl.n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(wl.n * args.slots * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    times = []
    for _ in range(args.launches):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        ctx.solve_device(d_q.data_ptr(), wl.n, wl.params, d_r.data_ptr(), d_c.data_ptr(), args.slots,
                         stream=s.cuda_stream)
        b.record(s)
        s.synchronize()
        times.append(a.elapsed_time(b))
    res = d_r.cpu().numpy().view(api.RESULT_DTYPE)
    print(json.dumps({"queries": wl.n, "mode": args.mode, "kernel_ms": times, "num_bv_tests": int(res["num_bv_tests"].sum()),
                      "num_tri_tests": int(res["num_tri_tests"].sum()),
                      "colliding": float(1 - res["collisionfree"].mean())}))


if __name__ == "__main__":
    main()
