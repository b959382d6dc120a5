"""Replicated query batches over two processes (gloo, CPU): each rank solves
its shard with the oracle port, the gathered results equal one process's."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from c2a_gb300.dist import shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port_no, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port_no))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from c2a_gb300 import workloads
    from oracle.oracle import Port

    wl = workloads.small_knots(37, seed=9, device="cpu")
    port = Port()
    sl = shard(wl.n, rank, world)
    res, _ = port.solve_batch(port.models(wl.meshes), wl.qint[sl], wl.poses[sl], wl.params, contacts_per_query=0)
    t = torch.from_numpy(np.stack([res["toc"], res["numCA"].astype(np.float64), res["collisionfree"].astype(np.float64)], 1))
    sizes = [shard(wl.n, r, world).stop - shard(wl.n, r, world).start for r in range(world)]
    gathered = [torch.zeros((s, 3), dtype=torch.float64) for s in sizes]
    dist.all_gather(gathered, t) if len(set(sizes)) == 1 else _gather_ragged(gathered, t)
    elapsed = torch.tensor([float(rank + 1)])
    dist.all_reduce(elapsed, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((torch.cat(gathered).numpy(), float(elapsed)))
    dist.barrier()
    dist.destroy_process_group()


def _gather_ragged(gathered, t):
    # pad to the largest shard, gather, trim
    m = max(g.shape[0] for g in gathered)
    pad = torch.zeros((m, 3), dtype=torch.float64)
    pad[: t.shape[0]] = t
    bufs = [torch.zeros((m, 3), dtype=torch.float64) for _ in gathered]
    dist.all_gather(bufs, pad)
    for g, b in zip(gathered, bufs):
        g.copy_(b[: g.shape[0]])


def test_shard_covers_every_query_once():
    for n in (0, 1, 7, 64, 65537):
        for w in (1, 2, 3, 8):
            idx = np.concatenate([np.arange(n)[shard(n, r, w)] for r in range(w)])
            assert np.array_equal(idx, np.arange(n))


def test_two_rank_replicas_match_single_process(port):
    from c2a_gb300 import workloads

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p_no = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, p_no, q)) for r in range(2)]
    for p in procs:
        p.start()
    got, elapsed = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    wl = workloads.small_knots(37, seed=9, device="cpu")
    res, _ = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, wl.params, contacts_per_query=0)
    exp = np.stack([res["toc"], res["numCA"].astype(np.float64), res["collisionfree"].astype(np.float64)], 1)
    assert got.tobytes() == exp.tobytes()
    assert elapsed == 2.0  # the max over ranks
