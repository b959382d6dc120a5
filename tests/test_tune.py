"""The launch autotuner and CUDA-graph replay (c2a_gb300/tune.py): the tuner
times every candidate launch on a sample of the batch and rejects any that
changes a result; a captured solve replays bit-identically, also after the
buffers are refilled with another batch of the same size."""
import json

import numpy as np
import pytest

from c2a_testutil import bits

pytestmark = pytest.mark.gpu


def _batch(ctx, n, seed, mode=0):
    import torch
    from c2a_gb300 import api, workloads

    wl = workloads.small_knots(n, seed=seed, device="cpu")
    mid = ctx.model(wl.meshes[0])
    q = wl.qint.copy()
    q[:, :2] = mid
    wl.params["mode"] = mode
    d_q = torch.from_numpy(api.make_queries(q, wl.poses).view(np.uint8).copy()).cuda()
    return wl, q, d_q


def _solve(ctx, d_q, n, params, slots=64, order=None):
    import torch
    from c2a_gb300 import api

    d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(n * slots * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    if order is None:
        ctx.solve_device(d_q.data_ptr(), n, params, d_r.data_ptr(), d_c.data_ptr(), slots)
    else:
        ctx.solve_ordered(d_q.data_ptr(), n, params, order.data_ptr(), d_r.data_ptr(), d_c.data_ptr(), slots)
    torch.cuda.synchronize()
    return d_r.cpu().numpy(), d_c.cpu().numpy()


@pytest.mark.parametrize("mode", [0, 1])
def test_tuner_picks_a_measured_launch_and_caches_it(gpu_ctx, tmp_path, mode):
    from c2a_gb300 import api, tune

    wl, q, d_q = _batch(gpu_ctx, 600, 71 + mode, mode)
    cache = str(tmp_path / "tune.json")
    t = tune.Tuner(gpu_ctx, cache=cache, sample=256, repeats=1)
    r = t.choose(d_q, wl.n, wl.params)
    rec = r["record"]
    names = [f"{tune.ENGINE_NAMES[e]}/{w or 'max'}" for e, w in t.candidates(wl.params) if not w]  # sample < batch
    assert sorted(rec["ms"]) == sorted(names) and not rec["cached"] and rec["sample_queries"] == 256
    exp, best = names[0], rec["ms"][names[0]]  # the default launch unless another is clearly faster
    for nm in names[1:]:
        if rec["ms"][nm] < best * (1 - rec["margin"]):
            exp, best = nm, rec["ms"][nm]
    assert rec["choice"]["name"] == exp
    assert r["params"]["engine"] == rec["choice"]["engine"]
    table = json.load(open(cache))
    assert list(table) == [rec["signature"]] and ("canonical" if mode else "reference") in rec["signature"]
    again = t.choose(d_q, wl.n, wl.params)
    assert again["record"]["cached"] and again["params"] == r["params"]
    # the tuned launch gives the default launch's results
    # a sample that is the whole batch also times the launch shapes
    whole = tune.Tuner(gpu_ctx, cache=None, sample=wl.n, repeats=1).measure(d_q, wl.n, wl.params)
    assert sorted(whole["ms"]) == sorted(f"{tune.ENGINE_NAMES[e]}/{w or 'max'}" for e, w in t.candidates(wl.params))
    ref = _solve(gpu_ctx, d_q, wl.n, wl.params)
    got = _solve(gpu_ctx, d_q, wl.n, r["params"])
    assert ref[0].tobytes() == got[0].tobytes() and ref[1].tobytes() == got[1].tobytes()
    assert (ref[0].view(api.RESULT_DTYPE)["numCA"] > 0).all()


@pytest.mark.parametrize("engine", ["warp", "thread", "spec", "ordered"])
def test_graph_replay_matches_direct_solves(gpu_ctx, engine):
    import torch
    from c2a_gb300 import api, tune

    n, slots = 384, 64
    wl, q, d_q = _batch(gpu_ctx, n, 81)
    _, _, d_q2 = _batch(gpu_ctx, n, 82)
    prm = dict(wl.params, engine={"warp": api.ENGINE_WARP, "thread": api.ENGINE_THREAD, "spec": api.ENGINE_SPEC,
                                  "ordered": api.ENGINE_WARP}[engine])
    order = torch.tensor(np.random.default_rng(83).permutation(n).astype(np.int32), device="cuda") \
        if engine == "ordered" else None
    d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(n * slots * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    live = d_q.clone()
    g = tune.GraphSolve(gpu_ctx, live, n, prm, d_r, d_c, slots, d_order=order)
    assert g.kernels >= 1
    for src in (d_q, d_q2, d_q):
        live.copy_(src)
        d_r.zero_()
        d_c.zero_()
        torch.cuda.synchronize()
        g.replay()
        g.stream.synchronize()
        exp = _solve(gpu_ctx, src, n, prm, slots, order)
        assert d_r.cpu().numpy().tobytes() == exp[0].tobytes()
        assert d_c.cpu().numpy().tobytes() == exp[1].tobytes()
    r = d_r.cpu().numpy().view(api.RESULT_DTYPE)
    assert (r["status"] & ~api.QUERY_CONTACT_OVERFLOW == 0).all() and bits(r["toc"]) != bits(np.zeros(n))


def test_graph_with_prologue_captures_the_order(gpu_ctx):
    """A prologue captured ahead of the solve (here: the order written on the
    device) is replayed with it."""
    import torch
    from c2a_gb300 import api, tune

    n, slots = 256, 64
    wl, q, d_q = _batch(gpu_ctx, n, 84)
    prm = dict(wl.params, engine=api.ENGINE_WARP)
    perm = torch.tensor(np.random.default_rng(85).permutation(n).astype(np.int32), device="cuda")
    d_order = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(n * slots * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    g = tune.GraphSolve(gpu_ctx, d_q, n, prm, d_r, d_c, slots, d_order=d_order,
                        prologue=lambda: d_order.copy_(torch.flip(perm, dims=[0])))
    d_order.zero_()
    d_r.zero_()
    torch.cuda.synchronize()
    g.replay()
    g.stream.synchronize()
    assert torch.equal(d_order, torch.flip(perm, dims=[0]))
    exp = _solve(gpu_ctx, d_q, n, prm, slots)
    assert d_r.cpu().numpy().tobytes() == exp[0].tobytes()
