"""The learned seeding: the network kernels (c2a_gb300/csrc/mlp.cu) against the
CPU oracle (oracle/mlp_ref.py), the oracle's backward against finite
differences, the cluster tables and features, training on labels the
library produces, and the hinted CANONICAL solve, whose results must equal
the plain solve's bit for bit (the hints only tighten a search bound)."""
import numpy as np
import pytest

from c2a_testutil import RESULT_FIELDS, bits
from c2a_gb300 import api, learned, meshes, workloads
from oracle import mlp_ref


def tiny_params(rng, nin=64, h=8, out=12, pool=3):
    W = [rng.normal(0, 0.4, (h, nin)), rng.normal(0, 0.4, (h, h)), rng.normal(0, 0.4, (h, h)),
         rng.normal(0, 0.4, (out, h))]
    W[0][:, 50:] = 0.0
    b = [rng.normal(0, 0.1, h), rng.normal(0, 0.1, h), rng.normal(0, 0.1, h), rng.normal(0, 0.1, out)]
    E = rng.normal(0, 0.5, (pool, 16))
    return W, b, E


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(5)
    W, b, E = tiny_params(rng)
    n = 6
    feat = rng.normal(size=(n, 18))
    ia, ib = rng.integers(0, 3, n), rng.integers(0, 3, n)
    lab = rng.integers(0, 12, n)
    _, _, g = mlp_ref.forward_backward(W, b, E, feat, ia, ib, lab, rounding=False)

    def loss_at(W2, b2, E2):
        return mlp_ref.forward_backward(W2, b2, E2, feat, ia, ib, lab, rounding=False)[0]

    h = 1e-6
    for li in range(4):
        for (r, c) in [(0, 0), (1, 3), (W[li].shape[0] - 1, min(7, W[li].shape[1] - 1))]:
            Wp = [w.copy() for w in W]
            Wm = [w.copy() for w in W]
            Wp[li][r, c] += h
            Wm[li][r, c] -= h
            fd = (loss_at(Wp, b, E) - loss_at(Wm, b, E)) / (2 * h)
            assert abs(fd - g["W"][li][r, c]) < 1e-7 + 1e-5 * abs(fd), (li, r, c)
        bp = [v.copy() for v in b]
        bm = [v.copy() for v in b]
        bp[li][1] += h
        bm[li][1] -= h
        fd = (loss_at(W, bp, E) - loss_at(W, bm, E)) / (2 * h)
        assert abs(fd - g["b"][li][1]) < 1e-7 + 1e-5 * abs(fd)
    for (r, c) in [(0, 0), (2, 15)]:
        Ep, Em = E.copy(), E.copy()
        Ep[r, c] += h
        Em[r, c] -= h
        fd = (loss_at(W, b, Ep) - loss_at(W, b, Em)) / (2 * h)
        assert abs(fd - g["E"][r, c]) < 1e-7 + 1e-5 * abs(fd)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e-3], dtype=np.float32)
    r = mlp_ref.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5  # ties to even
    assert abs(r[4] - 3.0e-3) < 3.0e-3 * 2 ** -8


def test_cluster_tables_cover_every_triangle():
    knot = meshes.torus_knot(2, 3, 40, 8)
    with api.Context(-1) as ctx:
        mid = ctx.model(knot)
        nt, nn, _ = ctx.model_info(mid)
        _, fc, _, _, _ = ctx.download(mid)
        t = learned.cluster_table(fc, nt)
    assert 32 < t.count <= 64 and (t.of_tri >= 0).all() and t.of_tri.max() == t.count - 1
    for c in range(t.count):  # the hint's path leads to the node holding exactly the cluster's triangles
        node, path, depth = 0, int(t.hint[c]) & 0xFFFF, int(t.hint[c]) >> 16
        for k in range(depth):
            node = int(fc[node]) + ((path >> k) & 1)
        tris, stack = [], [node]
        while stack:
            x = stack.pop()
            if fc[x] < 0:
                tris.append(-int(fc[x]) - 1)
            else:
                stack += [int(fc[x]), int(fc[x]) + 1]
        assert sorted(tris) == sorted(np.nonzero(t.of_tri == c)[0].tolist())


def test_features_of_known_motion():
    P = np.zeros((1, 48))
    eye = np.eye(3).reshape(9)
    P[0, 0:9] = P[0, 12:21] = eye
    Rz = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1.0]])
    P[0, 24:33] = eye
    P[0, 33:36] = [2.0, 0, 0]
    P[0, 36:45] = Rz.reshape(9)
    P[0, 45:48] = [1.0, 1.0, 0]
    f = learned.features(P, np.array([2.0]), np.array([2.0]))[0]
    assert np.allclose(f[:9], eye) and np.allclose(f[9:12], [1, 0, 0]) and np.allclose(f[12:15], [-0.5, 0.5, 0])
    assert np.allclose(f[15:18], [0, 0, np.pi / 2])


# ------------------------------------------------------------------- GPU


def to_bf16_np(a):
    return mlp_ref.bf16(a)


def test_checkpoint_round_trip(lib, tmp_path):
    """SeedNet and CostOrder checkpoints restore every weight, embedding,
    Adam moment and the step, and re-derive the BF16 copies the GEMMs read."""
    import torch

    rng = np.random.default_rng(9)
    net = learned.SeedNet(5, seed=1, device="cpu")
    for group in (net.params, net.m, net.v):
        for t in group:
            t.copy_(torch.from_numpy(rng.normal(size=tuple(t.shape)).astype(np.float32)))
    net.t = 17
    net.save(str(tmp_path / "net.npz"))
    back = learned.SeedNet.load(str(tmp_path / "net.npz"), device="cpu")
    assert back.t == 17 and back.E.shape == (5, learned.EMBED)
    for a, b in zip(net.params + net.m + net.v, back.params + back.m + back.v):
        assert torch.equal(a, b)
    for i, w in enumerate(net.W):
        assert torch.equal(back.Wb[i], w.to(torch.bfloat16))
        assert torch.equal(back.WbT[i], w.t().contiguous().to(torch.bfloat16))
    with pytest.raises(ValueError):
        learned.SeedNet(4, device="cpu").load_state(net.state())  # another mesh count

    co = learned.CostOrder(2, seed=3, device="cpu")
    co.top = 6.25
    co.save(str(tmp_path / "cost.npz"))
    co2 = learned.CostOrder.load(str(tmp_path / "cost.npz"), device="cpu")
    assert co2.top == 6.25
    assert all(torch.equal(a, b) for a, b in zip(co.net.params, co2.net.params))


@pytest.mark.gpu
def test_gpu_gemm_matches_numpy(gpu_ctx):
    import torch

    net = learned.SeedNet(3)
    rng = np.random.default_rng(8)
    A = to_bf16_np(rng.normal(size=(256, 96)).astype(np.float32))
    B = to_bf16_np(rng.normal(scale=96 ** -0.5, size=(384, 96)).astype(np.float32))  # pre-activations ~ N(0, 2)
    bias = rng.normal(size=384).astype(np.float32)
    At = torch.tensor(A, device="cuda").to(torch.bfloat16)
    Bt = torch.tensor(B, device="cuda").to(torch.bfloat16)
    bt = torch.tensor(bias, device="cuda")
    of = torch.empty((256, 384), dtype=torch.float32, device="cuda")
    ob = torch.empty((256, 384), dtype=torch.bfloat16, device="cuda")
    net.gemm(At, Bt, bt, learned.BIAS | learned.GELU, of, ob)
    torch.cuda.synchronize()
    exact = A.astype(np.float64) @ B.astype(np.float64).T + bias
    got = of.cpu().numpy()
    assert np.max(np.abs(got - exact) / (np.abs(A) @ np.abs(B).T + 1)) < 3e-5
    # GELU in the kernel's FP32 arithmetic (erff taken as correctly rounded), then bf16
    from scipy.special import erf

    t = (got * np.float32(0.70710678118654752)).astype(np.float32)
    one = (np.float32(1.0) + erf(t.astype(np.float64)).astype(np.float32)).astype(np.float32)
    g = mlp_ref.bf16(((np.float32(0.5) * got).astype(np.float32) * one).astype(np.float32))
    gb = ob.float().cpu().numpy()
    assert np.mean(gb == g) > 0.99 and np.allclose(gb, g, rtol=2 ** -7, atol=1e-6)


@pytest.mark.gpu
def test_gpu_network_gradients_match_oracle(gpu_ctx):
    import torch

    rng = np.random.default_rng(9)
    net = learned.SeedNet(5, seed=3)
    M = 256
    feat = rng.normal(size=(M, 18)).astype(np.float32)
    ia, ib = rng.integers(0, 5, M).astype(np.int32), rng.integers(0, 5, M).astype(np.int32)
    lab = rng.integers(0, learned.OUT, M).astype(np.int32)
    Ft, At, Bt, Yt = (torch.tensor(v, device="cuda") for v in (feat, ia, ib, lab))
    x = net.assemble(Ft, At, Bt, M)
    logits = net.forward(x)
    net.backward(logits, Yt, At, Bt, M)
    torch.cuda.synchronize()
    P = [p.cpu().numpy() for p in net.params]
    loss, lref, g = mlp_ref.forward_backward(P[0:4], P[4:8], P[8], feat, ia, ib, lab)

    def close(a, b):
        a, b = np.ravel(a).astype(np.float64), np.ravel(b).astype(np.float64)
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        return rel < 3e-2 and cos > 0.999, (rel, cos)

    ok, info = close(logits.cpu().numpy(), lref)
    assert ok, info
    for i in range(4):
        ok, info = close(net.g[i].cpu().numpy(), g["W"][i])
        assert ok, (i, info)
        ok, info = close(net.g[4 + i].cpu().numpy(), g["b"][i])
        assert ok, (i, info)
    ok, info = close(net.g[8].cpu().numpy(), g["E"])
    assert ok, info


def small_pool_workload(n, seed):
    return workloads.config3(n=n, seed=seed, pool=6, tri_range=(1000, 4000))


@pytest.mark.gpu
def test_gpu_training_learns_closest_cluster_pairs(gpu_ctx):
    wl = small_pool_workload(8192, 51)
    ids = np.array(gpu_ctx.models(wl.meshes))
    q = wl.qint.copy()
    q[:, 0], q[:, 1] = ids[wl.qint[:, 0]], ids[wl.qint[:, 1]]
    tables = {int(m): t for m, t in zip(ids, learned.cluster_tables(gpu_ctx, ids))}
    tab = [tables.get(i) for i in range(int(ids.max()) + 1)]
    lab = learned.labels(gpu_ctx, q, wl.poses, tab)
    diag = np.array([m.bbox_diag() for m in wl.meshes])
    feat = learned.features(wl.poses, diag[wl.qint[:, 0]], diag[wl.qint[:, 1]])
    net = learned.SeedNet(len(wl.meshes), seed=1)
    hist = net.train(feat, wl.qint[:, 0], wl.qint[:, 1], lab, epochs=25, batch=512)
    assert hist[-1] < 0.7 * hist[0], hist
    top = net.topk(feat, wl.qint[:, 0], wl.qint[:, 1], 8)
    hit8 = np.mean([lab[i] in top[i] for i in range(len(lab))])
    assert hit8 > 0.3, hit8  # far above chance (8 / 4096)


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [1, 2])
def test_gpu_hinted_solve_equals_plain(gpu_ctx, engine):
    wl = small_pool_workload(256, 52)
    ids = np.array(gpu_ctx.models(wl.meshes))
    q = wl.qint.copy()
    q[:, 0], q[:, 1] = ids[wl.qint[:, 0]], ids[wl.qint[:, 1]]
    tables = {int(m): t for m, t in zip(ids, learned.cluster_tables(gpu_ctx, ids))}
    tab = [tables.get(i) for i in range(int(ids.max()) + 1)]
    rng = np.random.default_rng(53)
    top = rng.integers(0, learned.OUT, (len(q), 8))
    lab = learned.labels(gpu_ctx, q, wl.poses, tab)
    top[: len(q) // 2, 0] = lab[: len(q) // 2]  # half of them hinted with the true pair
    hints = learned.hints_of(top, q, tab)
    prm = dict(wl.params, mode=1, engine=engine)
    plain, pc = gpu_ctx.solve(q, wl.poses, prm, contacts_per_query=128)
    hinted, hc = learned.solve_hinted(gpu_ctx, q, wl.poses, prm, hints, contacts_per_query=128)
    for f in RESULT_FIELDS:
        assert bits(plain[f]) == bits(hinted[f]), f
    for i in range(len(q)):
        n = min(int(plain[i]["num_contact"]), 128)
        a = pc[i][:n]
        b = hc[i * 128:i * 128 + n]
        for f in ("tri_a", "tri_b", "distance", "pa", "pb"):
            assert bits(a[f]) == bits(b[f]), (i, f)


@pytest.mark.gpu
def test_gpu_ordered_solve_equals_plain(gpu_ctx):
    import torch

    wl = workloads.small_knots(300, seed=61)
    mid = gpu_ctx.model(wl.meshes[0])
    q = wl.qint.copy()
    q[:, :2] = mid
    plain, pc = gpu_ctx.solve(q, wl.poses, wl.params, contacts_per_query=64)
    qs = api.make_queries(q, wl.poses)
    n = len(qs)
    d_q = torch.from_numpy(qs.view(np.uint8).copy()).cuda()
    for order in (np.random.default_rng(62).permutation(n), np.arange(n)[::-1].copy()):
        d_o = torch.tensor(order.astype(np.int32), device="cuda")
        d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        d_c = torch.zeros(n * 64 * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        gpu_ctx.solve_ordered(d_q.data_ptr(), n, wl.params, d_o.data_ptr(), d_r.data_ptr(), d_c.data_ptr(), 64)
        torch.cuda.synchronize()
        r = d_r.cpu().numpy().view(api.RESULT_DTYPE)
        c = d_c.cpu().numpy().view(api.CONTACT_DTYPE)
        for f in RESULT_FIELDS:
            assert bits(plain[f]) == bits(r[f]), f
        for i in range(n):
            m = min(int(plain[i]["num_contact"]), 64)
            for f in ("tri_a", "tri_b", "distance", "pa", "pb"):
                assert bits(pc[i][:m][f]) == bits(c[i * 64:i * 64 + m][f]), (i, f)
        # the host-buffer form: dense contacts as c2a_solve_batch returns them
        rh, ch = gpu_ctx.solve_ordered_host(q, wl.poses, wl.params, d_o.data_ptr(), contacts_per_query=64)
        for f in RESULT_FIELDS + ["contact_offset"]:
            assert bits(plain[f]) == bits(rh[f]), f
        for i in range(n):
            for f in ("tri_a", "tri_b", "distance", "pa", "pb"):
                assert bits(pc[i][f]) == bits(ch[i][f]), (i, f)
    # entries outside [0, n) are skipped, not read
    d_o = torch.tensor(np.r_[np.arange(n - 2), -1, n].astype(np.int32), device="cuda")
    d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    gpu_ctx.solve_ordered(d_q.data_ptr(), n, wl.params, d_o.data_ptr(), d_r.data_ptr(), None, 0)
    torch.cuda.synchronize()
    r = d_r.cpu().numpy().view(api.RESULT_DTYPE)
    assert bits(r["toc"][: n - 2]) == bits(plain["toc"][: n - 2]) and (r["numCA"][n - 2:] == 0).all()


@pytest.mark.gpu
def test_gpu_cost_order_learns(gpu_ctx):
    """The cost model's training and inference path on a cost that is a known
    function of two features (its predictive power on real CA costs is what
    bench.py measures on held-out queries)."""
    import torch

    rng = np.random.default_rng(63)
    n = 8192
    feat = rng.normal(size=(n, 18)).astype(np.float32)
    cost = np.exp(3.0 * feat[:, 12] + 2.0 * feat[:, 13] + 6.0)
    z = np.zeros(n, np.int32)
    model = learned.CostOrder(1, seed=2)
    hist = model.fit(feat[:6144], z[:6144], z[:6144], cost[:6144], epochs=40, batch=512)
    assert hist[-1] < 0.8 * hist[0], hist
    dev = lambda a: torch.tensor(a, device="cuda")
    e = model.expected(dev(feat[6144:]), dev(z[6144:]), dev(z[6144:])).cpu().numpy()
    r = np.corrcoef(np.argsort(np.argsort(e)), np.argsort(np.argsort(cost[6144:])))[0, 1]
    assert r > 0.8, r  # held-out rank correlation of predicted and true cost
    o = model.order(dev(feat), dev(z), dev(z)).cpu().numpy()
    assert sorted(o.tolist()) == list(range(n))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 1000, 70001])
def test_gpu_order_desc_is_a_stable_counting_sort(gpu_ctx, n):
    """c2a_mlp_order_desc against numpy: indices by decreasing quantised key,
    ties in increasing index; keys outside [0, key_max] and NaN clamp."""
    import torch

    rng = np.random.default_rng(64 + n)
    key = (rng.integers(0, 40, n) * 1.5 + rng.normal(scale=1e-4, size=n)).astype(np.float32)
    key[:: 97] = -3.0
    key[5:: 101] = 1e9
    if n > 7:
        key[7] = np.nan
    key_max = np.float32(63.0)
    t = np.clip(np.where(np.isnan(key), 0, key) / key_max, 0, 1).astype(np.float32)
    level = (t * np.float32(learned.ORDER_BINS - 1) + np.float32(0.5)).astype(np.int32)
    expect = np.argsort(-level, kind="stable")
    lib = learned.bind()
    d_k = torch.tensor(key, device="cuda")
    d_o = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    scratch = torch.empty(learned.order_scratch(n), dtype=torch.int32, device="cuda")
    assert lib.c2a_mlp_order_desc(d_k.data_ptr(), n, 63.0, d_o.data_ptr(), scratch.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_o.cpu().numpy(), expect)


@pytest.mark.gpu
@pytest.mark.parametrize("heavy", [1, 24, 5000])
def test_gpu_heavy_prefix_split_equals_plain(gpu_ctx, heavy):
    """An ordered batch whose head runs on SM sub-partitions of its own
    (c2a_params.heavy_prefix, the split warp kernel) gives the plain solve's
    results and contacts bit for bit."""
    import torch

    wl = workloads.small_knots(400, seed=65)
    mid = gpu_ctx.model(wl.meshes[0])
    q = wl.qint.copy()
    q[:, :2] = mid
    plain, pc = gpu_ctx.solve(q, wl.poses, wl.params, contacts_per_query=64)
    qs = api.make_queries(q, wl.poses)
    n = len(qs)
    d_q = torch.from_numpy(qs.view(np.uint8).copy()).cuda()
    cost = plain["num_bv_tests"].astype(np.float64)
    d_o = torch.tensor(np.argsort(-cost, kind="stable").astype(np.int32), device="cuda")
    d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(n * 64 * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    launches = gpu_ctx.launches()
    gpu_ctx.solve_ordered(d_q.data_ptr(), n, dict(wl.params, engine=api.ENGINE_WARP, heavy_prefix=heavy),
                          d_o.data_ptr(), d_r.data_ptr(), d_c.data_ptr(), 64)
    torch.cuda.synchronize()
    assert gpu_ctx.launches() - launches == 1
    r = d_r.cpu().numpy().view(api.RESULT_DTYPE)
    c = d_c.cpu().numpy().view(api.CONTACT_DTYPE)
    for f in RESULT_FIELDS:
        assert bits(plain[f]) == bits(r[f]), f
    for i in range(n):
        m = min(int(plain[i]["num_contact"]), 64)
        for f in ("tri_a", "tri_b", "distance", "pa", "pb"):
            assert bits(pc[i][:m][f]) == bits(c[i * 64:i * 64 + m][f]), (i, f)
