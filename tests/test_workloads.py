"""The uneven (config 3) and near-contact (config 4) workloads: generator
properties on the CPU, and the CUDA path against the oracle port on small
seeded instances of both (bit for bit, both modes and every engine), plus
the near-contact checks: no query ends later than the reference, and the
exact distance at every returned time of contact is within th_ca."""
import numpy as np
import pytest

from c2a_testutil import RESULT_FIELDS, describe, result_mismatches
from c2a_gb300 import meshes, workloads


def small_config3(n=96, seed=3):
    return workloads.config3(n=n, seed=seed, pool=6, tri_range=(1000, 4000), device="cpu")


def port_distance_fn(port, mesh):
    """An exact distance query through the oracle port (C2A_Distance, rel = abs = 0),
    with the closest points from the port's TriDist of the closest pair."""
    models = port.models([mesh])
    tv = mesh.tri_verts().reshape(-1, 3, 3)

    def fn(qint, poses):
        n = len(qint)
        d = np.zeros(n)
        p1 = np.zeros((n, 3))
        p2 = np.zeros((n, 3))
        for i in range(n):
            R = poses[i, 24:33].reshape(3, 3)
            T = poses[i, 33:36]
            d[i], ta, tb = port.distance(models, 0, 0, R, T, int(qint[i, 2]), int(qint[i, 3]))
            _, P, Q, _ = port.tridist(tv[ta], tv[tb] @ R.T + T)
            p1[i] = P
            p2[i] = R.T @ (Q - T)
        return d, p1, p2

    return fn


def test_config3_pool_and_queries():
    wl = small_config3()
    assert len(wl.meshes) == 6
    kinds = [m.name.rstrip("0123456789_x") for m in wl.meshes]
    assert kinds[0].startswith("torusknot") and kinds[1].startswith("icosphere") and kinds[2].startswith("soup")
    for m in wl.meshes:
        assert 1000 * 0.6 <= m.num_tris <= 4000 * 1.7, (m.name, m.num_tris)  # knots/icospheres round their counts
    assert wl.qint[:, :2].min() >= 0 and wl.qint[:, :2].max() < 6
    assert len(np.unique(wl.qint[:, 0] * 6 + wl.qint[:, 1])) > 10  # many model combinations in one batch
    v = np.linalg.norm(wl.poses[:, 45:48] - wl.poses[:, 33:36], axis=1)
    diag = np.array([wl.meshes[a].bbox_diag() for a in wl.qint[:, 0]])
    assert (v >= 0.01 * diag * (1 - 1e-9)).all() and (v <= 5 * diag * (1 + 1e-9)).all()
    assert np.ptp(np.log(v / diag)) > 4.0  # log-uniform over most of [0.01, 5]
    again = small_config3()
    assert (again.qint == wl.qint).all() and (again.poses == wl.poses).all()


def test_config3_oracle_runs(port):
    wl = small_config3()
    res, _ = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, wl.params, threads=8)
    assert (res["numCA"] >= 1).all()
    assert 0.05 < np.mean(res["collisionfree"] == 0) < 0.6


def test_near_contact_placement_with_port(port):
    knot = meshes.torus_knot(2, 3, 24, 6)
    fn = port_distance_fn(port, knot)
    qint, poses, d = workloads.near_contact_queries(knot, 12, 44, fn, device="cpu")
    diag = knot.bbox_diag()
    rng = np.random.default_rng(44)
    rng.standard_normal((12, 4)); rng.standard_normal((12, 3))  # R0b, u (same draws as the generator)
    gap = np.exp(rng.uniform(np.log(1e-6), np.log(1e-3), 12)) * diag
    assert (d > 0).all()
    assert np.allclose(d, gap, rtol=1e-6), np.c_[d, gap]
    # grazing: within 5 degrees of the tangent plane at the closest points
    dd, p1, p2 = fn(qint, poses)
    R = poses[:, 24:33].reshape(-1, 3, 3)
    nrm = np.einsum("nij,nj->ni", R, p2) + poses[:, 33:36] - p1
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    v = poses[:, 45:48] - poses[:, 33:36]
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    assert (np.abs(np.sum(v * nrm, axis=1)) <= np.sin(np.deg2rad(5.0)) + 1e-9).all()


_GPU_IDS = {}


def gpu_vs_port(ctx, port, wl, mode=0, engine=0):
    from c2a_gb300 import api

    key = (id(ctx), id(wl))
    if key not in _GPU_IDS:  # each workload's models built once per context
        _GPU_IDS[key] = np.array([ctx.model(m) for m in wl.meshes])
    ids = _GPU_IDS[key]
    q = wl.qint.copy()
    q[:, 0] = ids[wl.qint[:, 0]]
    q[:, 1] = ids[wl.qint[:, 1]]
    prm = dict(wl.params, mode=mode, engine=engine)
    res, con = ctx.solve(q, wl.poses, prm, contacts_per_query=256, check=False)
    exp, econ = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, prm, threads=8,
                                 contacts_per_query=256)
    ok = (res["status"] & ~(api.QUERY_ITER_CAP | api.QUERY_CONTACT_OVERFLOW)) == 0
    assert ok.all(), np.unique(res["status"])
    fields = RESULT_FIELDS if mode == 0 else [f for f in RESULT_FIELDS if f not in ("seed_a", "seed_b")]
    flat = np.concatenate([econ[k][:min(256, exp[k]["num_contact"])] for k in range(wl.n)])
    offs = np.concatenate([[0], np.cumsum(np.minimum(256, exp["num_contact"]))])
    bad = result_mismatches(res, exp, con, flat, offs, fields=fields)
    if mode == 1:
        # CANONICAL: with more contacts than slots, which ones fill the slots is
        # unspecified (their count and the overflow status are exact)
        over = [k for k in bad if exp[k]["num_contact"] > 256]
        assert not result_mismatches(res[over], exp[over], fields=fields)
        assert all(res[k]["status"] & api.QUERY_CONTACT_OVERFLOW for k in over)
        bad = [k for k in bad if k not in over]
    assert not bad, f"{len(bad)} of {wl.n} differ; first " + describe(res, exp, bad[0])
    return res, q


@pytest.mark.gpu
@pytest.mark.parametrize("mode,engine", [(0, 1), (0, 3), (1, 1), (1, 2)])
def test_gpu_config3_matches_port(gpu_ctx, port, mode, engine):
    gpu_vs_port(gpu_ctx, port, small_config3(n=128, seed=33), mode, engine)


@pytest.fixture(scope="module")
def config3_full():
    """Config 3 as specified: 4,096 pairs from a pool of 12 meshes, 1k-200k triangles log-uniform."""
    return workloads.config3(n=4096, seed=3, device="cpu")


@pytest.fixture(scope="module")
def config3_top():
    """The top of config 3's range: six meshes of 100k-200k triangles (knots and
    clustered soups; icospheres stop at 81,920), 2,048 pairs."""
    return workloads.config3(n=2048, seed=21, pool=6, tri_range=(100000, 200000), device="cpu")


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["full", "top"])
@pytest.mark.parametrize("mode,engine", [(0, 1), (0, 3), (0, 4), (1, 1), (1, 2)])
def test_gpu_config3_full_size_matches_port(gpu_ctx, port, request, which, mode, engine):
    """Every query of the full-size uneven batches, REFERENCE (warp, thread,
    speculative engines) and CANONICAL (warp, batched), bit for bit against
    the oracle; no query may overflow a stack or be rejected."""
    wl = request.getfixturevalue(f"config3_{which}")
    tris = sorted(m.num_tris for m in wl.meshes)
    if which == "top":
        assert tris[-1] >= 190000 and sum(t >= 150000 for t in tris) >= 2
    else:
        assert tris[0] < 2000 and len(tris) == 12
    gpu_vs_port(gpu_ctx, port, wl, mode, engine)


@pytest.mark.gpu
def test_gpu_config4_near_contact(gpu_ctx, port):
    knot = meshes.torus_knot(2, 3, 100, 16, 1.0, 0.15)
    mid = gpu_ctx.model(knot)
    qn, pn, d0 = workloads.near_contact_queries(knot, 96, 45, workloads.gpu_distance_fn(gpu_ctx, mid))
    diag = knot.bbox_diag()
    assert (d0 > 0).all() and (d0 >= 0.9e-6 * diag).all() and (d0 <= 1.1e-3 * diag).all()
    wl = workloads.Workload("near", [knot], qn, pn, workloads.default_params(diag, 1e-4, 64))
    res, q = gpu_vs_port(gpu_ctx, port, wl, 0, 1)
    # bit-exact with the reference, so never later than it; and where the CA
    # loop reached tolerance_d, the exact distance at the returned time of
    # contact is within th_ca.  (A query whose first step is already within
    # tolerance_d gets toc = that step's mint, a time the reference never
    # measured, C2A/src/C2A.cpp:2053-2092; it is kept bit for bit and left out
    # of this check.)
    hit = (res["collisionfree"] == 0) & (res["distance"] <= wl.params["tol_d"]) & (res["numCA"] >= 2) & \
          (res["distance"] > 0)
    P = np.zeros((int(hit.sum()), workloads.POSE_WIDTH))
    P[:, 0:9] = res["R_toc"][hit, 0]
    P[:, 9:12] = res["T_toc"][hit, 0]
    P[:, 24:33] = res["R_toc"][hit, 1]
    P[:, 33:36] = res["T_toc"][hit, 1]
    dq = q[hit].copy()
    dq[:, 2] = res["seed_a"][hit]
    dq[:, 3] = res["seed_b"][hit]
    exact = gpu_ctx.distance(dq, P)["distance"]
    assert hit.sum() > 10
    assert (exact >= 0).all() and (exact <= wl.params["th_ca"] * (1 + 1e-12)).all(), exact.max()
