"""The distance query: C2A_Distance with rel_err = abs_err = 0 (the exact
minimum TriDist over all triangle pairs), C2A/src/C2A_PQP.cpp:970-1056.

The oracle port is pinned against the reference's own C2A_Distance (golden
fixture from tests/golden/make_golden.py); the CUDA batch query
(c2a_distance_batch) is checked against both.  The distance is compared bit
for bit.  Among exactly tied closest pairs (touching or overlapping models
have many) the reference keeps the first pair its depth-first order meets and
the kernel the smallest pair; a differing pair is accepted only when the
reference's own query, seeded with the kernel's pair, keeps it, i.e. when it
is at exactly the minimum distance.
"""
import os

import numpy as np
import pytest

from c2a_testutil import GOLDEN, bits
from c2a_gb300 import meshes, workloads


def load_distance_fixture():
    z = np.load(os.path.join(GOLDEN, "distance_ref.npz"))
    ms = [meshes.Mesh(f"d{i}", z[f"mesh{i}_verts"], z[f"mesh{i}_faces"], np.zeros((1, 3)), 0.0)
          for i in range(int(z["num_meshes"]))]
    return ms, z["qint"], z["R"], z["T"], z["distance"], z["tri_a"], z["tri_b"]


def poses_of(R, T):
    """A at the identity, B at (R, T); the end poses repeat the start (unused)."""
    n = len(R)
    P = np.zeros((n, workloads.POSE_WIDTH))
    eye = np.eye(3).reshape(9)
    P[:, 0:9] = eye
    P[:, 12:21] = eye
    P[:, 24:33] = R
    P[:, 33:36] = T
    P[:, 36:45] = R
    P[:, 45:48] = T
    return P


def test_port_distance_matches_reference_fixture(port):
    ms, qint, R, T, dist, ta, tb = load_distance_fixture()
    models = port.models(ms)
    for i, (a, b, sa, sb) in enumerate(qint):
        d, pa, pb = port.distance(models, a, b, R[i], T[i], sa, sb)
        assert bits(d) == bits(dist[i]) and (pa, pb) == (ta[i], tb[i]), i


def check_against(port, models, res, qint, R, T, dist, ta=None, tb=None):
    ties = 0
    for i, (a, b, sa, sb) in enumerate(qint):
        r = res[i]
        assert r["status"] == 0, i
        assert bits(r["distance"]) == bits(dist[i]), (i, r["distance"], dist[i])
        if ta is not None and (r["tri_a"], r["tri_b"]) == (ta[i], tb[i]):
            continue
        # a different pair: the reference's order, seeded with it, must keep it
        d, pa, pb = port.distance(models, a, b, R[i], T[i], r["tri_a"], r["tri_b"])
        assert bits(d) == bits(dist[i]) and (pa, pb) == (r["tri_a"], r["tri_b"]), (i, d, pa, pb)
        ties += 1
    return ties


def points_consistent(res, R, T):
    """|p1 - (R p2 + T)| is the distance (the points are the closest pair's);
    overlapping pairs (distance 0) are left out: there TriDist's points are
    those of the last segment pair it tried, not a common point."""
    q = np.einsum("nij,nj->ni", R.reshape(-1, 3, 3), res["p2"]) + T
    gap = np.linalg.norm(res["p1"] - q, axis=1)
    pos = res["distance"] > 0
    return pos.sum() > 10 and np.allclose(gap[pos], res["distance"][pos], rtol=1e-9, atol=1e-12)


@pytest.mark.gpu
def test_gpu_distance_matches_reference_fixture(gpu_ctx, port):
    ms, qint, R, T, dist, ta, tb = load_distance_fixture()
    ids = [gpu_ctx.model(m) for m in ms]
    q = qint.copy()
    q[:, 0] = np.array(ids)[qint[:, 0]]
    q[:, 1] = np.array(ids)[qint[:, 1]]
    res = gpu_ctx.distance(q, poses_of(R, T))
    # every differing pair is checked to be an exact tie (a closest vertex or
    # edge is shared by several triangles, so ties are common)
    check_against(port, port.models(ms), res, qint, R, T, dist, ta, tb)
    assert points_consistent(res, R, T)


@pytest.mark.gpu
def test_gpu_distance_matches_port_random(gpu_ctx, port):
    rng = np.random.default_rng(41)
    ms = [meshes.torus_knot(3, 5, 60, 10, 1.0, 0.12), meshes.triangle_soup(3000, clusters=10, seed=42),
          meshes.icosphere(4, radius=1.1, noise=0.02, seed=43)]
    n = 96
    rows, Rs, Ts = [], [], []
    for k in range(n):
        a, b = rng.integers(0, 3, 2)
        rows.append([a, b, rng.integers(ms[a].num_tris), rng.integers(ms[b].num_tris)])
    qint = np.array(rows, dtype=np.int32)
    R = workloads.random_rotations(rng, n).reshape(n, 9)
    T = workloads.unit_vectors(rng, n) * rng.uniform(0.8, 4.0, (n, 1)) + rng.normal(scale=1e-3, size=(n, 3))
    models = port.models(ms)
    dist = np.array([port.distance(models, a, b, R[i], T[i], sa, sb)[0] for i, (a, b, sa, sb) in enumerate(qint)])
    ids = np.array([gpu_ctx.model(m) for m in ms])
    q = qint.copy()
    q[:, 0] = ids[qint[:, 0]]
    q[:, 1] = ids[qint[:, 1]]
    res = gpu_ctx.distance(q, poses_of(R, T))
    check_against(port, models, res, qint, R, T, dist)
    assert points_consistent(res, R, T)


@pytest.mark.gpu
def test_gpu_distance_bad_input(gpu_ctx):
    knot = meshes.torus_knot(2, 3, 24, 6)
    mid = gpu_ctx.model(knot)
    qint = np.array([[mid, mid, 0, knot.num_tris], [mid, 999, 0, 0]], dtype=np.int32)
    R = np.tile(np.eye(3).reshape(1, 9), (2, 1))
    T = np.array([[3.0, 0.5, 0.25]] * 2)
    res = gpu_ctx.distance(qint, poses_of(R, T), check=False)
    assert (res["status"] == 1).all()
