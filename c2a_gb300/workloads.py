"""Seeded CCD query workloads (the benchmark configurations, synthetic).

A workload is a list of meshes plus, per query, the two model indices, the
two seed triangles (C2A's initial upper-bound pair, ``dres.last_triA/B``) and
the four poses of C2A_Solve: begin/end of object A, begin/end of object B
(C2A/C2A.h:23-35).  Object A stays at the identity; object B starts at a
random orientation with a surface gap of ``s * diag``, translates towards A
inside a cone and rotates about a uniform axis: R1 = R0 * Rot(axis, |w|), so
the reference's body-frame axis/angle recovers exactly that rotation
(C2A/src/InterpMotion.cpp:228-270).

The reference measures nothing, so these stand in for its scenes: the shapes,
sizes and value ranges follow the benchmark configurations; the numbers are
drawn from numpy's PCG64 with a fixed seed.

Pose rows are 48 float64: R0a(9) T0a(3) R1a(9) T1a(3) R0b(9) T0b(3) R1b(9) T1b(3),
matrices row-major.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .meshes import Mesh, torus_knot, icosphere, triangle_soup

POSE_WIDTH = 48
# half-angle of the approach cone; tuned once with the oracle (400 queries on the
# 3,200-triangle knot at th_ca = 1e-4 diag: 29% colliding)
# so that about 30% of config-2 queries collide within t in [0, 1]
CONFIG2_CONE_DEG = 70.0


@dataclass
class Workload:
    name: str
    meshes: list
    qint: np.ndarray        # (n, 4) int32: model_a, model_b, seed_a, seed_b
    poses: np.ndarray       # (n, 48) float64
    params: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.qint.shape[0])

    def subset(self, idx) -> "Workload":
        idx = np.asarray(idx)
        return Workload(self.name, self.meshes, np.ascontiguousarray(self.qint[idx]),
                        np.ascontiguousarray(self.poses[idx]), dict(self.params))


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """(n, 3, 3) uniformly distributed rotations (normalised Gaussian quaternions)."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return quat_to_mat(q)


def quat_to_mat(q: np.ndarray) -> np.ndarray:
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((len(q), 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - w * z)
    R[:, 0, 2] = 2 * (x * z + w * y)
    R[:, 1, 0] = 2 * (x * y + w * z)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - w * x)
    R[:, 2, 0] = 2 * (x * z - w * y)
    R[:, 2, 1] = 2 * (y * z + w * x)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def axis_angle(axis: np.ndarray, ang: np.ndarray) -> np.ndarray:
    """(n, 3, 3) rotations about unit ``axis`` by ``ang`` (Rodrigues)."""
    half = 0.5 * ang
    q = np.concatenate([axis * np.sin(half)[:, None], np.cos(half)[:, None]], axis=1)
    return quat_to_mat(q)


def unit_vectors(rng: np.random.Generator, n: int) -> np.ndarray:
    v = rng.standard_normal((n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def cone_directions(rng: np.random.Generator, centre: np.ndarray, half_angle: float) -> np.ndarray:
    """Unit vectors uniform in the cone of ``half_angle`` around each row of ``centre``."""
    n = len(centre)
    cos_t = 1.0 - rng.uniform(0, 1, n) * (1.0 - np.cos(half_angle))
    sin_t = np.sqrt(np.maximum(0.0, 1.0 - cos_t * cos_t))
    phi = rng.uniform(0, 2 * np.pi, n)
    a = np.where(np.abs(centre[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    e1 = np.cross(centre, a)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(centre, e1)
    return (cos_t[:, None] * centre + sin_t[:, None] * (np.cos(phi)[:, None] * e1 + np.sin(phi)[:, None] * e2))


def _subsample(points: np.ndarray, k: int) -> np.ndarray:
    if len(points) <= k:
        return points
    idx = np.linspace(0, len(points) - 1, k).astype(np.int64)
    return points[idx]


def place_at_gap(mesh_a: Mesh, mesh_b: Mesh, R0: np.ndarray, u: np.ndarray, gap: np.ndarray,
                 skeleton_points: int = 128, device: str | None = None) -> np.ndarray:
    """Translations T0 putting B (rotated by R0) along direction u from A's
    centroid so that the skeleton estimate of the surface gap equals ``gap``
    (outermost crossing: coarse scan inwards, then bisection)."""
    import torch

    dev = device or ("cuda" if torch.cuda.is_available() else "cpu")
    sa = torch.as_tensor(_subsample(mesh_a.skeleton, skeleton_points), dtype=torch.float64, device=dev)
    sb = torch.as_tensor(_subsample(mesh_b.skeleton, skeleton_points), dtype=torch.float64, device=dev)
    ca = torch.as_tensor(mesh_a.verts.mean(axis=0), dtype=torch.float64, device=dev)
    cb = torch.as_tensor(mesh_b.verts.mean(axis=0), dtype=torch.float64, device=dev)
    rr = mesh_a.skeleton_radius + mesh_b.skeleton_radius
    n = len(u)
    out = np.empty((n, 3))
    chunk = 4096 if dev == "cuda" else 512
    dmax = mesh_a.bbox_diag() + mesh_b.bbox_diag() + float(np.max(gap)) + 1.0
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        Rt = torch.as_tensor(R0[s:e], dtype=torch.float64, device=dev)
        ut = torch.as_tensor(u[s:e], dtype=torch.float64, device=dev)
        gt = torch.as_tensor(gap[s:e], dtype=torch.float64, device=dev)
        bl = torch.einsum("nij,kj->nki", Rt, sb - cb)  # B skeleton about its centroid, rotated

        def g(D):
            pts = bl + (ca + ut * D[:, None])[:, None, :]
            d = torch.cdist(pts, sa.unsqueeze(0).expand(len(pts), -1, -1))
            return d.flatten(1).min(dim=1).values - rr

        hi = torch.full((e - s,), dmax, dtype=torch.float64, device=dev)
        lo = torch.zeros_like(hi)
        found = torch.zeros(e - s, dtype=torch.bool, device=dev)
        steps = 48
        for k in range(1, steps + 1):
            D = torch.full_like(hi, dmax * (1.0 - k / steps))
            below = (g(D) < gt) & ~found
            lo = torch.where(below, D, lo)
            hi = torch.where(below, D + dmax / steps, hi)
            found |= below
        for _ in range(30):
            mid = 0.5 * (lo + hi)
            below = g(mid) < gt
            lo = torch.where(below, mid, lo)
            hi = torch.where(below, hi, mid)
        D = hi
        T = (ca + ut * D[:, None]) - torch.einsum("nij,j->ni", Rt, cb)
        out[s:e] = T.cpu().numpy()
    return out


def ccd_queries(mesh_a: Mesh, mesh_b: Mesh, n: int, seed: int, gap_range=(0.05, 1.0), speed_range=(0.5, 3.0),
                speed_log=False, cone_deg: float = 30.0, max_rot: float = np.pi, device: str | None = None,
                model_a: int = 0, model_b: int = 1, subset: int | None = None,
                indices: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
    """``n`` queries of the benchmark family: returns (qint (n, 4), poses (n, 48)).
    With ``subset`` only the first ``subset`` of the n queries are placed and
    returned, with ``indices`` only those queries (same random draws as the
    full set either way)."""
    rng = np.random.default_rng(seed)
    diag = mesh_a.bbox_diag()
    R0b = random_rotations(rng, n)
    u = unit_vectors(rng, n)
    gap = rng.uniform(gap_range[0], gap_range[1], n) * diag
    if speed_log:
        speed = np.exp(rng.uniform(np.log(speed_range[0]), np.log(speed_range[1]), n)) * diag
    else:
        speed = rng.uniform(speed_range[0], speed_range[1], n) * diag
    vdir = cone_directions(rng, -u, np.deg2rad(cone_deg))
    axis = unit_vectors(rng, n)
    ang = rng.uniform(0.0, max_rot, n)
    if subset is not None and subset < n:
        n = subset
        R0b, u, gap, speed, vdir, axis, ang = (x[:n] for x in (R0b, u, gap, speed, vdir, axis, ang))
    if indices is not None:
        idx = np.asarray(indices)
        n = len(idx)
        R0b, u, gap, speed, vdir, axis, ang = (x[idx] for x in (R0b, u, gap, speed, vdir, axis, ang))
    T0b = place_at_gap(mesh_a, mesh_b, R0b, u, gap, device=device)
    T1b = T0b + speed[:, None] * vdir
    R1b = np.einsum("nij,njk->nik", R0b, axis_angle(axis, ang))
    poses = np.zeros((n, POSE_WIDTH))
    eye = np.eye(3).reshape(9)
    poses[:, 0:9] = eye
    poses[:, 12:21] = eye
    poses[:, 24:33] = R0b.reshape(n, 9)
    poses[:, 33:36] = T0b
    poses[:, 36:45] = R1b.reshape(n, 9)
    poses[:, 45:48] = T1b
    qint = np.zeros((n, 4), dtype=np.int32)
    qint[:, 0] = model_a
    qint[:, 1] = model_b
    return qint, poses


def default_params(diag: float, th_ca_rel: float, qsize: int) -> dict:
    """Harness mapping of C2A_Solve's constants: th_ca -> tolerance_d and
    m_toc_delta (C2A_Solve ignores th_ca, C2A/src/C2A.cpp:2326, 2384-2388);
    t_delta 1e-4; contact threshold 2 d + 0.001 (C2A.cpp:2433); 150 CA
    iterations (C2A.cpp:2079).  qsize is the GPU front capacity."""
    th_ca = th_ca_rel * diag
    return dict(tol_d=th_ca, tol_t=1e-4, toc_delta=th_ca, contact_abs=0.001, with_contacts=1, max_iters=150,
                qsize=qsize, th_ca=th_ca)


def config1(n: int = 1000, seed: int = 1, device: str | None = None) -> Workload:
    """Two (2,3) torus-knot tubes, 100 x 16 = 3,200 triangles each; 1,000
    queries; gap U[0.05, 1] diag; |v| U[0.5, 3] diag; |w| U[0, pi];
    th_ca = 1e-3 diag; qsize 40."""
    knot = torus_knot(2, 3, 100, 16, 1.0, 0.15)
    qint, poses = ccd_queries(knot, knot, n, seed, device=device, model_a=0, model_b=0)
    return Workload("config1_torusknot3200_1000q", [knot], qint, poses, default_params(knot.bbox_diag(), 1e-3, 40))


def config2(n: int = 65536, seed: int = 2, device: str | None = None, subset: int | None = None,
            indices: np.ndarray | None = None) -> Workload:
    """Same family at 400 x 50 = 40,000 triangles, 65,536 queries,
    th_ca = 1e-4 diag, qsize 64, about 30% colliding within t in [0, 1].
    ``subset``/``indices`` place only some of the n queries (see ccd_queries)."""
    knot = torus_knot(2, 3, 400, 50, 1.0, 0.15)
    qint, poses = ccd_queries(knot, knot, n, seed, device=device, model_a=0, model_b=0, subset=subset,
                              cone_deg=CONFIG2_CONE_DEG, indices=indices)
    return Workload("config2_torusknot40000_65536q", [knot], qint, poses, default_params(knot.bbox_diag(), 1e-4, 64))


def pool_mesh(kind: int, tris: int, seed: int) -> Mesh:
    """One mesh of the uneven pool: kind 0 a torus knot ((2,3) or (3,5)), 1 a
    noisy icosphere (sigma 0.02; 20 * 4^k triangles, the k closest to ``tris``
    in log scale, 3 <= k <= 6), 2 a clustered soup (edge length lognormal
    mu = -4, sigma = 0.5 of the diagonal)."""
    if kind == 0:
        pq = (2, 3) if seed % 2 == 0 else (3, 5)
        around = max(6, int(round(np.sqrt(tris / 16.0))))
        segments = max(24, int(round(tris / (2.0 * around))))
        return torus_knot(pq[0], pq[1], segments, around, 1.0, 0.15 if pq == (2, 3) else 0.1)
    if kind == 1:
        k = int(np.clip(np.round(np.log(tris / 20.0) / np.log(4.0)), 3, 6))
        return icosphere(k, radius=1.0, noise=0.02, seed=seed)
    return triangle_soup(int(tris), clusters=8, diag=2.0, mu=-4.0, sigma=0.5, seed=seed)


def config3(n: int = 4096, seed: int = 3, pool: int = 12, tri_range=(1000, 200000), device: str | None = None,
            subset: int | None = None) -> Workload:
    """The uneven batch: ``n`` pairs drawn from a seeded pool of ``pool`` meshes
    (torus knots, noisy icospheres, clustered soups in turn), triangle counts
    log-uniform in ``tri_range``; |v| log-uniform in [0.01, 5] diag so CA
    iteration counts span 1 to the cap; gap U[0.05, 1] diag, |w| U[0, pi];
    th_ca = 1e-3 of the pool's median diagonal, qsize 64."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]), pool))
    ms = [pool_mesh(k % 3, counts[k], seed * 1000 + k) for k in range(pool)]
    pa = rng.integers(0, pool, n)
    pb = rng.integers(0, pool, n)
    seeds = rng.integers(0, 2**31 - 1, n)
    m = n if subset is None else min(subset, n)
    qint = np.zeros((m, 4), dtype=np.int32)
    poses = np.zeros((m, POSE_WIDTH))
    order = np.lexsort((pb[:m], pa[:m]))
    i = 0
    while i < m:  # one placement batch per (a, b) combination
        a, b = pa[order[i]], pb[order[i]]
        j = i
        while j < m and pa[order[j]] == a and pb[order[j]] == b:
            j += 1
        idx = order[i:j]
        q, p = ccd_queries(ms[a], ms[b], len(idx), int(seeds[idx[0]]), speed_range=(0.01, 5.0), speed_log=True,
                           cone_deg=CONFIG2_CONE_DEG, device=device, model_a=int(a), model_b=int(b))
        qint[idx] = q
        poses[idx] = p
        i = j
    diag = float(np.median([x.bbox_diag() for x in ms]))
    return Workload(f"config3_pool{pool}_{m}q", ms, qint, poses, default_params(diag, 1e-3, 64))


def near_contact_queries(mesh: Mesh, n: int, seed: int, distance_fn, gap_range=(1e-6, 1e-3), tangent_deg=5.0,
                         speed_range=(0.5, 3.0), max_rot: float = 0.05 * np.pi, device: str | None = None,
                         model: int = 0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """``n`` grazing queries of ``mesh`` against itself: B starts at an exact
    surface gap log-uniform in ``gap_range`` * diag and moves within
    ``tangent_deg`` of the tangent plane at its closest point (towards or away
    from A), turning by at most ``max_rot``.

    distance_fn(qint, poses) -> (distance, p1, p2) is an exact distance query
    (C2A_Distance, rel = abs = 0) for A at pose[0:12] and B at pose[24:36];
    the skeleton placement is refined along the approach direction by
    bisection on it.  Returns (qint, poses, achieved gaps)."""
    rng = np.random.default_rng(seed)
    diag = mesh.bbox_diag()
    R0b = random_rotations(rng, n)
    u = unit_vectors(rng, n)
    gap = np.exp(rng.uniform(np.log(gap_range[0]), np.log(gap_range[1]), n)) * diag
    speed = rng.uniform(speed_range[0], speed_range[1], n) * diag
    tang = unit_vectors(rng, n)
    phi = np.deg2rad(rng.uniform(-tangent_deg, tangent_deg, n))
    axis = unit_vectors(rng, n)
    ang = rng.uniform(0.0, max_rot, n)
    T0 = place_at_gap(mesh, mesh, R0b, u, np.maximum(gap, 1e-3 * diag), device=device)
    qint = np.zeros((n, 4), dtype=np.int32)
    qint[:, 0] = qint[:, 1] = model
    eye = np.eye(3).reshape(9)

    def poses_at(T):
        P = np.zeros((n, POSE_WIDTH))
        P[:, 0:9] = eye
        P[:, 12:21] = eye
        P[:, 24:33] = R0b.reshape(n, 9)
        P[:, 33:36] = T
        P[:, 36:45] = R0b.reshape(n, 9)
        P[:, 45:48] = T
        return P

    def dist(D):
        d, _, _ = distance_fn(qint, poses_at(T0 + u * D[:, None]))
        return d

    # bracket the target gap along u (the skeleton estimate is good to ~1e-3 diag), then bisect
    lo = np.full(n, -4e-3 * diag)
    hi = np.full(n, 4e-3 * diag)
    for _ in range(6):
        dl, dh = dist(lo), dist(hi)
        lo = np.where(dl >= gap, lo * 2.0, lo)
        hi = np.where(dh <= gap, hi * 2.0, hi)
    for _ in range(48):
        mid = 0.5 * (lo + hi)
        below = dist(mid) <= gap
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    T = T0 + u * hi[:, None]
    d, p1, p2 = distance_fn(qint, poses_at(T))
    q2 = np.einsum("nij,nj->ni", R0b, p2) + T  # B's closest point in A's frame
    nrm = q2 - p1
    nn = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(nn > 0, nrm / np.where(nn > 0, nn, 1.0), u)
    t = tang - np.sum(tang * nrm, axis=1, keepdims=True) * nrm
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    vdir = np.cos(phi)[:, None] * t - np.sin(phi)[:, None] * nrm  # phi > 0: towards A
    poses = poses_at(T)
    poses[:, 45:48] = T + speed[:, None] * vdir
    poses[:, 36:45] = np.einsum("nij,njk->nik", R0b, axis_angle(axis, ang)).reshape(n, 9)
    return qint, poses, d


def gpu_distance_fn(ctx, mesh_id: int):
    """distance_fn for near_contact_queries through the library's batch distance query."""
    def fn(qint, poses):
        q = qint.copy()
        q[:, 0] = q[:, 1] = mesh_id
        r = ctx.distance(q, poses)
        return r["distance"].copy(), r["p1"].copy(), r["p2"].copy()
    return fn


def config4(distance_fn, n: int = 65536, n_near: int = 16384, seed: int = 4, device: str | None = None,
            subset: int | None = None, near_subset: int | None = None) -> Workload:
    """Config 2's knots and queries plus ``n_near`` near-contact grazing
    queries (initial gap log-uniform in [1e-6, 1e-3] diag, velocity within 5
    degrees of the tangent plane)."""
    base = config2(n=n, seed=2, device=device, subset=subset)
    knot = base.meshes[0]
    m = n_near if near_subset is None else min(near_subset, n_near)
    qn, pn, _ = near_contact_queries(knot, m, seed, distance_fn, device=device)
    return Workload(f"config4_torusknot40000_{base.n}q+{m}near", [knot], np.concatenate([base.qint, qn]),
                    np.concatenate([base.poses, pn]), dict(base.params))


def small_knots(n: int, seed: int, segments: int = 24, around: int = 6, device: str | None = None) -> Workload:
    """A quick-to-check variant of config 1 (288-triangle knots) for unit tests."""
    knot = torus_knot(2, 3, segments, around, 1.0, 0.15)
    qint, poses = ccd_queries(knot, knot, n, seed, device=device, model_a=0, model_b=0)
    return Workload(f"knot{knot.num_tris}_{n}q", [knot], qint, poses, default_params(knot.bbox_diag(), 1e-3, 40))
