"""Procedural triangle meshes for the CCD workloads.

The reference ships one mesh fixture (``tri_models/bunny_noholes.tri``) and
measures nothing; the workloads here are the procedural families the
benchmark configurations name: (p, q) torus-knot tubes, noisy icospheres and
clustered triangle soups.  Every mesh also carries a *skeleton* (points plus a
radius) whose offset surface approximates it; the query generators use it to
place objects at a requested surface gap without an exact distance query.

All generators are seeded and return float64 vertices and int32 faces.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Mesh:
    """A triangle soup with shared vertices.

    verts: (V, 3) float64; faces: (F, 3) int32 vertex indices.
    skeleton: (K, 3) float64 points whose ``skeleton_radius`` offset is close to
    the surface (used only to place objects at a target gap).
    """

    name: str
    verts: np.ndarray
    faces: np.ndarray
    skeleton: np.ndarray
    skeleton_radius: float

    @property
    def num_tris(self) -> int:
        return int(self.faces.shape[0])

    def tri_verts(self) -> np.ndarray:
        """(F, 9) float64: p1, p2, p3 of every triangle (C2A_Model::AddTri order)."""
        return np.ascontiguousarray(self.verts[self.faces].reshape(-1, 9))

    def bbox_diag(self) -> float:
        lo = self.verts.min(axis=0)
        hi = self.verts.max(axis=0)
        return float(np.linalg.norm(hi - lo))


def _knot_centreline(p: int, q: int, n: int, scale: float) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Points, unit tangents and unit normals of a (p, q) torus knot."""
    phi = 2.0 * np.pi * np.arange(n) / n

    def curve(t):
        r = 1.0 + 0.5 * np.cos(q * t)
        return scale * np.stack([r * np.cos(p * t), r * np.sin(p * t), 0.5 * np.sin(q * t)], axis=-1)

    h = 1e-4
    c = curve(phi)
    d1 = (curve(phi + h) - curve(phi - h)) / (2 * h)
    d2 = (curve(phi + h) - 2 * c + curve(phi - h)) / (h * h)
    tan = d1 / np.linalg.norm(d1, axis=1, keepdims=True)
    nrm = d2 - np.sum(d2 * tan, axis=1, keepdims=True) * tan
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return c, tan, nrm


def torus_knot(p: int = 2, q: int = 3, segments: int = 100, around: int = 16, scale: float = 1.0,
               tube_radius: float = 0.15) -> Mesh:
    """Closed tube of radius ``tube_radius`` around a (p, q) torus knot.

    ``segments`` rings of ``around`` vertices; 2 * segments * around triangles
    (100 x 16 -> 3,200; 400 x 50 -> 40,000).  The ring frame is the Frenet
    frame of the centreline, which closes up because a torus knot's
    curvature never vanishes.
    """
    c, tan, nrm = _knot_centreline(p, q, segments, scale)
    bin_ = np.cross(tan, nrm)
    th = 2.0 * np.pi * np.arange(around) / around
    ct, st = np.cos(th), np.sin(th)
    verts = (c[:, None, :] + tube_radius * (ct[None, :, None] * nrm[:, None, :] + st[None, :, None] * bin_[:, None, :]))
    verts = verts.reshape(-1, 3)
    i = np.arange(segments)[:, None]
    j = np.arange(around)[None, :]
    v00 = i * around + j
    v10 = ((i + 1) % segments) * around + j
    v11 = ((i + 1) % segments) * around + (j + 1) % around
    v01 = i * around + (j + 1) % around
    f1 = np.stack([v00, v10, v11], axis=-1).reshape(-1, 3)
    f2 = np.stack([v00, v11, v01], axis=-1).reshape(-1, 3)
    faces = np.stack([f1, f2], axis=1).reshape(-1, 3).astype(np.int32)
    skel, _, _ = _knot_centreline(p, q, max(4 * segments, 400), scale)
    return Mesh(f"torusknot{p}{q}_{segments}x{around}", np.ascontiguousarray(verts, dtype=np.float64),
                np.ascontiguousarray(faces), skel, tube_radius)


def icosphere(subdiv: int, radius: float = 1.0, noise: float = 0.02, seed: int = 0) -> Mesh:
    """Subdivided icosahedron (20 * 4**subdiv triangles) with radial noise."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    verts = list(v / np.linalg.norm(v, axis=1, keepdims=True))
    faces = f
    for _ in range(subdiv):
        cache: dict[tuple[int, int], int] = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        faces = np.array(nf, dtype=np.int64)
    V = np.array(verts)
    rng = np.random.default_rng(seed)
    V = V * (radius * (1.0 + noise * rng.standard_normal(len(V))))[:, None]
    return Mesh(f"icosphere{subdiv}", np.ascontiguousarray(V), faces.astype(np.int32),
                np.zeros((1, 3)), radius * (1.0 - 3 * noise))


def triangle_soup(num_tris: int, clusters: int = 8, diag: float = 2.0, mu: float = -4.0, sigma: float = 0.5,
                  seed: int = 0) -> Mesh:
    """Clustered random triangles; edge lengths lognormal(mu, sigma) times ``diag``."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-0.35 * diag, 0.35 * diag, size=(clusters, 3))
    which = rng.integers(0, clusters, size=num_tris)
    spread = 0.12 * diag
    c = centres[which] + spread * rng.standard_normal((num_tris, 3))
    edge = diag * np.exp(mu + sigma * rng.standard_normal(num_tris))
    d1 = rng.standard_normal((num_tris, 3))
    d1 /= np.linalg.norm(d1, axis=1, keepdims=True)
    d2 = rng.standard_normal((num_tris, 3))
    d2 -= np.sum(d2 * d1, axis=1, keepdims=True) * d1
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    ang = rng.uniform(np.pi / 6, np.pi / 2, size=num_tris)
    p1 = c
    p2 = c + edge[:, None] * d1
    p3 = c + edge[:, None] * (np.cos(ang)[:, None] * d1 + np.sin(ang)[:, None] * d2)
    verts = np.stack([p1, p2, p3], axis=1).reshape(-1, 3)
    faces = np.arange(3 * num_tris, dtype=np.int32).reshape(-1, 3)
    idx = rng.choice(len(verts), size=min(len(verts), 512), replace=False)
    return Mesh(f"soup{num_tris}", np.ascontiguousarray(verts), faces, verts[idx], 0.0)


def read_tri(path: str) -> Mesh:
    """Reads the reference's ``.tri`` format: ``TRI nv nt``, vertices, 0-based
    index triples (reader: CCDDemo/mainTorusknot.cpp:445-488)."""
    with open(path) as fh:
        tok = fh.read().split()
    nv, nt = int(tok[1]), int(tok[2])
    v = np.array(tok[3:3 + 3 * nv], dtype=np.float64).reshape(nv, 3)
    f = np.array(tok[3 + 3 * nv:3 + 3 * nv + 3 * nt], dtype=np.int32).reshape(nt, 3)
    idx = np.linspace(0, nv - 1, min(nv, 512)).astype(np.int64)
    return Mesh(path.rsplit("/", 1)[-1], v, f, v[idx], 0.0)
