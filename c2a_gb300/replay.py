"""Headless replay of the reference demo's scenes: `.tri` meshes and `.ani`
key-frame files, turned into the CCD queries the demo solves frame by frame.

The `.ani` format (reader: CCDDemo/mainTorusknot.cpp:565-598): a header
"<nframes>f", then per frame "<index>f", nine numbers of R written column by
column (R[0][0] R[1][0] R[2][0] R[0][1] ...), and the three of T.

The demo's queries (cb_display, CCDDemo/mainTorusknot.cpp:207-325): frame i
(0 .. nframes - 1, the display loop's iframe)
moves object 0 from key frame step1 to step2 (0->1 for i < 101, 101->102 for
i < 202, else 202->203) and object 1 from its own translations at step1 and
step2 with the rotation of its key frame i held fixed, every frame solved
with C2A_Solve (th_ca ignored there, so tolerance 1e-4).  The demo seeds each
frame with the triangles the previous query left in the models' last_tri
(C2A.cpp:1175 mutates them); this library never mutates a model, so the
replay takes explicit seeds (triangle 0 unless given; the shipped scene's
fixture records the reference's per-frame seeds).  The shipped scene: both
objects tri_models/bunny_noholes.tri, object 0 keyed by models/torusknot1.ani,
object 1 by models/torusknot2.ani (mainTorusknot.cpp:53-57).
"""
from __future__ import annotations

import numpy as np

from . import workloads


def read_ani(path: str) -> tuple[np.ndarray, np.ndarray]:
    """(R (n, 3, 3), T (n, 3)) of an `.ani` file, indexed by frame number."""
    with open(path) as fh:
        tok = fh.read().split()
    n = int(float(tok[0].rstrip("f")))
    R = np.zeros((n, 3, 3))
    T = np.zeros((n, 3))
    k = 1
    while k + 12 < len(tok):
        i = int(float(tok[k].rstrip("f")))
        v = np.array(tok[k + 1:k + 13], dtype=np.float64)
        R[i] = v[:9].reshape(3, 3).T  # written column by column
        T[i] = v[9:12]
        k += 13
    return R, T


def write_ani(path: str, R: np.ndarray, T: np.ndarray):
    """The inverse of read_ani (for tests and generated scenes)."""
    with open(path, "w") as fh:
        fh.write(f"{len(R)}f\n")
        for i in range(len(R)):
            fh.write(f"{i}f\n")
            fh.write(" ".join(repr(float(x)) for x in R[i].T.reshape(9)) + "\n")
            fh.write(" ".join(repr(float(x)) for x in T[i]) + "\n")


def demo_steps(i: int) -> tuple[int, int, int]:
    """(step1, step2, step3) of frame i in cb_display."""
    if i < 101:
        s1, s2 = 0, 1
    elif i < 202:
        s1, s2 = 101, 102
    else:
        s1, s2 = 202, 203
    return s1, s2, i


def demo_queries(ani0, ani1, nframes: int | None = None, seeds=(0, 0),
                 model_a: int = 0, model_b: int = 1) -> tuple[np.ndarray, np.ndarray]:
    """The demo's per-frame queries for frames 0 .. nframes - 1 (qint, poses);
    seeds is one (seed_a, seed_b) pair for every frame or one pair per frame."""
    (R0, T0), (R1, T1) = ani0, ani1
    n = nframes if nframes is not None else len(R0)
    poses = np.zeros((n, workloads.POSE_WIDTH))
    for i in range(n):
        s1, s2, s3 = demo_steps(i)
        poses[i, 0:9] = R0[s1].reshape(9)
        poses[i, 9:12] = T0[s1]
        poses[i, 12:21] = R0[s2].reshape(9)
        poses[i, 21:24] = T0[s2]
        poses[i, 24:33] = R1[s3].reshape(9)
        poses[i, 33:36] = T1[s1]
        poses[i, 36:45] = R1[s3].reshape(9)
        poses[i, 45:48] = T1[s2]
    qint = np.zeros((n, 4), dtype=np.int32)
    qint[:, 0], qint[:, 1] = model_a, model_b
    sd = np.asarray(seeds, dtype=np.int32)
    qint[:, 2:4] = sd if sd.ndim == 2 else sd[None, :]
    return qint, poses


def demo_params(th_ca: float = 1e-4) -> dict:
    """C2A_Solve's constants as the demo runs it (th_ca ignored: 1e-4)."""
    return dict(tol_d=th_ca, tol_t=1e-4, toc_delta=th_ca, contact_abs=0.001, with_contacts=1, max_iters=150,
                qsize=2, th_ca=th_ca)


def synthetic_scene(frames: int = 40, seed: int = 0, gap: float = 0.6):
    """Key frames for two objects in the demo's layout: object 0 sweeps
    through object 1's place between consecutive key frames while turning
    about z; object 1 turns about a fixed axis from frame to frame."""
    rng = np.random.default_rng(seed)
    R0 = workloads.axis_angle(np.tile([0.0, 0.0, 1.0], (frames, 1)), 0.3 * np.arange(frames))
    T0 = np.zeros((frames, 3))
    for i in range(frames):
        T0[i] = [-gap - 2.0 + 2.5 * i, 0.01 * rng.normal(), 0.0]
    axis = np.array([0.3, 0.4, 0.866])
    R1 = workloads.axis_angle(np.tile(axis / np.linalg.norm(axis), (frames, 1)), np.linspace(0, 2.0, frames))
    T1 = np.tile([gap, 0.0, 0.0], (frames, 1)) + 0.02 * np.linspace(0, 1, frames)[:, None]
    return (R0, T0), (R1, T1)
