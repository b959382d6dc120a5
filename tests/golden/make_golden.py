"""Generates the golden fixtures from the reference's own C2A sources.

Run where the reference is compiled (``make -C oracle ref``):

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py canonical  # the canonical-mode ones only
    python tests/golden/make_golden.py demo       # the shipped demo scene only

Each fixture stores its inputs (mesh vertices and faces, query poses and
seeds, parameters) together with what the reference computed, so checking it
needs neither the reference nor a cross-platform-identical mesh generator.
The reference runs through oracle/_ref/libc2a_ref.so: C2A's sources compiled
unmodified against the PQP-interface restatement, with sin/cos/acos routed to
the deterministic implementation (correctly rounded).
"""
from __future__ import annotations

import contextlib
import ctypes
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from c2a_gb300 import meshes, replay, workloads  # noqa: E402
from oracle.oracle import RESULT_DTYPE, CONTACT_DTYPE, Ref, build  # noqa: E402


@contextlib.contextmanager
def quiet_stdout():
    """The reference's EndModel and C2A_Solve print to stdout; keep the log clean."""
    libc = ctypes.CDLL(None)
    sys.stdout.flush()
    libc.fflush(None)
    fd = os.dup(1)
    with open(os.devnull, "w") as dn:
        os.dup2(dn.fileno(), 1)
        try:
            yield
        finally:
            libc.fflush(None)
            sys.stdout.flush()
            os.dup2(fd, 1)
            os.close(fd)


def run_ref(ref, handles, wl, shipped=False, max_contacts=4096, handles_b=None):
    """handles_b: separate model objects for side B (the canonical composition
    needs them: C2A_Distance records its closest pair in each model's last_tri)."""
    res = np.zeros(wl.n, dtype=RESULT_DTYPE)
    cons, offs = [], [0]
    canonical = wl.params.get("mode", 0) == 1
    hb = handles if handles_b is None else handles_b
    with quiet_stdout():
        for q in range(wl.n):
            ma, mb, sa, sb = (int(x) for x in wl.qint[q])
            r, c = ref.solve(handles[ma], hb[mb], wl.poses[q], sa, sb, wl.params, max_contacts=max_contacts,
                             shipped=shipped)
            res[q] = r
            # the reference's list is push_front: store in visiting order
            # (the canonical composition returns them sorted by triangle pair)
            cons.append(np.ascontiguousarray(c if canonical else c[::-1]))
            offs.append(offs[-1] + len(c))
    con = np.concatenate(cons) if offs[-1] else np.zeros(0, dtype=CONTACT_DTYPE)
    return res, con, np.array(offs, dtype=np.int64)


def save_workload(name, wl, res, con, offs, extra=None):
    arrays = dict(qint=wl.qint, poses=wl.poses, results=res, contacts=con, contact_offsets=offs,
                  params=np.array([wl.params["tol_d"], wl.params["tol_t"], wl.params["toc_delta"],
                                   wl.params["contact_abs"], wl.params.get("with_contacts", 1),
                                   wl.params.get("max_iters", 150)]))
    for i, m in enumerate(wl.meshes):
        arrays[f"mesh{i}_verts"] = m.verts
        arrays[f"mesh{i}_faces"] = m.faces
    arrays["num_meshes"] = np.array(len(wl.meshes))
    if extra:
        arrays.update(extra)
    np.savez_compressed(os.path.join(HERE, name), **arrays)
    print(f"{name}: {wl.n} queries, {int((1 - res['collisionfree']).sum())} colliding, "
          f"{len(con)} contacts, mean numCA {res['numCA'].mean():.2f}")


def translation_queries(mesh, n, seed):
    """Both objects purely translating (|w| = 0): C2A's translation-only CA
    (C2A/src/C2A.cpp:2391-2395).  Object A moves (the reference uses only
    object 1's velocity, InterpMotion.cpp:663-665)."""
    rng = np.random.default_rng(seed)
    diag = mesh.bbox_diag()
    poses = np.zeros((n, 48))
    eye = np.eye(3).reshape(9)
    for q in range(n):
        R = workloads.random_rotations(rng, 1)[0].reshape(9)
        d = workloads.unit_vectors(rng, 1)[0]
        T0b = d * diag * rng.uniform(1.05, 1.6)
        vA = (d + 0.3 * workloads.unit_vectors(rng, 1)[0]) * diag * rng.uniform(0.2, 1.5)
        poses[q, 0:9] = eye
        poses[q, 9:12] = 0.0
        poses[q, 12:21] = eye
        poses[q, 21:24] = vA
        poses[q, 24:33] = R
        poses[q, 33:36] = T0b
        poses[q, 36:45] = R
        poses[q, 45:48] = T0b
    qint = np.zeros((n, 4), dtype=np.int32)
    return qint, poses


def geometry_vectors(ref, seed=11, n=400):
    rng = np.random.default_rng(seed)
    Rab = workloads.random_rotations(rng, n).reshape(n, 9)
    # a few exactly parallel / axis-aligned rectangles (the 1e-7 slab tests)
    Rab[: n // 8] = np.tile(np.eye(3).reshape(9), (n // 8, 1))
    Rab[n // 8: n // 4] = workloads.axis_angle(np.tile([[0.0, 0.0, 1.0]], (n // 8, 1)),
                                              rng.choice([0.0, np.pi / 2, np.pi], n // 8)).reshape(-1, 9)
    Tab = rng.normal(0, 1.0, (n, 3))
    Tab[n // 4: n // 3, 2] = 0.0  # coplanar rectangles
    a = rng.uniform(0, 1.5, (n, 2))
    b = rng.uniform(0, 1.5, (n, 2))
    a[::17] = 0.0  # degenerate rectangles (segments / points)
    rd = np.zeros(n)
    rS = np.full((n, 3), np.nan)
    for i in range(n):
        d, P, Q, S = ref.rectdist(Rab[i], Tab[i], a[i], b[i])
        rd[i] = d
        rS[i] = S
    S9 = rng.normal(0, 1.0, (n, 9))
    T9 = S9 + rng.normal(0, 0.8, (n, 9))
    T9[: n // 10] = S9[: n // 10] + 0.01 * rng.normal(size=(n // 10, 9))  # overlapping / touching
    S9[n // 10: n // 5, 6:9] = S9[n // 10: n // 5, 0:3]  # degenerate triangles (two equal vertices)
    T9[n // 5: n // 4, 2::3] = 0.0  # coplanar with S after the next line
    S9[n // 5: n // 4, 2::3] = 0.0
    td = np.zeros(n)
    tP = np.zeros((n, 3))
    tQ = np.zeros((n, 3))
    tf = np.zeros((n, 5), dtype=np.int32)
    for i in range(n):
        d, P, Q, f = ref.tridist(S9[i], T9[i])
        td[i], tP[i], tQ[i], tf[i] = d, P, Q, f
    np.savez_compressed(os.path.join(HERE, "geometry_ref.npz"), Rab=Rab, Tab=Tab, a=a, b=b, rect_d=rd, rect_S=rS,
                        S9=S9, T9=T9, tri_d=td, tri_P=tP, tri_Q=tQ, tri_f=tf)
    print(f"geometry_ref.npz: {n} rectangle pairs, {n} triangle pairs")


def motion_vectors(ref, seed=12, n=200):
    rng = np.random.default_rng(seed)
    R0 = workloads.random_rotations(rng, n)
    axis = workloads.unit_vectors(rng, n)
    ang = rng.uniform(0, np.pi, n)
    ang[:10] = 0.0  # pure translation
    ang[10:15] = np.pi  # half turn (s == 0)
    R1 = np.einsum("nij,njk->nik", R0, workloads.axis_angle(axis, ang))
    R1[:10] = R0[:10]
    T0 = rng.normal(0, 2, (n, 3))
    T1 = T0 + rng.normal(0, 2, (n, 3))
    t = rng.uniform(0, 1.2, n)
    consts = np.zeros((n, 7))
    Rt = np.zeros((n, 9))
    Tt = np.zeros((n, 3))
    for i in range(n):
        axis_i, w, cv, R, T = ref.motion(R0[i], T0[i], R1[i], T1[i], t[i])
        consts[i, :3], consts[i, 3], consts[i, 4:] = axis_i, w, cv
        Rt[i], Tt[i] = R, T
    np.savez_compressed(os.path.join(HERE, "motion_ref.npz"), R0=R0.reshape(n, 9), T0=T0, R1=R1.reshape(n, 9),
                        T1=T1, t=t, consts=consts, Rt=Rt, Tt=Tt)
    print(f"motion_ref.npz: {n} motions")


def bvh_hashes(ref):
    out = {}
    fams = {"knot23_100x16": meshes.torus_knot(2, 3, 100, 16), "knot35_60x12": meshes.torus_knot(3, 5, 60, 12),
            "icosphere3": meshes.icosphere(3, noise=0.02, seed=3), "soup2000": meshes.triangle_soup(2000, seed=4),
            "knot23_400x50": meshes.torus_knot(2, 3, 400, 50), "icosphere1": meshes.icosphere(1, noise=0.02, seed=5)}
    for name, m in fams.items():
        with quiet_stdout():
            h = ref.model(m)
        f, fc, tv, tid, tidx = ref.dump(h)
        dig = hashlib.sha256()
        for a in (f, fc, tv, tid, tidx):
            dig.update(np.ascontiguousarray(a).tobytes())
        mesh_dig = hashlib.sha256(np.ascontiguousarray(m.verts).tobytes() + np.ascontiguousarray(m.faces).tobytes())
        out[name] = (dig.hexdigest(), mesh_dig.hexdigest())
        if m.num_tris <= 100:
            np.savez_compressed(os.path.join(HERE, f"bvh_{name}_ref.npz"), verts=m.verts, faces=m.faces, node_f=f,
                                first_child=fc, tri_v=tv, tri_id=tid, tri_idx=tidx)
    # the hashed arrays: node_f (n x 25 float64: R, Tr, l, r, angularRadius, R_loc), first_child
    # (int32), triangle vertices (float64), ids and vertex indices (int32), in post-build order
    with open(os.path.join(HERE, "bvh_hashes_ref.txt"), "w") as fh:
        for k, (v, mv) in out.items():
            fh.write(f"{k} {v} {mv}\n")
    print("bvh hashes:", out)


def canonical_fixtures(ref):
    """The CANONICAL composition of the reference's own functions: C2A_Distance
    (rel_err = abs_err = 0) seeds every rotation step with the closest pair."""
    wl = workloads.config1(n=64, seed=201, device="cpu")
    wl.params["mode"] = 1
    with quiet_stdout():
        hs = [ref.model(m) for m in wl.meshes]
        hb = [ref.model(m) for m in wl.meshes]
    save_workload("canonical_config1_ref.npz", wl, *run_ref(ref, hs, wl, handles_b=hb))

    knot = meshes.torus_knot(2, 3, 24, 6)
    ico = meshes.icosphere(2, radius=0.8, noise=0.02, seed=7)
    qa, pa = workloads.ccd_queries(knot, knot, 48, 202, gap_range=(0.0, 0.6), device="cpu", model_a=0, model_b=0)
    qb, pb = workloads.ccd_queries(knot, ico, 48, 203, gap_range=(0.02, 0.6), device="cpu", model_a=0, model_b=1)
    rng = np.random.default_rng(204)
    qa[:, 2] = rng.integers(0, knot.num_tris, len(qa))
    qa[:, 3] = rng.integers(0, knot.num_tris, len(qa))
    qb[:, 2] = rng.integers(0, knot.num_tris, len(qb))
    qb[:, 3] = rng.integers(0, ico.num_tris, len(qb))
    wl2 = workloads.Workload("canonical_mixed", [knot, ico], np.concatenate([qa, qb]), np.concatenate([pa, pb]),
                             workloads.default_params(knot.bbox_diag(), 1e-3, 40))
    wl2.params["mode"] = 1
    with quiet_stdout():
        hs = [ref.model(m) for m in wl2.meshes]
        hb = [ref.model(m) for m in wl2.meshes]
    save_workload("canonical_mixed_ref.npz", wl2, *run_ref(ref, hs, wl2, handles_b=hb))


def distance_queries(meshes_, pairs, n_per, seed):
    """Distance-query inputs: for each model pair, random rotations and
    translations of B (no zero entries, so placing A at the identity leaves
    R and T unchanged), from overlapping to well apart; random seed pairs."""
    rng = np.random.default_rng(seed)
    rows, Rs, Ts = [], [], []
    for ia, ib in pairs:
        R = workloads.random_rotations(rng, n_per).reshape(n_per, 9)
        u = workloads.unit_vectors(rng, n_per)
        scale = meshes_[ia].bbox_diag() * rng.choice([0.3, 0.7, 1.0, 1.5], n_per) * rng.uniform(0.6, 1.0, n_per)
        T = u * scale[:, None] + rng.normal(scale=1e-3, size=(n_per, 3))
        for k in range(n_per):
            rows.append([ia, ib, rng.integers(meshes_[ia].num_tris), rng.integers(meshes_[ib].num_tris)])
        Rs.append(R)
        Ts.append(T)
    return np.array(rows, dtype=np.int32), np.concatenate(Rs), np.concatenate(Ts)


def distance_fixtures(ref):
    """C2A_Distance (rel_err = abs_err = 0) of the reference on a knot, a soup and an icosphere."""
    ms = [meshes.torus_knot(2, 3, 100, 16, 1.0, 0.15), meshes.triangle_soup(1000, clusters=6, seed=31),
          meshes.icosphere(3, radius=0.9, noise=0.02, seed=32)]
    qint, R, T = distance_queries(ms, [(0, 0), (0, 1), (1, 2), (2, 0), (2, 2)], 24, 301)
    with quiet_stdout():
        ha = [ref.model(m) for m in ms]
        hb = [ref.model(m) for m in ms]
    out = np.array([ref.distance(ha[a], hb[b], R[i], T[i], sa, sb) for i, (a, b, sa, sb) in enumerate(qint)])
    arrays = dict(num_meshes=len(ms), qint=qint, R=R, T=T, distance=out[:, 0], tri_a=out[:, 1].astype(np.int32),
                  tri_b=out[:, 2].astype(np.int32))
    for i, m in enumerate(ms):
        arrays[f"mesh{i}_verts"] = m.verts
        arrays[f"mesh{i}_faces"] = m.faces
    np.savez_compressed(os.path.join(HERE, "distance_ref.npz"), **arrays)


def static_query_fixtures(ref):
    """C2A_Tolerance (qsize 2) and C2A_Collide (every contact) of the reference
    on a knot, a soup and an icosphere, placed from overlapping to apart."""
    ms = [meshes.torus_knot(2, 3, 40, 8), meshes.triangle_soup(600, clusters=5, seed=91),
          meshes.icosphere(2, radius=0.8, noise=0.02, seed=92)]
    with quiet_stdout():
        ha = [ref.model(m) for m in ms]
        hb = [ref.model(m) for m in ms]
    rng = np.random.default_rng(93)
    n = 96
    ab = rng.integers(0, 3, (n, 2)).astype(np.int32)
    R = workloads.random_rotations(rng, n).reshape(n, 9)
    T = workloads.unit_vectors(rng, n) * rng.uniform(0.0, 2.0, (n, 1)) + rng.normal(scale=1e-3, size=(n, 3))
    tol = rng.uniform(0.0, 0.3, n)
    closer = np.zeros(n, np.int32)
    tol_out = np.zeros((n, 9))
    pairs, offs, ccount = [], [0], np.zeros((n, 2), np.int64)
    for i, (a, b) in enumerate(ab):
        c, d, p1, p2, nbv, ntri = ref.tolerance(ha[a], hb[b], R[i], T[i], tol[i])
        closer[i] = c
        tol_out[i] = [d, *p1, *p2, nbv, ntri]
        pr, cbv, ctri = ref.collide(ha[a], hb[b], R[i], T[i], 1)
        pairs.append(pr)
        offs.append(offs[-1] + len(pr))
        ccount[i] = [cbv, ctri]
    arrays = dict(num_meshes=len(ms), ab=ab, R=R, T=T, tol=tol, closer=closer, tol_out=tol_out,
                  pairs=np.concatenate(pairs).astype(np.int32), pair_offsets=np.array(offs), collide_counts=ccount)
    for i, m in enumerate(ms):
        arrays[f"mesh{i}_verts"] = m.verts
        arrays[f"mesh{i}_faces"] = m.faces
    np.savez_compressed(os.path.join(HERE, "static_queries_ref.npz"), **arrays)


REF_DIR = os.environ.get("C2A_REF_DIR", "/root/reference")


def demo_scene_fixture(ref):
    """The shipped demo scene replayed through the reference frame by frame as
    cb_display does (CCDDemo/mainTorusknot.cpp:207-325): both objects the
    shipped bunny (69,664 triangles), key frames from the two shipped .ani
    files, every one of the 303 frames seeded with the models' last_tri that
    the previous frame left.  Stores each frame's seeds, results and contacts,
    and the bunny exactly: its vertices are six-decimal text, kept as integer
    millionths (integer / 1e6 is the correctly rounded double that the
    reader's %lf gives)."""
    path = os.path.join(REF_DIR, "tri_models", "bunny_noholes.tri")
    bunny = meshes.read_tri(path)
    tok = open(path).read().split()
    nv = int(tok[1])
    micro = np.array([int(t.replace(".", "")) for t in tok[3:3 + 3 * nv]], dtype=np.int64).reshape(nv, 3)
    assert np.abs(micro).max() < 2 ** 31 and all(len(t.split(".")[1]) == 6 for t in tok[3:3 + 3 * nv])
    assert np.array_equal(micro / 1e6, bunny.verts)
    a0 = replay.read_ani(os.path.join(REF_DIR, "models", "torusknot1.ani"))
    a1 = replay.read_ani(os.path.join(REF_DIR, "models", "torusknot2.ani"))
    n = len(a0[0])
    qint, poses = replay.demo_queries(a0, a1)
    params = replay.demo_params()
    res = np.zeros(n, dtype=RESULT_DTYPE)
    cons, offs = [], [0]
    with quiet_stdout():
        ha, hb = ref.model(bunny), ref.model(bunny)
        for i in range(n):
            qint[i, 2], qint[i, 3] = ref.last_tri(ha), ref.last_tri(hb)
            r, c = ref.solve(ha, hb, poses[i], int(qint[i, 2]), int(qint[i, 3]), params, shipped=True)
            res[i] = r
            cons.append(np.ascontiguousarray(c[::-1]))  # push_front list: stored in visiting order
            offs.append(offs[-1] + len(c))
    np.savez_compressed(os.path.join(HERE, "demo_scene_ref.npz"), verts_micro=micro.astype(np.int32),
                        faces=bunny.faces.astype(np.int32), qint=qint, poses=poses, results=res,
                        contacts=np.concatenate(cons) if cons else np.zeros(0, CONTACT_DTYPE),
                        contact_offsets=np.array(offs))
    print(f"demo_scene_ref.npz: {n} frames, {int((1 - res['collisionfree']).sum())} colliding, "
          f"{offs[-1]} contacts, mean numCA {res['numCA'].mean():.2f}")


def main():
    build(ref=True)
    ref = Ref()
    if sys.argv[1:] == ["demo"]:
        demo_scene_fixture(ref)
        return
    if sys.argv[1:] == ["static"]:
        static_query_fixtures(ref)
        return
    if sys.argv[1:] == ["canonical"]:
        canonical_fixtures(ref)
        return
    if sys.argv[1:] == ["distance"]:
        distance_fixtures(ref)
        return

    # 1. config-1 mesh (3,200-triangle (2,3) knots), 96 queries of the config-1 family, default seeds
    wl = workloads.config1(n=96, seed=101, device="cpu")
    with quiet_stdout():
        hs = [ref.model(m) for m in wl.meshes]
    save_workload("config1_ref.npz", wl, *run_ref(ref, hs, wl))

    # 2. small knots, random seed pairs, mixed models (knot A vs icosphere B), gap down to touching
    knot = meshes.torus_knot(2, 3, 24, 6)
    ico = meshes.icosphere(2, radius=0.8, noise=0.02, seed=7)
    qa, pa = workloads.ccd_queries(knot, knot, 64, 102, gap_range=(0.0, 0.6), device="cpu", model_a=0, model_b=0)
    qb, pb = workloads.ccd_queries(knot, ico, 64, 103, gap_range=(0.02, 0.6), device="cpu", model_a=0, model_b=1)
    rng = np.random.default_rng(104)
    qa[:, 2] = rng.integers(0, knot.num_tris, len(qa))
    qa[:, 3] = rng.integers(0, knot.num_tris, len(qa))
    qb[:, 2] = rng.integers(0, knot.num_tris, len(qb))
    qb[:, 3] = rng.integers(0, ico.num_tris, len(qb))
    wl2 = workloads.Workload("mixed", [knot, ico], np.concatenate([qa, qb]), np.concatenate([pa, pb]),
                             workloads.default_params(knot.bbox_diag(), 1e-3, 40))
    with quiet_stdout():
        hs = [ref.model(m) for m in wl2.meshes]
    save_workload("mixed_ref.npz", wl2, *run_ref(ref, hs, wl2))

    # 3. the shipped C2A_Solve entry point (th_ca ignored: 1e-4 everywhere)
    wl3 = workloads.small_knots(48, seed=105, device="cpu")
    wl3.params.update(tol_d=1e-4, tol_t=1e-4, toc_delta=1e-4, contact_abs=0.001)
    with quiet_stdout():
        hs = [ref.model(m) for m in wl3.meshes]
    save_workload("shipped_solve_ref.npz", wl3, *run_ref(ref, hs, wl3, shipped=True))

    # 4. translation-only CA
    tq, tp = translation_queries(knot, 48, 106)
    wl4 = workloads.Workload("translation", [knot], tq, tp, workloads.default_params(knot.bbox_diag(), 1e-3, 40))
    with quiet_stdout():
        hs = [ref.model(m) for m in wl4.meshes]
    save_workload("translation_ref.npz", wl4, *run_ref(ref, hs, wl4))

    geometry_vectors(ref)
    motion_vectors(ref)
    bvh_hashes(ref)
    canonical_fixtures(ref)
    distance_fixtures(ref)
    static_query_fixtures(ref)
    demo_scene_fixture(ref)


if __name__ == "__main__":
    main()
