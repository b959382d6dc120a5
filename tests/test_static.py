"""The static proximity queries beside the CA path: C2A_Tolerance (qsize 2)
and C2A_Collide, batched on the GPU (c2a_tolerance_batch /
c2a_collide_batch).  On the CPU: the OBB hierarchy the collide query walks
against the oracle's; on the GPU: every output bit for bit against the
reference's own outputs (tests/golden/static_queries_ref.npz) and against the
oracle on meshes of up to 40,000 triangles."""
import numpy as np
import pytest

from c2a_testutil import GOLDEN, bits


def _meshes_of(z):
    from c2a_gb300 import meshes

    return [meshes.Mesh(f"s{i}", z[f"mesh{i}_verts"], z[f"mesh{i}_faces"], np.zeros((1, 3)), 0.0)
            for i in range(int(z["num_meshes"]))]


def _poses(R, T):
    """model a at the identity, model b at (R, T): the relative transform the
    oracle's static queries take"""
    n = len(R)
    P = np.zeros((n, 48))
    P[:, 0:9] = np.eye(3).reshape(9)
    P[:, 24:33] = np.asarray(R).reshape(n, 9)
    P[:, 33:36] = T
    P[:, 12:24] = P[:, 0:12]
    P[:, 36:48] = P[:, 24:36]
    return P


def _static_meshes():
    from c2a_gb300 import meshes

    return [meshes.torus_knot(2, 3, 400, 50), meshes.triangle_soup(6000, clusters=8, seed=71),
            meshes.icosphere(4, radius=0.9, noise=0.02, seed=72)]


def _placements(n, seed, reach=2.0):
    from c2a_gb300 import workloads

    rng = np.random.default_rng(seed)
    R = workloads.random_rotations(rng, n).reshape(n, 9)
    T = workloads.unit_vectors(rng, n) * rng.uniform(0.0, reach, (n, 1))
    return R, T


@pytest.mark.parametrize("which", [0, 1, 2])
def test_obb_hierarchy_matches_oracle(lib, port, which):
    """The collide query's OBBs (centre in the parent's frame, half extents)
    are the oracle's bit for bit; the oracle's are pinned to the reference by
    the static-query fixture."""
    from c2a_gb300 import api, meshes

    m = [meshes.torus_knot(2, 3, 60, 12), meshes.triangle_soup(700, clusters=4, seed=5),
         meshes.icosphere(2, radius=0.8, noise=0.02, seed=6)][which]
    nodes, _ = port.dump(port.models([m]), 0)
    with api.Context(-1) as ctx:
        o = ctx.download_obb(ctx.model(m))
    assert o.shape == (len(nodes), 6)
    assert bits(o[:, 0:3]) == bits(nodes["To"]) and bits(o[:, 3:6]) == bits(nodes["d"])


def test_static_queries_need_a_device(lib):
    from c2a_gb300 import api, meshes

    with api.Context(-1) as ctx:
        mid = ctx.model(meshes.torus_knot(2, 3, 12, 4))
        q = np.array([[mid, mid, 0, 0]], dtype=np.int32)
        with pytest.raises(api.C2AError) as e:
            ctx.tolerance(q, _poses(np.eye(3).reshape(1, 9), np.zeros((1, 3))), 0.1)
        assert e.value.status == api.ERR_NO_DEVICE
        with pytest.raises(api.C2AError) as e:
            ctx.collide(q, _poses(np.eye(3).reshape(1, 9), np.zeros((1, 3))))
        assert e.value.status == api.ERR_NO_DEVICE


@pytest.mark.gpu
def test_static_queries_match_reference_fixture(gpu_ctx):
    """All 96 fixture pairs: closer, distance, both points and the counters of
    C2A_Tolerance; every contacting pair in order and the counters of
    C2A_Collide."""
    z = np.load(f"{GOLDEN}/static_queries_ref.npz")
    mids = gpu_ctx.models(_meshes_of(z))
    q = np.zeros((len(z["ab"]), 4), dtype=np.int32)
    q[:, 0] = [mids[a] for a in z["ab"][:, 0]]
    q[:, 1] = [mids[b] for b in z["ab"][:, 1]]
    P = _poses(z["R"], z["T"])
    tr = gpu_ctx.tolerance(q, P, z["tol"])
    e = z["tol_out"]
    assert np.array_equal(tr["closer"], z["closer"]) and (tr["status"] == 0).all()
    assert np.array_equal(tr["num_bv_tests"], e[:, 7].astype(np.int64))
    assert np.array_equal(tr["num_tri_tests"], e[:, 8].astype(np.int64))
    c = z["closer"] == 1
    assert 10 < c.sum() < len(c)
    assert bits(tr["distance"][c]) == bits(e[c, 0])
    assert bits(tr["p1"][c]) == bits(e[c, 1:4]) and bits(tr["p2"][c]) == bits(e[c, 4:7])
    offs = z["pair_offsets"]
    slots = int(np.diff(offs).max())
    cr, pairs = gpu_ctx.collide(q, P, 1, slots)
    assert (cr["status"] == 0).all()
    assert np.array_equal(cr["num_pairs"], np.diff(offs))
    assert np.array_equal(np.stack([cr["num_bv_tests"], cr["num_tri_tests"]], 1), z["collide_counts"])
    for i in range(len(q)):
        assert np.array_equal(pairs[i, :cr["num_pairs"][i]], z["pairs"][offs[i]:offs[i + 1]]), i


@pytest.mark.gpu
def test_tolerance_matches_oracle_on_large_meshes(gpu_ctx, port):
    ms = _static_meshes()
    models = port.models(ms)
    mids = gpu_ctx.models(ms)
    rng = np.random.default_rng(73)
    n = 384
    ab = rng.integers(0, 3, (n, 2))
    R, T = _placements(n, 74, reach=3.0)
    tol = rng.uniform(0.0, 0.2, n)
    tol[::17] = 0.0
    q = np.zeros((n, 4), dtype=np.int32)
    q[:, 0] = [mids[a] for a in ab[:, 0]]
    q[:, 1] = [mids[b] for b in ab[:, 1]]
    tr = gpu_ctx.tolerance(q, _poses(R, T), tol)
    closer = 0
    for i, (a, b) in enumerate(ab):
        c, d, p1, p2, nbv, ntri = port.tolerance(models, a, b, R[i], T[i], tol[i])
        assert (tr["closer"][i], tr["num_bv_tests"][i], tr["num_tri_tests"][i]) == (c, nbv, ntri), i
        if c:
            closer += 1
            assert bits(tr["distance"][i]) == bits(d) and bits(tr["p1"][i]) == bits(p1), i
            assert bits(tr["p2"][i]) == bits(p2), i
    assert 0.1 * n < closer < 0.95 * n


@pytest.mark.gpu
@pytest.mark.parametrize("flag", [1, 2])
def test_collide_matches_oracle_on_large_meshes(gpu_ctx, port, flag):
    ms = _static_meshes()
    models = port.models(ms)
    mids = gpu_ctx.models(ms)
    rng = np.random.default_rng(75 + flag)
    n = 256
    ab = rng.integers(0, 3, (n, 2))
    R, T = _placements(n, 77 + flag, reach=3.0)
    q = np.zeros((n, 4), dtype=np.int32)
    q[:, 0] = [mids[a] for a in ab[:, 0]]
    q[:, 1] = [mids[b] for b in ab[:, 1]]
    slots = 96  # fewer than some queries find: the overflowing ones keep their first 96 pairs
    cr, pairs = gpu_ctx.collide(q, _poses(R, T), flag, slots)
    hit = over = 0
    for i, (a, b) in enumerate(ab):
        exp, nbv, ntri = port.collide(models, a, b, R[i], T[i], flag)
        assert (cr["num_pairs"][i], cr["num_bv_tests"][i], cr["num_tri_tests"][i]) == (len(exp), nbv, ntri), i
        k = min(len(exp), slots)
        assert np.array_equal(pairs[i, :k], exp[:k]), i
        assert cr["status"][i] == (4 if len(exp) > slots else 0), i  # C2A_QUERY_CONTACT_OVERFLOW
        hit += len(exp) > 0
        over += len(exp) > slots
    assert 0.1 * n < hit < n
    if flag == 1:
        assert over > 0
    else:
        assert (cr["num_pairs"] <= 1).all()


@pytest.mark.gpu
def test_static_queries_reject_bad_models(gpu_ctx):
    from c2a_gb300 import api

    q = np.array([[0, 9999, 0, 0]], dtype=np.int32)
    P = _poses(np.eye(3).reshape(1, 9), np.zeros((1, 3)))
    with pytest.raises(api.C2AError) as e:
        gpu_ctx.tolerance(q, P, 0.1)
    assert e.value.status == api.ERR_QUERY_FAILED
    r = gpu_ctx.tolerance(q, P, 0.1, check=False)
    assert r["status"][0] == api.QUERY_BAD_INPUT
    r, _ = gpu_ctx.collide(q, P, 1, 4, check=False)
    assert r["status"][0] == api.QUERY_BAD_INPUT
    assert len(gpu_ctx.tolerance(q[:0], P[:0], 0.1)) == 0


@pytest.mark.gpu
def test_cpp_dropin_static_queries_match_reference_fixture(lib, port):
    """C2A_Tolerance, C2A_Collide and C2A_Distance of the C++ drop-in
    (include/c2a_gb300_cpp.h) on the fixture's 96 pairs: the reference's
    outputs, and the oracle's distance."""
    import os
    import subprocess

    from c2a_gb300 import build

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = os.path.join(build.OUT_DIR, "static_dropin")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "cpp", "static_dropin.cpp"), "-o", exe, build.LIB,
                    f"-Wl,-rpath,{build.OUT_DIR}"], check=True)
    z = np.load(f"{GOLDEN}/static_queries_ref.npz")
    ms = _meshes_of(z)
    inp = os.path.join(build.OUT_DIR, "static_dropin.bin")
    with open(inp, "wb") as fh:
        np.array([len(ms)], np.int32).tofile(fh)
        for m in ms:
            np.array([len(m.verts), m.num_tris], np.int32).tofile(fh)
            m.verts.astype(np.float64).tofile(fh)
            m.faces.astype(np.int32).tofile(fh)
        np.array([len(z["ab"])], np.int32).tofile(fh)
        for i, (a, b) in enumerate(z["ab"]):
            np.array([a, b], np.int32).tofile(fh)
            z["R"][i].astype(np.float64).tofile(fh)
            z["T"][i].astype(np.float64).tofile(fh)
            np.array([z["tol"][i]], np.float64).tofile(fh)
    lines = subprocess.run([exe, inp], check=True, capture_output=True, text=True).stdout.strip().split("\n")
    assert len(lines) == 3 * len(z["ab"])
    models = port.models(ms)
    offs = z["pair_offsets"]
    for i, (a, b) in enumerate(z["ab"]):
        t = lines[3 * i].split()
        e = z["tol_out"][i]
        assert int(t[0]) == z["closer"][i] and (int(t[8]), int(t[9])) == (int(e[7]), int(e[8])), i
        if int(t[0]):
            assert [float(x) for x in t[1:8]] == e[:7].tolist(), i
        c = list(map(int, lines[3 * i + 1].split()))
        assert c[0] == offs[i + 1] - offs[i] and (c[1], c[2]) == tuple(z["collide_counts"][i]), i
        assert np.array_equal(np.array(c[3:], np.int32).reshape(-1, 2), z["pairs"][offs[i]:offs[i + 1]]), i
        d = lines[3 * i + 2].split()
        pd, _, _ = port.distance(models, a, b, z["R"][i], z["T"][i], 0, 0)
        assert float(d[0]) == pd, i
