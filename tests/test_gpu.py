"""The CUDA path against the reference: golden fixtures and the oracle port,
bit for bit, through the C ABI of libc2a_gb300.so."""
import os
import subprocess

import numpy as np
import pytest

from c2a_testutil import CONTACT_FIELDS, RESULT_FIELDS, bits, describe, load_fixture, result_mismatches

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def gpu_solve(ctx, meshes_, qint, poses, params, slots=4096):
    ids = ctx.models(meshes_)
    q = qint.copy()
    q[:, 0] = np.asarray(ids)[qint[:, 0]]
    q[:, 1] = np.asarray(ids)[qint[:, 1]]
    return ctx.solve(q, poses, params, contacts_per_query=slots)


@pytest.mark.parametrize("name", ["config1", "mixed", "translation"])
def test_gpu_matches_reference_fixture(gpu_ctx, name):
    ms, qint, poses, params, exp, econ, off = load_fixture(name)
    res, con = gpu_solve(gpu_ctx, ms, qint, poses, params)
    assert (res["status"] == 0).all()
    bad = result_mismatches(res, exp, con, econ, off)
    assert not bad, f"{len(bad)} of {len(exp)} differ; first " + describe(res, exp, bad[0])


def test_gpu_matches_shipped_c2a_solve(gpu_ctx):
    ms, qint, poses, params, exp, econ, off = load_fixture("shipped_solve")
    res, con = gpu_solve(gpu_ctx, ms, qint, poses, params)
    bad = result_mismatches(res, exp, con, econ, off, fields=[f for f in RESULT_FIELDS if f != "mint"])
    assert not bad, describe(res, exp, bad[0])


def test_gpu_matches_port_config1_full(gpu_ctx, port):
    """Config 1 in full: 1,000 queries, two 3,200-triangle (2,3) torus knots."""
    from c2a_gb300 import workloads

    wl = workloads.config1(n=1000, seed=1)
    res, con = gpu_solve(gpu_ctx, wl.meshes, wl.qint, wl.poses, wl.params, slots=512)
    pres, pcon = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, wl.params, threads=os.cpu_count(),
                                  contacts_per_query=512)
    flat = np.concatenate([pcon[q][:min(512, pres[q]["num_contact"])] for q in range(wl.n)])
    offs = np.concatenate([[0], np.cumsum(np.minimum(512, pres["num_contact"]))])
    bad = result_mismatches(res, pres, con, flat, offs)
    assert not bad, describe(res, pres, bad[0])
    assert 0.05 < 1 - res["collisionfree"].mean() < 0.99


def test_gpu_matches_port_mesh_families(gpu_ctx, port):
    """Icospheres, clustered soups and (3,5) knots against each other, random
    seed pairs, gaps down to touching."""
    from c2a_gb300 import meshes, workloads

    ms = [meshes.icosphere(3, radius=1.0, noise=0.02, seed=1), meshes.triangle_soup(1500, seed=2),
          meshes.torus_knot(3, 5, 80, 10)]
    rng = np.random.default_rng(4)
    qi, ps = [], []
    for k, (a, b) in enumerate([(0, 1), (1, 2), (2, 0), (1, 1)]):
        q, p = workloads.ccd_queries(ms[a], ms[b], 40, 50 + k, gap_range=(0.0, 0.5), device="cpu", model_a=a,
                                     model_b=b)
        q[:, 2] = rng.integers(0, ms[a].num_tris, len(q))
        q[:, 3] = rng.integers(0, ms[b].num_tris, len(q))
        qi.append(q)
        ps.append(p)
    qint, poses = np.concatenate(qi), np.concatenate(ps)
    params = workloads.default_params(ms[0].bbox_diag(), 1e-3, 40)
    res, con = gpu_solve(gpu_ctx, ms, qint, poses, params, slots=256)
    pres, pcon = port.solve_batch(port.models(ms), qint, poses, params, threads=os.cpu_count(),
                                  contacts_per_query=256)
    flat = np.concatenate([pcon[q][:min(256, pres[q]["num_contact"])] for q in range(len(qint))])
    offs = np.concatenate([[0], np.cumsum(np.minimum(256, pres["num_contact"]))])
    bad = result_mismatches(res, pres, con, flat, offs)
    assert not bad, describe(res, pres, bad[0])


def test_gpu_step_matches_port(gpu_ctx, port):
    """C2A_TimeOfContactStep at chosen times and schedule inputs."""
    import ctypes as C
    from c2a_gb300 import workloads
    from oracle.oracle import RESULT_DTYPE as PORT_RESULT, _params

    wl = workloads.small_knots(64, seed=21)
    rng = np.random.default_rng(8)
    lam = np.where(rng.random(wl.n) < 0.3, 0.0, rng.uniform(0, 0.9, wl.n))
    num_ca = rng.integers(0, 8, wl.n).astype(np.int32)
    prev = rng.choice([1.0, 0.004, 0.3], wl.n)
    ids = gpu_ctx.models(wl.meshes)
    q = wl.qint.copy()
    q[:, :2] = ids[0]
    res = gpu_ctx.step(q, wl.poses, lam, num_ca, prev, wl.params)
    L = port.lib
    L.c2a_port_step.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double,
                                C.c_void_p, C.c_void_p]
    models = port.models(wl.meshes)
    prm = _params(wl.params)
    for i in range(wl.n):
        out = np.zeros(1, dtype=PORT_RESULT)
        L.c2a_port_step(C.byref(models[0]), C.byref(models[0]), wl.poses[i].ctypes.data, 0, 0, float(lam[i]),
                        int(num_ca[i]), float(prev[i]), C.byref(prm), out.ctypes.data)
        for f in ("distance", "mint", "num_bv_tests", "num_tri_tests", "translation"):
            assert bits(res[i][f]) == bits(out[0][f]), (i, f)


def test_gpu_contact_only_matches_port(gpu_ctx, port):
    import ctypes as C
    from c2a_gb300 import workloads
    from oracle.oracle import CONTACT_DTYPE, _PortModel

    wl = workloads.small_knots(32, seed=22)
    thr = np.random.default_rng(1).uniform(0.0, 0.3, wl.n)
    # the end poses of the motions, where most pairs interpenetrate
    poses = wl.poses.copy()
    poses[:, 0:12], poses[:, 24:36] = wl.poses[:, 12:24], wl.poses[:, 36:48]
    wl.poses = poses
    ids = gpu_ctx.models(wl.meshes)
    q = wl.qint.copy()
    q[:, :2] = ids[0]
    res, con = gpu_ctx.contact_only(q, wl.poses, thr, contacts_per_query=2048)
    L = port.lib
    models = port.models(wl.meshes)
    for i in range(wl.n):
        p = wl.poses[i]
        buf = np.zeros(2048, dtype=CONTACT_DTYPE)
        n = L.c2a_port_contact_only(C.byref(models[0]), C.byref(models[0]), p[0:9].ctypes.data, p[9:12].ctypes.data,
                                    p[24:33].ctypes.data, p[33:36].ctypes.data, float(thr[i]), buf.ctypes.data, 2048)
        assert res[i]["num_contact"] == n, i
        for f in CONTACT_FIELDS:
            assert bits(con[i][:n][f]) == bits(buf[:n][f]), (i, f)
    assert res["num_contact"].sum() > 0


def test_gpu_edge_cases(gpu_ctx, port):
    from c2a_gb300 import api, meshes, workloads

    wl = workloads.small_knots(24, seed=23)
    ids = gpu_ctx.models(wl.meshes)
    q = wl.qint.copy()
    q[:, :2] = ids[0]
    # empty batch
    r, _ = gpu_ctx.solve(q[:0], wl.poses[:0], wl.params)
    assert len(r) == 0
    # bad model id and out-of-range seed: flagged per query, others unaffected
    bad = q.copy()
    bad[0, 0] = 999
    bad[1, 2] = 10 ** 6
    r, _ = gpu_ctx.solve(bad, wl.poses, wl.params, check=False)
    assert r[0]["status"] == api.QUERY_BAD_INPUT and r[1]["status"] == api.QUERY_BAD_INPUT
    good, _ = gpu_ctx.solve(q, wl.poses, wl.params)
    assert bits(r[2:]["toc"]) == bits(good[2:]["toc"])
    # one contact slot: the count stays exact and the overflow is flagged
    r1, c1 = gpu_ctx.solve(q, wl.poses, wl.params, contacts_per_query=1)
    many = good["num_contact"] > 1
    assert many.any()
    assert np.array_equal(r1["num_contact"], good["num_contact"])
    assert (r1["status"][many] & api.QUERY_CONTACT_OVERFLOW).all()
    # iteration cap: same answer as the oracle with the same cap
    capped = dict(wl.params, max_iters=2)
    rc, _ = gpu_ctx.solve(q, wl.poses, capped)
    pc, _ = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, capped, contacts_per_query=0)
    assert (rc["status"] & api.QUERY_ITER_CAP).any()
    for f in ("toc", "numCA", "collisionfree", "num_bv_tests"):
        assert bits(rc[f]) == bits(pc[f]), f
    # single-triangle models and a pair touching at t = 0
    tri = meshes.Mesh("tri", np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0.0]]), np.array([[0, 1, 2]], np.int32),
                      np.zeros((1, 3)), 0.0)
    pose = np.zeros((2, 48))
    eye = np.eye(3).reshape(9)
    for k in (0, 1):
        pose[k, 0:9] = pose[k, 12:21] = pose[k, 24:33] = eye
        pose[k, 33:36] = [0.2, 0.2, 0.5 if k == 0 else 0.0]
        pose[k, 36:45] = eye
        pose[k, 45:48] = [0.2, 0.2, -0.5]
    pose[:, 36:45] = workloads.axis_angle(np.array([[0, 0, 1.0]] * 2), np.array([0.3, 0.3])).reshape(2, 9)
    qi = np.zeros((2, 4), dtype=np.int32)
    r, c = gpu_solve(gpu_ctx, [tri], qi, pose, dict(wl.params, tol_d=1e-3, toc_delta=1e-3), slots=4)
    pr, pc = port.solve_batch(port.models([tri]), qi, pose, dict(wl.params, tol_d=1e-3, toc_delta=1e-3),
                              contacts_per_query=4)
    for f in RESULT_FIELDS:
        assert bits(r[f]) == bits(pr[f]), f
    assert r[1]["collisionfree"] == 0


def test_gpu_device_buffers_and_stream(gpu_ctx):
    """c2a_solve_batch_device on torch-allocated device memory and stream."""
    import torch
    from c2a_gb300 import api, workloads

    wl = workloads.small_knots(40, seed=24)
    ids = gpu_ctx.models(wl.meshes)
    q = wl.qint.copy()
    q[:, :2] = ids[0]
    host_res, _ = gpu_ctx.solve(q, wl.poses, wl.params, contacts_per_query=0)
    qs = api.make_queries(q, wl.poses)
    dq = torch.from_numpy(qs.view(np.uint8).copy()).cuda()
    dr = torch.zeros(wl.n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        gpu_ctx.solve_device(dq.data_ptr(), wl.n, wl.params, dr.data_ptr(), None, 0, stream=s.cuda_stream)
    s.synchronize()
    res = dr.cpu().numpy().view(api.RESULT_DTYPE)
    assert bits(res["toc"]) == bits(host_res["toc"]) and np.array_equal(res["numCA"], host_res["numCA"])


def test_gpu_config2_mesh_against_port(gpu_ctx, port):
    """Config 2's 40,000-triangle knots and th_ca = 1e-4 diag, on a sample of
    queries the oracle finishes quickly."""
    from c2a_gb300 import workloads

    wl = workloads.config2(n=96, seed=2)
    res, con = gpu_solve(gpu_ctx, wl.meshes, wl.qint, wl.poses, wl.params, slots=256)
    pres, pcon = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, wl.params, threads=os.cpu_count(),
                                  contacts_per_query=256)
    flat = np.concatenate([pcon[q][:min(256, pres[q]["num_contact"])] for q in range(wl.n)])
    offs = np.concatenate([[0], np.cumsum(np.minimum(256, pres["num_contact"]))])
    bad = result_mismatches(res, pres, con, flat, offs)
    assert not bad, describe(res, pres, bad[0])


def test_cpp_dropin_api(lib, port):
    """The C++ drop-in (C2A_Model, C2A_Solve, C2A_SolveBatch, ...) compiled
    against include/c2a_gb300_cpp.h and linked with the library."""
    from c2a_gb300 import build, workloads

    exe = os.path.join(build.OUT_DIR, "dropin_test")
    src = os.path.join(ROOT, "tests", "cpp", "dropin_test.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), src, "-o",
                    exe, build.LIB, f"-Wl,-rpath,{build.OUT_DIR}"], check=True)
    wl = workloads.small_knots(16, seed=25)
    inp = os.path.join(build.OUT_DIR, "dropin_in.bin")
    with open(inp, "wb") as fh:
        m = wl.meshes[0]
        np.array([m.num_tris, len(m.verts), wl.n], dtype=np.int32).tofile(fh)
        m.verts.astype(np.float64).tofile(fh)
        m.faces.astype(np.int32).tofile(fh)
        wl.poses.astype(np.float64).tofile(fh)
        np.array([wl.params["tol_d"]], dtype=np.float64).tofile(fh)
    out = subprocess.run([exe, inp], check=True, capture_output=True, text=True).stdout.split("\n")
    rows = [list(map(float, l.split())) for l in out if l.strip()]
    pres, _ = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, wl.params, contacts_per_query=0)
    assert len(rows) == 2 * wl.n
    for i in range(wl.n):
        for r in (rows[i], rows[wl.n + i]):  # C2A_Solve, then C2A_SolveBatch
            toc, numca, ncont, cf = r[0], int(r[1]), int(r[2]), int(r[3])
            assert toc == pres[i]["toc"] and numca == pres[i]["numCA"], i
            assert cf == pres[i]["collisionfree"] and ncont == pres[i]["num_contact"], i


@pytest.mark.parametrize("engine", [1, 3])
@pytest.mark.parametrize("name", ["config1", "mixed"])
def test_gpu_reference_engines_match_fixture(gpu_ctx, name, engine):
    """Both reference-order kernels: one warp per query (the node-pair tests
    split across the lanes) and one thread per query."""
    ms, qint, poses, params, exp, econ, off = load_fixture(name)
    prm = dict(params)
    prm["engine"] = engine
    res, con = gpu_solve(gpu_ctx, ms, qint, poses, prm)
    assert (res["status"] == 0).all()
    bad = result_mismatches(res, exp, con, econ, off)
    assert not bad, f"engine {engine}: {len(bad)} of {len(exp)} differ; first " + describe(res, exp, bad[0])


@pytest.mark.parametrize("engine", [0, 1, 3])
def test_gpu_config2_1024_queries_every_field(gpu_ctx, port, engine):
    """Config 2 (two 40,000-triangle knots, th_ca = 1e-4 diag): 1,024 queries
    through the default, warp and thread engines, every result field (TOC
    poses included) and every contact against the oracle."""
    from c2a_gb300 import workloads

    wl = workloads.config2(n=1024, seed=2, device="cpu")
    res, con = gpu_solve(gpu_ctx, wl.meshes, wl.qint, wl.poses, dict(wl.params, engine=engine), slots=256)
    pres, pcon = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, wl.params, threads=os.cpu_count(),
                                  contacts_per_query=256)
    flat = np.concatenate([pcon[q][:min(256, pres[q]["num_contact"])] for q in range(wl.n)])
    offs = np.concatenate([[0], np.cumsum(np.minimum(256, pres["num_contact"]))])
    bad = result_mismatches(res, pres, con, flat, offs)
    assert not bad, f"engine {engine}: {len(bad)} of {wl.n} differ; first " + describe(res, pres, bad[0])
    assert 0.05 < 1 - res["collisionfree"].mean() < 0.95 and (res["status"] & ~4 == 0).all()
