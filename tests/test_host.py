"""The library's host side without a GPU: its ABI surface, the RSS hierarchy
build (bit-identical to the reference's EndModel) and the motion model."""
import hashlib
import os
import re

import numpy as np
import pytest

from c2a_testutil import GOLDEN, bits

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header="c2a_gb300.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(c2a_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    from c2a_gb300 import api, learned

    names = declared_symbols()
    assert len(names) >= 14
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(api.ABI_SYMBOLS) == names
    probe = declared_symbols("c2a_probe.h")
    assert sorted(api.PROBE_SYMBOLS) == probe and all(hasattr(lib, n) for n in probe)
    mlp = declared_symbols("c2a_mlp.h")
    assert [n for n in mlp if not hasattr(lib, n)] == []
    assert sorted(learned.MLP_SYMBOLS) == mlp
    learned.bind(lib)  # every signature binds


def test_status_strings_and_host_only_context(lib):
    from c2a_gb300 import api, meshes, workloads

    assert api.status_str(0) == "ok"
    assert "no CUDA device" in api.status_str(2)
    with api.Context(-1) as ctx:
        knot = meshes.torus_knot(2, 3, 12, 4)
        mid = ctx.model(knot)
        assert ctx.model_info(mid) == (96, 191, ctx.model_info(mid)[2])
        qint = np.zeros((1, 4), dtype=np.int32)
        poses = np.zeros((1, 48))
        with pytest.raises(api.C2AError) as e:
            ctx.solve(qint, poses, workloads.default_params(1.0, 1e-3, 40))
        assert e.value.status == 2
        ctx.free_model(mid)
        with pytest.raises(api.C2AError):
            ctx.model_info(mid)


def test_empty_model_is_rejected(lib):
    import ctypes as C
    from c2a_gb300 import api

    with api.Context(-1) as ctx:
        mid = C.c_int32()
        assert lib.c2a_model_build(ctx.h, 0, None, None, None, C.byref(mid)) == 5  # C2A_ERR_EMPTY_MODEL


def _node_fields(ctx, mid):
    f, fc, tv, tid, tidx = ctx.download(mid)
    return f, fc, tv, tid, tidx


def test_bvh_matches_reference_dump(lib):
    from c2a_gb300 import api, meshes

    z = np.load(f"{GOLDEN}/bvh_icosphere1_ref.npz")
    m = meshes.Mesh("ico1", z["verts"], z["faces"], np.zeros((1, 3)), 0.0)
    with api.Context(-1) as ctx:
        f, fc, tv, tid, tidx = _node_fields(ctx, ctx.model(m))
    assert bits(f) == bits(z["node_f"]) and np.array_equal(fc, z["first_child"])
    assert bits(tv) == bits(z["tri_v"]) and np.array_equal(tid, z["tri_id"]) and np.array_equal(tidx, z["tri_idx"])


@pytest.mark.parametrize("name", ["knot23_100x16", "knot35_60x12", "icosphere3", "soup2000", "knot23_400x50"])
def test_bvh_matches_reference_hash(lib, name):
    from c2a_gb300 import api, meshes

    table = {l.split()[0]: l.split()[1:] for l in open(f"{GOLDEN}/bvh_hashes_ref.txt")}
    bvh_hash, mesh_hash = table[name]
    gen = {"knot23_100x16": lambda: meshes.torus_knot(2, 3, 100, 16),
           "knot35_60x12": lambda: meshes.torus_knot(3, 5, 60, 12),
           "icosphere3": lambda: meshes.icosphere(3, noise=0.02, seed=3),
           "soup2000": lambda: meshes.triangle_soup(2000, seed=4),
           "knot23_400x50": lambda: meshes.torus_knot(2, 3, 400, 50)}[name]
    m = gen()
    mh = hashlib.sha256(np.ascontiguousarray(m.verts).tobytes() + np.ascontiguousarray(m.faces).tobytes())
    if mh.hexdigest() != mesh_hash:
        pytest.skip("this platform's numpy generates a different mesh than the fixture's")
    with api.Context(-1) as ctx:
        arrays = _node_fields(ctx, ctx.model(m))
    dig = hashlib.sha256()
    for a in arrays:
        dig.update(np.ascontiguousarray(a).tobytes())
    assert dig.hexdigest() == bvh_hash


def test_bvh_matches_port_on_degenerate_soups(lib, port):
    """Degenerate triangles, repeated vertices, 1- and 2-triangle models."""
    from c2a_gb300 import api, meshes

    rng = np.random.default_rng(3)
    cases = []
    for n in (1, 2, 3, 7, 100):
        v = rng.normal(size=(3 * n, 3))
        f = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
        if n >= 3:
            v[3] = v[4]  # a zero-length edge
            v[6:9] = v[0]  # a triangle collapsed to a point
        cases.append(meshes.Mesh(f"soup{n}", v, f, v, 0.0))
    v = np.zeros((30, 3))
    v[:, 0] = np.arange(30)  # all collinear
    cases.append(meshes.Mesh("line", v, np.arange(30, dtype=np.int32).reshape(10, 3), v, 0.0))
    with api.Context(-1) as ctx:
        for m in cases:
            f, fc, tv, tid, tidx = _node_fields(ctx, ctx.model(m))
            nodes, tris = port.dump(port.models([m]), 0)
            pf = np.concatenate([nodes["R"], nodes["Tr"], nodes["l"], nodes["r"][:, None], nodes["angR"][:, None],
                                 nodes["Rloc"]], axis=1)
            assert bits(f) == bits(pf), m.name
            assert np.array_equal(fc, nodes["first_child"]), m.name
            assert bits(tv) == bits(tris["v"]), m.name


def _model_digest(ctx, mid):
    dig = hashlib.sha256()
    for a in ctx.download(mid):
        dig.update(np.ascontiguousarray(a).tobytes())
    dig.update(ctx.download_obb(mid).tobytes())
    return dig.hexdigest()


def test_threaded_build_is_bit_identical(lib, monkeypatch):
    """Subtrees split over host threads (a 40,000-triangle knot spawns them at
    4,096 triangles), alone or beside other models in c2a_model_build_many:
    the same tree whatever the thread count."""
    from c2a_gb300 import api, meshes

    ms = [meshes.torus_knot(2, 3, 400, 50), meshes.triangle_soup(9000, seed=5), meshes.torus_knot(3, 5, 60, 12),
          meshes.icosphere(3, noise=0.02, seed=3)]
    want = {}
    monkeypatch.setenv("C2A_BUILD_THREADS", "1")
    with api.Context(-1) as ctx:
        for m in ms:
            want[m.name] = _model_digest(ctx, ctx.model(m))
    for threads in ("2", "7", "16"):
        monkeypatch.setenv("C2A_BUILD_THREADS", threads)
        with api.Context(-1) as ctx:
            got = _model_digest(ctx, ctx.model(ms[0]))
        assert got == want[ms[0].name], threads
    for threads in (1, 3, 8):
        with api.Context(-1) as ctx:
            mid0 = ctx.model(ms[3])
            ids = ctx.models(ms, threads=threads)
            assert ids == [mid0 + 1 + i for i in range(len(ms))]
            assert [_model_digest(ctx, i) for i in ids] == [want[m.name] for m in ms], threads


def _chain_soup(n: int, ratio: float = 1.01) -> np.ndarray:
    """n small triangles at x = -ratio^i: every split at the mean cuts off a
    few hundred of the farthest, so the tree is a chain of large subtrees
    (depth ~57 for 40,000 triangles)."""
    x = -(ratio ** np.arange(n))
    s = 0.01 * np.abs(x)
    v = np.zeros((3 * n, 3))
    v[0::3, 0] = x
    v[1::3, 0], v[1::3, 1] = x, s
    v[2::3, 0], v[2::3, 2] = x, s
    return v


def test_threaded_build_matches_port_on_large_degenerate_soups(lib, port, monkeypatch):
    """Splits that fall back to n/2 (every centroid on one side) and repeated
    triangles, large enough that subtrees go to other threads: the threaded
    build against the oracle's sequential one."""
    from c2a_gb300 import api, meshes

    rng = np.random.default_rng(11)
    tri = rng.normal(size=(3, 3))
    same = np.tile(tri, (12000, 1))  # 12,000 copies of one triangle
    mixed = np.concatenate([same[:9000 * 3], rng.normal(size=(3 * 9000, 3))])
    cases = [meshes.Mesh(name, v, np.arange(len(v), dtype=np.int32).reshape(-1, 3), v, 0.0)
             for name, v in (("copies", same), ("copies+soup", mixed), ("chain", _chain_soup(30000)))]
    monkeypatch.setenv("C2A_BUILD_THREADS", "8")
    with api.Context(-1) as ctx:
        ids = ctx.models(cases, threads=8)
        for m, mid in zip(cases, ids):
            f, fc, tv, tid, tidx = ctx.download(mid)
            nodes, tris = port.dump(port.models([m]), 0)
            pf = np.concatenate([nodes["R"], nodes["Tr"], nodes["l"], nodes["r"][:, None], nodes["angR"][:, None],
                                 nodes["Rloc"]], axis=1)
            assert bits(f) == bits(pf), m.name
            assert np.array_equal(fc, nodes["first_child"]), m.name
            assert bits(tv) == bits(tris["v"]), m.name
            assert ctx.model_info(mid)[2] == int(np.ceil(np.log2(m.num_tris))) or m.name != "copies"
            assert ctx.model_info(mid)[2] > 40 or m.name != "chain"


@pytest.mark.parametrize("sanitizer", ["thread", "address,undefined"])
def test_threaded_build_under_sanitizer(tmp_path, sanitizer):
    """The threaded build (the subtree pool, record passes, the thread
    budget) compiled with ThreadSanitizer, then AddressSanitizer + UBSan,
    against the sequential build of a 40,000-triangle knot and of a
    chain-shaped tree: no report, and the same bytes in every record."""
    import shutil
    import subprocess

    from c2a_gb300 import meshes

    if not shutil.which("g++"):
        pytest.skip("no g++")
    knot = meshes.torus_knot(2, 3, 400, 50)
    soups = []
    for name, tv in (("knot", knot.tri_verts()), ("chain", _chain_soup(40000).reshape(-1, 9))):
        soups.append(tmp_path / f"{name}.bin")
        with open(soups[-1], "wb") as f:
            f.write(np.int32(len(tv)).tobytes())
            f.write(np.ascontiguousarray(tv).tobytes())
    exe = str(tmp_path / "build_race")
    subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-ffp-contract=off",
                    f"-fsanitize={sanitizer}", "-fno-sanitize-recover=all", "-pthread", "-o", exe,
                    os.path.join(ROOT, "tests", "cpp", "build_race.cpp"),
                    os.path.join(ROOT, "c2a_gb300", "csrc", "host", "bvh_build.cpp")], check=True)
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=1", ASAN_OPTIONS="halt_on_error=1:detect_leaks=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    for soup in soups:
        r = subprocess.run([exe, str(soup), "8"], capture_output=True, text=True, env=env, timeout=600)
        assert r.returncode == 0 and r.stdout.startswith("same"), r.stdout + r.stderr[-4000:]


def test_build_many_rejects_bad_input_and_keeps_nothing(lib):
    import ctypes as C
    from c2a_gb300 import api, meshes

    knot = meshes.torus_knot(2, 3, 12, 4)
    tv = knot.tri_verts()
    with api.Context(-1) as ctx:
        counts = np.array([knot.num_tris, 0], dtype=np.int32)
        ptrs = (C.c_void_p * 2)(tv.ctypes.data, tv.ctypes.data)
        ids = np.full(2, -1, dtype=np.int32)
        pp = C.cast(ptrs, C.c_void_p)
        assert lib.c2a_model_build_many(ctx.h, 2, api._ptr(counts), pp, None, None, 0, api._ptr(ids)) == \
            api.ERR_EMPTY_MODEL
        assert lib.c2a_model_build_many(ctx.h, -1, None, None, None, None, 0, None) == api.ERR_INVALID_ARGUMENT
        assert lib.c2a_model_build_many(ctx.h, 1, api._ptr(counts), pp, None, None, -2, api._ptr(ids)) == \
            api.ERR_INVALID_ARGUMENT
        assert lib.c2a_model_build_many(ctx.h, 0, None, None, None, None, 0, None) == api.OK
        assert ctx.models([]) == []
        assert ctx.model(knot) == 0  # the failed calls kept no model
        # per-model id and vertex-index arrays, one of them NULL: caller ids kept, the NULL entry numbered 0..n-1
        ids_in = np.arange(1000, 1000 + knot.num_tris, dtype=np.int32)
        vidx = np.ascontiguousarray(knot.faces, dtype=np.int32)
        counts = np.array([knot.num_tris, knot.num_tris], dtype=np.int32)
        id_ptrs = (C.c_void_p * 2)(ids_in.ctypes.data, None)
        vidx_ptrs = (C.c_void_p * 2)(None, vidx.ctypes.data)
        out = np.full(2, -1, dtype=np.int32)
        assert lib.c2a_model_build_many(ctx.h, 2, api._ptr(counts), pp, C.cast(id_ptrs, C.c_void_p),
                                        C.cast(vidx_ptrs, C.c_void_p), 2, api._ptr(out)) == api.OK
        assert list(out) == [1, 2]
        _, _, _, tid0, tidx0 = ctx.download(1)
        _, _, _, tid1, tidx1 = ctx.download(2)
        assert sorted(tid0) == list(ids_in) and sorted(tid1) == list(range(knot.num_tris))
        assert (tidx0 == -1).all() and np.array_equal(np.sort(tidx1, axis=None), np.sort(vidx, axis=None))
        assert np.array_equal(tid0 - 1000, tid1)  # the same tree


def test_async_build_equals_build(lib):
    """c2a_model_build_async + c2a_model_wait: the same tree as c2a_model_build,
    ids in the order the waits register them, errors reported by the wait or
    at once."""
    import ctypes as C
    from c2a_gb300 import api, meshes

    ms = [meshes.torus_knot(2, 3, 400, 50), meshes.icosphere(3, noise=0.02, seed=3), meshes.triangle_soup(5000, seed=2)]
    with api.Context(-1) as ctx:
        want = [_model_digest(ctx, ctx.model(m)) for m in ms]
    with api.Context(-1) as ctx:
        handles = [ctx.model_async(m) for m in ms]  # all three build at once
        ids = [ctx.model_wait(h) for h in reversed(handles)]
        assert ids == [0, 1, 2]
        assert [_model_digest(ctx, i) for i in reversed(ids)] == want
        h = C.c_void_p()
        assert lib.c2a_model_build_async(ctx.h, 0, None, None, None, C.byref(h)) == api.ERR_EMPTY_MODEL
        assert not h.value
        assert lib.c2a_model_build_async(ctx.h, 1, None, None, None, None) == api.ERR_INVALID_ARGUMENT
        assert lib.c2a_model_wait(None, None) == api.ERR_INVALID_ARGUMENT
        assert ctx.model(ms[1]) == 3


@pytest.mark.parametrize("value", ["0", "-3", "many", "1", "64"])
def test_build_threads_variable(lib, monkeypatch, value):
    """C2A_BUILD_THREADS: a positive count caps the threads, anything else
    means every hardware thread; the tree is the same either way."""
    from c2a_gb300 import api, meshes

    knot = meshes.torus_knot(2, 3, 200, 50)
    monkeypatch.setenv("C2A_BUILD_THREADS", value)
    with api.Context(-1) as ctx:
        got = _model_digest(ctx, ctx.model(knot))
    monkeypatch.setenv("C2A_BUILD_THREADS", "1")
    with api.Context(-1) as ctx:
        assert got == _model_digest(ctx, ctx.model(knot))


def test_motion_matches_reference(lib):
    """CInterpMotion_Linear constants and integrate() (InterpMotion.cpp:228-287,
    486-568) against the reference, bit for bit."""
    from c2a_gb300 import api

    z = np.load(f"{GOLDEN}/motion_ref.npz")
    for i in range(len(z["t"])):
        c = api.motion_setup(z["R0"][i], z["T0"][i], z["R1"][i], z["T1"][i])
        assert bits(c[:7]) == bits(z["consts"][i]), i
        R, T, qua = api.motion_integrate(z["R0"][i], z["T0"][i], z["R1"][i], z["T1"][i], z["t"][i])
        assert bits(R) == bits(z["Rt"][i]) and bits(T) == bits(z["Tt"][i]), i


def test_fp64_probe_and_static_queries_validate_arguments(lib):
    """Without a device the FP64 probe reports it; argument checks come first."""
    import ctypes as C
    from c2a_gb300 import api

    f, a = C.c_double(), C.c_double()
    assert lib.c2a_probe_fp64_peak(0, 1, C.byref(f), C.byref(a)) == api.ERR_NO_DEVICE
    assert lib.c2a_probe_fp64_peak(0, 0, C.byref(f), C.byref(a)) == api.ERR_INVALID_ARGUMENT
    assert lib.c2a_probe_fp64_peak(0, 1, None, C.byref(a)) == api.ERR_INVALID_ARGUMENT
    with api.Context(-1) as ctx:
        assert lib.c2a_collide_batch(ctx.h, None, 1, 3, 4, None, None) == api.ERR_INVALID_ARGUMENT  # flag 3
        assert lib.c2a_tolerance_batch(ctx.h, None, 1, None, None) == api.ERR_INVALID_ARGUMENT
        assert lib.c2a_tolerance_batch(ctx.h, None, 0, None, None) == api.ERR_NO_DEVICE
