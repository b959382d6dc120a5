"""The warp-per-query REFERENCE engines' device code on the CPU: 32 host
threads emulate one warp (tests/cpp/warp_emu.h), so the speculative engine's
replay, speculation and record bookkeeping -- and the sequential warp
traversal it must agree with -- run here against the golden fixtures and the
oracle port, bit for bit.  A warp collective reached by only some lanes
aborts the emulation."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from c2a_testutil import describe, load_fixture, result_mismatches

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
WARP, SPEC = 1, 4
SLOTS = 512


def _build_emu(tmp_path_factory, name, defines=(), flags=()):
    out = str(tmp_path_factory.mktemp(name) / f"lib{name}.so")
    subprocess.run(["g++", "-std=c++20", "-O1", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
                    "-w", *flags, *[f"-D{d}" for d in defines], "-o", out,
                    os.path.join(ROOT, "tests", "cpp", "spec_emu.cpp"),
                    os.path.join(ROOT, "c2a_gb300", "csrc", "host", "bvh_build.cpp")], check=True)
    return out


@pytest.fixture(scope="module")
def emu_filter(tmp_path_factory):
    """the warp engine with its node-pair tests in the certified FP32 filter
    (the half-warp table form, C2A_WARP_FILTER=2)"""
    lib = C.CDLL(_build_emu(tmp_path_factory, "emu_filter", ("C2A_WARP_FILTER=2",)))
    lib.spec_emu_model.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    lib.spec_emu_solve.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
    return lib


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    out = _build_emu(tmp_path_factory, "emu")
    lib = C.CDLL(out)
    lib.spec_emu_model.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    lib.spec_emu_solve.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
    return lib


def _run(lib, meshes_, qint, poses, params, engine):
    from c2a_gb300 import api

    lib.spec_emu_reset()
    ids = []
    for m in meshes_:
        tv = np.ascontiguousarray(m.tri_verts())
        vidx = np.ascontiguousarray(m.faces, dtype=np.int32)
        ids.append(lib.spec_emu_model(m.num_tris, tv.ctypes.data, vidx.ctypes.data))
    q = qint.copy()
    q[:, 0] = np.asarray(ids)[qint[:, 0]]
    q[:, 1] = np.asarray(ids)[qint[:, 1]]
    qs = api.make_queries(q, poses)
    prm = api.make_params(dict(params, engine=engine), SLOTS)
    n = len(q)
    res = np.zeros(n, dtype=api.RESULT_DTYPE)
    con = np.zeros(n * SLOTS, dtype=api.CONTACT_DTYPE)
    lib.spec_emu_solve(qs.ctypes.data, n, C.byref(prm), res.ctypes.data, con.ctypes.data, 120.0)
    return res, con.reshape(n, SLOTS)


@pytest.mark.parametrize("engine", [WARP, SPEC])
@pytest.mark.parametrize("name", ["config1", "mixed", "translation"])
def test_emulated_engine_matches_fixture(emu, name, engine):
    ms, qint, poses, params, exp, econ, off = load_fixture(name)
    sel = np.linspace(0, len(qint) - 1, 6).astype(int)
    res, con = _run(emu, ms, qint[sel], poses[sel], params, engine)
    flat = np.concatenate([econ[off[i]:off[i + 1]][:SLOTS] for i in sel])
    offs = np.concatenate([[0], np.cumsum([min(SLOTS, off[i + 1] - off[i]) for i in sel])])
    bad = result_mismatches(res, exp[sel], con, flat, offs)
    assert not bad, f"engine {engine}: " + describe(res, exp[sel], bad[0])


def test_emulated_spec_matches_port_small_models(emu, port):
    """Small knots (many leaves per round), an iteration cap, and tiny models."""
    from c2a_gb300 import workloads

    for wl, prm in ((workloads.small_knots(10, seed=41, device="cpu"), None),
                    (workloads.small_knots(6, seed=42, device="cpu"), {"max_iters": 2}),
                    (workloads.small_knots(6, seed=43, segments=4, around=3, device="cpu"), None)):
        params = dict(wl.params, **(prm or {}))
        res, con = _run(emu, wl.meshes, wl.qint, wl.poses, params, SPEC)
        pres, pcon = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, params, contacts_per_query=SLOTS)
        flat = np.concatenate([pcon[q][:min(SLOTS, pres[q]["num_contact"])] for q in range(wl.n)])
        offs = np.concatenate([[0], np.cumsum(np.minimum(SLOTS, pres["num_contact"]))])
        bad = result_mismatches(res, pres, con, flat, offs)
        assert not bad, describe(res, pres, bad[0])


@pytest.mark.parametrize("name", ["config1", "mixed"])
def test_emulated_filtered_warp_engine_matches_fixture(emu_filter, name):
    """The filtered warp engine decides most node pairs from certified FP32
    intervals and recomputes the rest in FP64: the reference's bits."""
    ms, qint, poses, params, exp, econ, off = load_fixture(name)
    sel = np.linspace(0, len(qint) - 1, 6).astype(int)
    res, con = _run(emu_filter, ms, qint[sel], poses[sel], params, WARP)
    flat = np.concatenate([econ[off[i]:off[i + 1]][:SLOTS] for i in sel])
    offs = np.concatenate([[0], np.cumsum([min(SLOTS, off[i + 1] - off[i]) for i in sel])])
    bad = result_mismatches(res, exp[sel], con, flat, offs)
    assert not bad, describe(res, exp[sel], bad[0])


def test_emulated_engines_under_address_sanitizer(tmp_path_factory):
    """The warp and speculative engines' device source on the host emulator,
    built with AddressSanitizer + UBSan and run in a child process with the
    sanitizer runtime preloaded: fixture queries run without a report and
    give the reference's bits."""
    import sys

    asan = subprocess.run(["g++", "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not os.path.isabs(asan) or not os.path.exists(asan):
        pytest.skip("no AddressSanitizer runtime")
    lib = _build_emu(tmp_path_factory, "emu_asan",
                     flags=("-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined", "-fno-sanitize-recover=all"))
    tests_dir = os.path.join(ROOT, "tests")
    script = f"""
import ctypes as C, sys
import numpy as np
sys.path[:0] = [{tests_dir!r}, {ROOT!r}]
import test_spec_emu as t
from c2a_testutil import load_fixture, result_mismatches
lib = C.CDLL({lib!r})
lib.spec_emu_model.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
lib.spec_emu_solve.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]
for name in ("mixed", "translation"):
    ms, qint, poses, params, exp, econ, off = load_fixture(name)
    sel = np.linspace(0, len(qint) - 1, 4).astype(int)
    flat = np.concatenate([econ[off[i]:off[i + 1]][:t.SLOTS] for i in sel])
    offs = np.concatenate([[0], np.cumsum([min(t.SLOTS, off[i + 1] - off[i]) for i in sel])])
    for engine in (t.WARP, t.SPEC):
        res, con = t._run(lib, ms, qint[sel], poses[sel], params, engine)
        assert not result_mismatches(res, exp[sel], con, flat, offs), (name, engine)
print("clean")
"""
    env = dict(os.environ, LD_PRELOAD=asan, ASAN_OPTIONS="detect_leaks=0:halt_on_error=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0 and "clean" in r.stdout, r.stdout[-2000:] + r.stderr[-6000:]
