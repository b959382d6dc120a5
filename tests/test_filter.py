"""CPU soundness of the kernels' FP32 filter (no GPU).

The traversal decides most comparisons on FP32 values v with certified
bounds e on their distance to the FP64 value the reference computes.  This
test compiles the same geometry headers for the host (tests/cpp/
filter_check.cpp, directed roundings derived exactly from double
arithmetic), walks real config-2 hierarchies, and checks that every
certified result satisfies |v - x64| <= e, that a certified "zero"
distance is exactly zero in FP64, and that the filter certifies nearly
all BV tests (an uncertified test costs an FP64 recompute on the GPU).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from c2a_gb300 import api, workloads

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fc(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fc") / "libfc.so")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-DC2A_EF_WHERE",
           "-Wno-unknown-pragmas", "-fPIC", "-shared", "-o", out, os.path.join(HERE, "cpp", "filter_check.cpp")]
    subprocess.run(cmd, check=True)
    lib = C.CDLL(out)
    vp = C.c_void_p
    lib.c2a_fc_bv.argtypes = [vp, vp, vp, vp, C.c_int, vp, vp, vp]
    lib.c2a_fc_tri.argtypes = [vp, vp, vp, vp, vp]
    return lib


def _p(a):
    return np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)


def _walk(fc, mesh, poses, walks, rng):
    ctx = api.Context(-1)
    mid = ctx.model(mesh)
    f, fch, tv, _, _ = ctx.download(mid)
    out = np.zeros(16)
    rec = {"bv": 0, "bv_ok": 0, "bv_lane_ok": 0, "tri": 0, "tri_ok": 0, "viol": []}
    for P in poses:
        R1, T1 = P[0:9].reshape(3, 3), P[9:12]
        R2, T2 = P[24:33].reshape(3, 3), P[33:36]
        Rm, Tm = R1.T @ R2, R1.T @ (T2 - T1)
        Ra, Tra = f[0, 0:9].reshape(3, 3), f[0, 9:12]
        for _ in range(walks):
            R = Ra.T @ (Rm @ Ra)
            T = Ra.T @ ((Rm @ Tra + Tm) - Tra)
            i = j = 0
            while True:
                li, lj = fch[i] < 0, fch[j] < 0
                if li and lj:
                    fc.c2a_fc_tri(_p(tv[-fch[i] - 1]), _p(tv[-fch[j] - 1]), _p(Rm.ravel()), _p(Tm), _p(out))
                    rec["tri"] += 1
                    if out[3] == 1:
                        rec["tri_ok"] += 1
                        if abs(out[1] - out[0]) > out[2]:
                            rec["viol"].append(("tri", out.copy()))
                    break
                side = 0 if (lj or (not li and rng.random() < 0.5)) else 1
                kids = []
                for k in (0, 1):
                    ci, cj = (fch[i] + k, j) if side == 0 else (i, fch[j] + k)
                    fc.c2a_fc_bv(_p(R.ravel()), _p(T), _p(f[ci]), _p(f[cj]), side, _p(P), _p(R1.ravel()), _p(out))
                    rec["bv"] += 1
                    if out[6] == 1:
                        rec["bv_ok"] += 1
                        if out[8] == 1:
                            if out[0] != 0.0:
                                rec["viol"].append(("zero", out.copy()))
                        elif abs(out[2] - out[0]) > out[3] or (
                                np.isfinite(out[1]) and abs(out[4] - out[1]) > out[5]):
                            rec["viol"].append(("bv", out.copy()))
                    if out[11] == 1:  # the one-lane RectDist of the speculative engine
                        rec["bv_lane_ok"] += 1
                        if out[12] == 1:
                            if out[0] != 0.0:
                                rec["viol"].append(("lane zero", out.copy()))
                        elif abs(out[9] - out[0]) > out[10]:
                            rec["viol"].append(("lane", out.copy()))
                    kids.append((out[0], ci, cj))
                k = 0 if kids[0][0] <= kids[1][0] else 1
                if rng.random() < 0.3:
                    k = 1 - k
                _, ci, cj = kids[k]
                if side == 0:
                    Rc, Trc = f[ci, 0:9].reshape(3, 3), f[ci, 9:12]
                    R, T = Rc.T @ R, Rc.T @ (T - Trc)
                else:
                    Rc, Trc = f[cj, 0:9].reshape(3, 3), f[cj, 9:12]
                    R, T = R @ Rc, R @ Trc + T
                i, j = ci, cj
    return rec


def test_filter_bounds_hold_config2(fc):
    wl = workloads.config2(n=65536, seed=2, subset=6)
    rec = _walk(fc, wl.meshes[0], wl.poses, 12, np.random.default_rng(5))
    assert not rec["viol"], rec["viol"][:3]
    assert rec["bv"] > 2000 and rec["tri"] > 50
    assert rec["bv_ok"] >= 0.99 * rec["bv"], rec
    assert rec["bv_lane_ok"] >= 0.99 * rec["bv"], rec
    assert rec["tri_ok"] >= 0.3 * rec["tri"], rec


def test_filter_bounds_hold_small_knots(fc):
    wl = workloads.small_knots(24, seed=11)
    rec = _walk(fc, wl.meshes[0], wl.poses, 8, np.random.default_rng(6))
    assert not rec["viol"], rec["viol"][:3]
    assert rec["bv_ok"] >= 0.95 * rec["bv"], rec


def test_rect_cases_lane_parallel_match_sequential(fc):
    """rect_cases.cuh (C2ARectDist's 16 cases evaluated independently, the
    first that holds wins, else the face-separation tail) and rect_table.cuh
    (the same with the shared sums spread over lanes and the operands read
    through tables) against the sequential rect_dist and the reference's own
    RectDist outputs, bit for bit."""
    from c2a_testutil import GOLDEN

    fc.c2a_fc_rect_lanes.argtypes = [C.c_void_p] * 5
    fc.c2a_fc_rect_table.argtypes = [C.c_void_p] * 5
    z = np.load(os.path.join(GOLDEN, "geometry_ref.npz"))
    out = np.zeros(9)
    tab = np.zeros(5)
    for i in range(len(z["rect_d"])):
        fc.c2a_fc_rect_lanes(_p(z["Rab"][i]), _p(z["Tab"][i]), _p(z["a"][i]), _p(z["b"][i]), _p(out))
        fc.c2a_fc_rect_table(_p(z["Rab"][i]), _p(z["Tab"][i]), _p(z["a"][i]), _p(z["b"][i]), _p(tab))
        assert out[4].tobytes() == np.float64(z["rect_d"][i]).tobytes(), i
        assert out[0].tobytes() == out[4].tobytes() and out[1:4].tobytes() == out[5:8].tobytes(), i
        assert tab[:4].tobytes() == out[4:8].tobytes() and tab[4] == out[8], i
    rng = np.random.default_rng(7)
    Rs = workloads.random_rotations(rng, 20000).reshape(-1, 9)
    cases = set()
    for i in range(20000):
        R = Rs[i] if i % 5 else np.round(Rs[i] * 2) / 2  # also near-axis-aligned, degenerate frames
        T = rng.normal(size=3) * rng.choice([0.01, 0.3, 2.0])
        a = rng.uniform(0, 1, 2) * (rng.random(2) > 0.05)
        b = rng.uniform(0, 1, 2) * (rng.random(2) > 0.05)
        fc.c2a_fc_rect_lanes(_p(R), _p(T), _p(a), _p(b), _p(out))
        fc.c2a_fc_rect_table(_p(R), _p(T), _p(a), _p(b), _p(tab))
        assert out[0].tobytes() == out[4].tobytes() and out[1:4].tobytes() == out[5:8].tobytes(), i
        assert tab[:4].tobytes() == out[4:8].tobytes() and tab[4] == out[8], i
        cases.add(int(out[8]))
    assert cases == set(range(-1, 16)), sorted(cases)


def test_rect_dist_one_lane_matches_sequential(fc):
    """rect_dist_lane (the speculative engine's RectDist: the cases in order
    through one code path) against the sequential rect_dist and the
    reference's RectDist outputs, bit for bit, over every case and the tail."""
    from c2a_testutil import GOLDEN

    fc.c2a_fc_rect_one_lane.argtypes = [C.c_void_p] * 5
    z = np.load(os.path.join(GOLDEN, "geometry_ref.npz"))
    out = np.zeros(8)
    for i in range(len(z["rect_d"])):
        fc.c2a_fc_rect_one_lane(_p(z["Rab"][i]), _p(z["Tab"][i]), _p(z["a"][i]), _p(z["b"][i]), _p(out))
        assert out[4].tobytes() == np.float64(z["rect_d"][i]).tobytes(), i
        assert out[0:4].tobytes() == out[4:8].tobytes(), i
    rng = np.random.default_rng(8)
    Rs = workloads.random_rotations(rng, 20000).reshape(-1, 9)
    for i in range(20000):
        R = Rs[i] if i % 5 else np.round(Rs[i] * 2) / 2
        T = rng.normal(size=3) * rng.choice([0.01, 0.3, 2.0])
        a = rng.uniform(0, 1, 2) * (rng.random(2) > 0.05)
        b = rng.uniform(0, 1, 2) * (rng.random(2) > 0.05)
        fc.c2a_fc_rect_one_lane(_p(R), _p(T), _p(a), _p(b), _p(out))
        assert out[0:4].tobytes() == out[4:8].tobytes(), i
