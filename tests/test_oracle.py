"""The CPU oracle pinned against the reference.

The reference has no tests and no stored outputs, so its known answers are
produced by running the reference's own C2A sources (tests/golden/
make_golden.py); these tests check the plain-C oracle port against those
fixtures bit for bit, and against the live reference where it is compiled.
"""
import ctypes as C

import numpy as np
import pytest

from c2a_testutil import GOLDEN, RESULT_FIELDS, bits, describe, load_fixture, result_mismatches


@pytest.mark.parametrize("name", ["config1", "mixed", "translation"])
def test_port_matches_reference_fixture(port, name):
    ms, qint, poses, params, exp, econ, off = load_fixture(name)
    models = port.models(ms)
    res, con = port.solve_batch(models, qint, poses, params, threads=4, contacts_per_query=4096)
    bad = result_mismatches(res, exp, con, econ, off)
    assert not bad, f"{len(bad)} of {len(exp)} queries differ; first " + describe(res, exp, bad[0])


def test_port_matches_shipped_c2a_solve(port):
    """C2A_Solve as shipped: th_ca ignored, 1e-4 tolerances (C2A.cpp:2384-2388).
    Its dres.mint is the contact query's reset value 1 when a contact was
    found (C2A.cpp:1757), so mint is compared on collision-free queries only."""
    ms, qint, poses, params, exp, econ, off = load_fixture("shipped_solve")
    models = port.models(ms)
    res, con = port.solve_batch(models, qint, poses, params, threads=4, contacts_per_query=4096)
    fields = [f for f in RESULT_FIELDS if f != "mint"]
    bad = result_mismatches(res, exp, con, econ, off, fields=fields)
    assert not bad, describe(res, exp, bad[0])
    free = exp["collisionfree"] == 1
    assert bits(res["mint"][free]) == bits(exp["mint"][free])
    assert np.all(exp["mint"][~free] == 1.0)


def test_fixture_coverage():
    """The fixtures exercise both outcomes, contacts, the translation-only CA,
    several mesh families and non-default seeds."""
    _, qint, _, _, exp, econ, _ = load_fixture("mixed")
    assert 0 < exp["collisionfree"].sum() < len(exp)
    assert len(econ) > 100 and set(np.unique(econ["type_a"])) >= {1, 2}
    assert (qint[:, 2] != 0).any() and (qint[:, 1] == 1).any()
    _, _, _, _, t, _, _ = load_fixture("translation")
    assert t["translation"].all() and 0 < t["collisionfree"].sum() < len(t)


def test_port_rect_and_triangle_distance(port):
    z = np.load(f"{GOLDEN}/geometry_ref.npz")
    for i in range(len(z["rect_d"])):
        d, P, Q, S = port.rectdist(z["Rab"][i], z["Tab"][i], z["a"][i], z["b"][i])
        assert bits(d) == bits(z["rect_d"][i]), i
        if d > 0:
            assert bits(S) == bits(z["rect_S"][i]), i
    for i in range(len(z["tri_d"])):
        d, P, Q, f = port.tridist(z["S9"][i], z["T9"][i])
        assert bits(d) == bits(z["tri_d"][i]), i
        assert f == tuple(int(x) for x in z["tri_f"][i]), i
        if d > 0:
            assert bits(P) == bits(z["tri_P"][i]) and bits(Q) == bits(z["tri_Q"][i]), i
    assert (z["tri_d"] == 0).sum() > 5 and (z["rect_d"] == 0).sum() > 5


def test_port_bvh_matches_reference(port):
    from c2a_gb300 import meshes

    z = np.load(f"{GOLDEN}/bvh_icosphere1_ref.npz")
    m = meshes.Mesh("ico1", z["verts"], z["faces"], np.zeros((1, 3)), 0.0)
    nodes, tris = port.dump(port.models([m]), 0)
    f = np.concatenate([nodes["R"], nodes["Tr"], nodes["l"], nodes["r"][:, None], nodes["angR"][:, None],
                        nodes["Rloc"]], axis=1)
    assert bits(f) == bits(z["node_f"])
    assert np.array_equal(nodes["first_child"], z["first_child"])
    assert bits(tris["v"]) == bits(z["tri_v"]) and np.array_equal(tris["idx"], z["tri_idx"])


def test_deterministic_math_is_correctly_rounded(port):
    """sin/cos/acos of the motion model (InterpMotion.cpp:251, 275-278) against
    200-bit mpmath: the double-double evaluation rounds correctly."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    L = port.lib
    for fn in ("c2a_port_det_sin", "c2a_port_det_cos", "c2a_port_det_acos"):
        getattr(L, fn).argtypes = [C.c_double]
        getattr(L, fn).restype = C.c_double
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(0, np.pi / 2, 3000), [0.0, 1e-300, 1e-9, np.pi / 4, np.pi / 2]])
    for x in xs:
        assert L.c2a_port_det_sin(float(x)) == float(mpmath.sin(mpmath.mpf(float(x)))), x
        assert L.c2a_port_det_cos(float(x)) == float(mpmath.cos(mpmath.mpf(float(x)))), x
    ys = np.concatenate([rng.uniform(-1, 1, 3000), [-1.0, 1.0, 0.0, 1 - 2 ** -53, -1 + 2 ** -53]])
    for y in ys:
        assert L.c2a_port_det_acos(float(y)) == float(mpmath.acos(mpmath.mpf(float(y)))), y
    assert np.isnan(L.c2a_port_det_acos(1.0000000000000002))


def test_port_matches_live_reference(port, ref):
    """Fresh random queries (random seed pairs, gaps down to contact) against
    the reference compiled here."""
    from c2a_gb300 import meshes, workloads
    import contextlib, io

    knot = meshes.torus_knot(3, 5, 40, 8)
    qint, poses = workloads.ccd_queries(knot, knot, 48, 777, gap_range=(0.0, 0.8), device="cpu", model_a=0,
                                        model_b=0)
    rng = np.random.default_rng(5)
    qint[:, 2] = rng.integers(0, knot.num_tris, len(qint))
    qint[:, 3] = rng.integers(0, knot.num_tris, len(qint))
    params = workloads.default_params(knot.bbox_diag(), 1e-3, 40)
    res, con = port.solve_batch(port.models([knot]), qint, poses, params, contacts_per_query=4096)
    h = ref.model(knot)
    for q in range(len(qint)):
        r, c = ref.solve(h, h, poses[q], int(qint[q, 2]), int(qint[q, 3]), params)
        for f in RESULT_FIELDS:
            assert bits(res[q][f]) == bits(r[f]), (q, f)
        n = int(r["num_contact"])
        assert bits(con[q][:n]) == bits(np.ascontiguousarray(c[::-1])), q


def test_port_tolerance_matches_reference(port, ref):
    """C2A_Tolerance (qsize 2), C2A/src/C2A_PQP.cpp:1498-1603, 1762-1845: the
    port against the compiled reference on a knot, a soup and an icosphere,
    with tolerances below, around and above each pair's exact distance --
    the flag, the counters and, where a pair is found, its distance and
    points, bit for bit."""
    from c2a_gb300 import meshes, workloads

    ms = [meshes.torus_knot(2, 3, 40, 8), meshes.triangle_soup(600, clusters=5, seed=71),
          meshes.icosphere(2, radius=0.8, noise=0.02, seed=72)]
    models = port.models(ms)
    ha = [ref.model(m) for m in ms]
    hb = [ref.model(m) for m in ms]
    rng = np.random.default_rng(73)
    found = 0
    for k in range(120):
        a, b = rng.integers(0, 3, 2)
        R = workloads.random_rotations(rng, 1).reshape(9)
        T = workloads.unit_vectors(rng, 1)[0] * rng.uniform(0.5, 3.0) + rng.normal(scale=1e-3, size=3)
        d, _, _ = port.distance(models, a, b, R, T, 0, 0)
        tol = d * rng.choice([0.5, 0.999, 1.0, 1.001, 2.0]) if d > 0 else rng.uniform(0, 0.1)
        got = port.tolerance(models, a, b, R, T, tol)
        exp = ref.tolerance(ha[a], hb[b], R, T, tol)
        assert got[0] == exp[0] and got[4:] == exp[4:], (k, got, exp)
        if exp[0]:
            found += 1
            assert bits(got[1]) == bits(exp[1]) and bits(got[2]) == bits(exp[2]) and bits(got[3]) == bits(exp[3]), k
    assert 30 < found < 120


def test_port_collide_matches_reference(port, ref):
    """C2A_Collide (the PQP_CollideResult form, C2A/src/C2A_PQP.cpp:798-968):
    the port against the compiled reference, both with every contact and
    with the first only -- the colliding triangle-id pairs in the order
    found and the BV/triangle counters, exactly.  The hierarchy's OBB fields
    (C2A_BV.cpp:144-170, make_parent_relative) come from the port's build."""
    from c2a_gb300 import meshes, workloads

    ms = [meshes.torus_knot(2, 3, 40, 8), meshes.triangle_soup(600, clusters=5, seed=81),
          meshes.icosphere(2, radius=0.8, noise=0.02, seed=82)]
    models = port.models(ms)
    ha = [ref.model(m) for m in ms]
    hb = [ref.model(m) for m in ms]
    rng = np.random.default_rng(83)
    hits = 0
    for k in range(80):
        a, b = rng.integers(0, 3, 2)
        R = workloads.random_rotations(rng, 1).reshape(9)
        T = workloads.unit_vectors(rng, 1)[0] * rng.uniform(0.0, 1.6) + rng.normal(scale=1e-3, size=3)
        for flag in (1, 2):
            got = port.collide(models, a, b, R, T, flag)
            exp = ref.collide(ha[a], hb[b], R, T, flag)
            assert np.array_equal(got[0], exp[0]) and got[1:] == exp[1:], (k, flag, len(got[0]), len(exp[0]),
                                                                          got[1:], exp[1:])
            if flag == 1 and len(exp[0]):
                hits += 1
                assert len(port.collide(models, a, b, R, T, 2)[0]) == 1
    assert 15 < hits < 80, hits


def test_port_static_queries_match_reference_fixture(port):
    """C2A_Tolerance and C2A_Collide of the port against the reference's own
    outputs stored in tests/golden/static_queries_ref.npz (runs where the
    reference sources are absent)."""
    from c2a_gb300 import meshes

    z = np.load(f"{GOLDEN}/static_queries_ref.npz")
    ms = [meshes.Mesh(f"s{i}", z[f"mesh{i}_verts"], z[f"mesh{i}_faces"], np.zeros((1, 3)), 0.0)
          for i in range(int(z["num_meshes"]))]
    models = port.models(ms)
    offs = z["pair_offsets"]
    for i, (a, b) in enumerate(z["ab"]):
        c, d, p1, p2, nbv, ntri = port.tolerance(models, a, b, z["R"][i], z["T"][i], z["tol"][i])
        e = z["tol_out"][i]
        assert c == z["closer"][i] and (nbv, ntri) == (int(e[7]), int(e[8])), i
        if c:
            assert bits(d) == bits(e[0]) and bits(p1) == bits(e[1:4]) and bits(p2) == bits(e[4:7]), i
        pairs, cbv, ctri = port.collide(models, a, b, z["R"][i], z["T"][i], 1)
        assert np.array_equal(pairs, z["pairs"][offs[i]:offs[i + 1]]), i
        assert (cbv, ctri) == tuple(z["collide_counts"][i]), i


def _rel(RA, TA, RB, TB):
    """B's pose in A's frame: R = RA^T RB, T = RA^T (TB - TA)."""
    RA, RB = RA.reshape(3, 3), RB.reshape(3, 3)
    return RA.T @ RB, RA.T @ (TB - TA)


def test_toc_is_never_late_and_nothing_touches_earlier(port):
    """The CA guarantee on config 1 (oracle = reference, bit for bit): where
    the CA loop reached tolerance_d, the exact distance at the returned time
    of contact is within th_ca and not negative, and at earlier times along
    both motions (a quarter, half and three quarters of the TOC) the objects
    are still apart."""
    from c2a_gb300 import api, workloads

    wl = workloads.config1(n=192, seed=7, device="cpu")
    models = port.models(wl.meshes)
    res, _ = port.solve_batch(models, wl.qint, wl.poses, wl.params, threads=4, contacts_per_query=0)
    hit = np.flatnonzero((res["collisionfree"] == 0) & (res["distance"] <= wl.params["tol_d"]) &
                         (res["numCA"] >= 2) & (res["distance"] > 0))
    assert len(hit) >= 10
    th = wl.params["th_ca"]
    for q in hit:
        r = res[q]
        R, T = _rel(r["R_toc"][0], r["T_toc"][0], r["R_toc"][1], r["T_toc"][1])
        d, _, _ = port.distance(models, 0, 0, R, T, int(r["seed_a"]), int(r["seed_b"]))
        assert 0 <= d <= th * (1 + 1e-12), (q, d, th)
        P = wl.poses[q]
        for frac in (0.25, 0.5, 0.75):
            t = frac * float(r["toc"])
            RA, TA, _ = api.motion_integrate(P[0:9], P[9:12], P[12:21], P[21:24], t)
            RB, TB, _ = api.motion_integrate(P[24:33], P[33:36], P[36:45], P[45:48], t)
            R, T = _rel(RA, TA, RB, TB)
            d_early, _, _ = port.distance(models, 0, 0, R, T, 0, 0)
            assert d_early > 0, (q, frac, d_early)
