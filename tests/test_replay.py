"""The demo-scene replay (c2a_gb300/replay.py): the `.ani` reader against
the reference reader's layout (CCDDemo/mainTorusknot.cpp:565-598), the
per-frame query construction of cb_display (207-325), and the replayed
frames on the GPU against the oracle port."""
import os

import numpy as np
import pytest

from c2a_testutil import RESULT_FIELDS, bits
from c2a_gb300 import meshes, replay


def test_ani_layout_and_roundtrip(tmp_path):
    p = tmp_path / "a.ani"
    p.write_text("2f\n0f\n1 2 3 4 5 6 7 8 9\n-300.0 0.0 0.5\n1f\n1 0 0 0 1 0 0 0 1\n0.25 0.5 0.75\n")
    R, T = replay.read_ani(str(p))
    assert R.shape == (2, 3, 3)
    # the reader fills R[0][0], R[1][0], R[2][0], R[0][1], ...: the file lists columns
    assert np.array_equal(R[0], np.array([[1, 4, 7], [2, 5, 8], [3, 6, 9.0]]))
    assert np.array_equal(T[0], [-300.0, 0.0, 0.5]) and np.array_equal(R[1], np.eye(3))
    q = tmp_path / "b.ani"
    replay.write_ani(str(q), R, T)
    R2, T2 = replay.read_ani(str(q))
    assert np.array_equal(R, R2) and np.array_equal(T, T2)


def test_demo_frame_steps_and_queries():
    assert replay.demo_steps(0) == (0, 1, 0) and replay.demo_steps(100) == (0, 1, 100)
    assert replay.demo_steps(101) == (101, 102, 101) and replay.demo_steps(202) == (202, 203, 202)
    a0, a1 = replay.synthetic_scene(12)
    qint, poses = replay.demo_queries(a0, a1, seeds=(3, 5))
    assert qint.shape == (12, 4) and (qint[:, 2] == 3).all() and (qint[:, 3] == 5).all()
    per = np.arange(24, dtype=np.int32).reshape(12, 2)
    assert np.array_equal(replay.demo_queries(a0, a1, seeds=per)[0][:, 2:4], per)
    i = 7
    assert np.array_equal(poses[i, 0:9], a0[0][0].reshape(9)) and np.array_equal(poses[i, 12:21], a0[0][1].reshape(9))
    assert np.array_equal(poses[i, 24:33], a1[0][i].reshape(9)) and np.array_equal(poses[i, 36:45], a1[0][i].reshape(9))
    assert np.array_equal(poses[i, 33:36], a1[1][0]) and np.array_equal(poses[i, 45:48], a1[1][1])


def test_demo_replay_runs_on_the_oracle(port):
    knot = meshes.torus_knot(2, 3, 40, 8)
    a0, a1 = replay.synthetic_scene(30)
    qint, poses = replay.demo_queries(a0, a1)
    res, _ = port.solve_batch(port.models([knot, knot]), qint, poses, replay.demo_params(), threads=4)
    assert (res["translation"] == 0).all() and (res["numCA"] >= 1).all()
    assert (res["collisionfree"] == 0).all()  # object 0 sweeps through object 1 in every frame


@pytest.mark.gpu
def test_gpu_demo_replay_matches_port(gpu_ctx, port):
    knot = meshes.torus_knot(2, 3, 100, 16, 1.0, 0.15)
    a0, a1 = replay.synthetic_scene(60, seed=4)
    qint, poses = replay.demo_queries(a0, a1)
    ids = gpu_ctx.models([knot, knot])
    q = qint.copy()
    q[:, 0], q[:, 1] = ids
    res, con = gpu_ctx.solve(q, poses, replay.demo_params(), contacts_per_query=256)
    pres, pcon = port.solve_batch(port.models([knot, knot]), qint, poses, replay.demo_params(), threads=4,
                                  contacts_per_query=256)
    for f in RESULT_FIELDS:
        assert bits(res[f]) == bits(pres[f]), f
    for i in range(len(q)):
        n = min(int(pres[i]["num_contact"]), 256)
        assert bits(con[i]["tri_a"]) == bits(pcon[i][:n]["tri_a"]) and bits(con[i]["pa"]) == bits(pcon[i][:n]["pa"])


def _demo_scene():
    from c2a_testutil import GOLDEN

    z = np.load(f"{GOLDEN}/demo_scene_ref.npz")
    bunny = meshes.Mesh("bunny_noholes", z["verts_micro"] / 1e6, z["faces"], np.zeros((1, 3)), 0.0)
    return bunny, z


def _check_demo(res, con, z):
    """Every field and contact bit for bit; mint on collision-free frames only:
    the shipped C2A_Solve leaves the contact query's reset value 1 there
    (C2A.cpp:1757)."""
    from c2a_testutil import RESULT_FIELDS as F, result_mismatches

    exp = z["results"]
    bad = result_mismatches(res, exp, con, z["contacts"], z["contact_offsets"], fields=[f for f in F if f != "mint"])
    assert not bad, bad[:10]
    free = exp["collisionfree"] == 1
    assert bits(res["mint"][free]) == bits(exp["mint"][free]) and (exp["mint"][~free] == 1.0).all()


def test_shipped_demo_scene_on_the_oracle(port):
    """The shipped scene (bunny against bunny, torusknot1/2.ani, 303 frames) on
    the oracle port against the reference's own per-frame results and
    contacts, with the seeds the demo's last_tri chain gave each frame."""
    bunny, z = _demo_scene()
    assert bunny.num_tris == 69664
    assert z["poses"].shape == (303, 48) and z["qint"].shape == (303, 4)
    res, con = port.solve_batch(port.models([bunny, bunny]), z["qint"], z["poses"], replay.demo_params(), threads=8,
                                contacts_per_query=128)
    _check_demo(res, con, z)
    assert (z["results"]["collisionfree"] == 0).sum() > 100


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ["auto", "thread", "spec"])
def test_gpu_shipped_demo_scene_matches_reference(gpu_ctx, engine):
    """Every frame of the shipped scene on the GPU through c2a_solve_batch:
    every result field and every contact bit for bit as the reference
    computed them."""
    from c2a_gb300 import api

    bunny, z = _demo_scene()
    ids = gpu_ctx.models([bunny, bunny])
    q = z["qint"].copy()
    q[:, 0], q[:, 1] = ids
    prm = dict(replay.demo_params(), engine={"auto": api.ENGINE_AUTO, "thread": api.ENGINE_THREAD,
                                             "spec": api.ENGINE_SPEC}[engine])
    res, con = gpu_ctx.solve(q, z["poses"], prm, contacts_per_query=128)
    _check_demo(res, [con[i] for i in range(len(q))], z)
    assert (res["status"] == 0).all()
