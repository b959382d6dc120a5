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
    assert qint.shape == (11, 4) and (qint[:, 2] == 3).all() and (qint[:, 3] == 5).all()
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
