"""The speculative REFERENCE engine (C2A_ENGINE_SPEC: one warp per query,
node pairs tested ahead of the reference's depth-first order and the
reference's decisions replayed over them) against the golden fixtures and
the oracle port, bit for bit, through the C ABI."""
import os

import numpy as np
import pytest

from c2a_testutil import RESULT_FIELDS, describe, load_fixture, result_mismatches

pytestmark = pytest.mark.gpu

SPEC = 4


def _solve(ctx, meshes_, qint, poses, params, slots):
    ids = ctx.models(meshes_)
    q = qint.copy()
    q[:, 0] = np.asarray(ids)[qint[:, 0]]
    q[:, 1] = np.asarray(ids)[qint[:, 1]]
    return ctx.solve(q, poses, dict(params, engine=SPEC), contacts_per_query=slots)


def _against_port(ctx, port, meshes_, qint, poses, params, slots=256):
    res, con = _solve(ctx, meshes_, qint, poses, params, slots)
    pres, pcon = port.solve_batch(port.models(meshes_), qint, poses, params, threads=os.cpu_count(),
                                  contacts_per_query=slots)
    flat = np.concatenate([pcon[q][:min(slots, pres[q]["num_contact"])] for q in range(len(qint))])
    offs = np.concatenate([[0], np.cumsum(np.minimum(slots, pres["num_contact"]))])
    bad = result_mismatches(res, pres, con, flat, offs)
    assert not bad, f"{len(bad)} of {len(qint)} differ; first " + describe(res, pres, bad[0])
    return res


@pytest.mark.parametrize("name", ["config1", "mixed", "translation", "shipped_solve"])
def test_spec_matches_reference_fixture(gpu_ctx, name):
    ms, qint, poses, params, exp, econ, off = load_fixture(name)
    res, con = _solve(gpu_ctx, ms, qint, poses, params, 4096)
    fields = [f for f in RESULT_FIELDS if f != "mint"] if name == "shipped_solve" else RESULT_FIELDS
    bad = result_mismatches(res, exp, con, econ, off, fields=fields)
    assert not bad, f"{len(bad)} of {len(exp)} differ; first " + describe(res, exp, bad[0])


def test_spec_matches_port_config2(gpu_ctx, port):
    """Config 2's 40,000-triangle knots, th_ca = 1e-4 diag: 1,024 queries, every
    result field and every contact."""
    from c2a_gb300 import workloads

    wl = workloads.config2(n=1024, seed=2, device="cpu")
    res = _against_port(gpu_ctx, port, wl.meshes, wl.qint, wl.poses, wl.params)
    assert 0.05 < 1 - res["collisionfree"].mean() < 0.95


def test_spec_matches_port_config1_full(gpu_ctx, port):
    from c2a_gb300 import workloads

    wl = workloads.config1(n=1000, seed=1, device="cpu")
    _against_port(gpu_ctx, port, wl.meshes, wl.qint, wl.poses, wl.params, slots=512)


def test_spec_matches_port_mesh_families(gpu_ctx, port):
    """Icospheres, clustered soups and (3,5) knots, random seed pairs, gaps
    down to touching."""
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
    params = workloads.default_params(ms[0].bbox_diag(), 1e-3, 40)
    _against_port(gpu_ctx, port, ms, np.concatenate(qi), np.concatenate(ps), params)


def test_spec_iteration_cap_and_tiny_models(gpu_ctx, port):
    from c2a_gb300 import api, workloads

    wl = workloads.small_knots(48, seed=23, device="cpu")
    capped = dict(wl.params, max_iters=2)
    res = _against_port(gpu_ctx, port, wl.meshes, wl.qint, wl.poses, capped, slots=64)
    assert (res["status"] & api.QUERY_ITER_CAP).any()
    tiny = workloads.small_knots(32, seed=24, segments=6, around=3, device="cpu")
    _against_port(gpu_ctx, port, tiny.meshes, tiny.qint, tiny.poses, tiny.params, slots=64)
