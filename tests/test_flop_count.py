"""The per-unit FP64 flop counts of the CA kernel's roofline: the oracle
compiled with a counting double (oracle/flop_count.cpp) walks exactly the
port's traversal, and its flops per node-pair test and per leaf triangle
test on the benchmark batch are the figures bench.py multiplies by the
launch's counters."""
import numpy as np


def test_flop_counts_match_bench_figures(port):
    import bench
    from c2a_gb300 import workloads

    idx = bench.strided(65536, 256)
    wl = workloads.config2(n=65536, seed=2, device="cpu", indices=idx)
    models = port.models(wl.meshes)
    r = port.count_flops(models, wl.qint, wl.poses, wl.params)
    res, _ = port.solve_batch(models, wl.qint, wl.poses, wl.params, threads=4)
    # the counting build takes every decision the plain one takes
    assert r["num_bv_tests"] == int(res["num_bv_tests"].sum())
    assert r["num_tri_tests"] == int(res["num_tri_tests"].sum())
    ops = r["ops"]
    flops = ops[:, :4].sum(axis=1)  # add/sub, mul, div, sqrt; compares are not flops
    f_bv = flops[1] / r["num_bv_tests"]
    f_tri = flops[2] / r["num_tri_tests"]
    assert abs(f_bv / bench.F_BV - 1) < 0.02, f_bv
    assert abs(f_tri / bench.F_TRI - 1) < 0.05, f_tri
    # the node-pair and triangle tests are nearly all of the work
    assert (flops[1] + flops[2]) / flops.sum() > 0.95
    assert (ops[1, 3] > 0) and (ops[2, 2] > 0)  # square roots in the RSS tests, divisions in the triangle tests
