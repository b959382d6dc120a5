"""c2a_solve_batch_noalloc: the entry point for callers that may not allocate
device memory at query time (an engine or simulator that owns the device
memory budget and forbids cudaMalloc after start-up, or a real-time loop
that cannot afford cudaMalloc/cudaFree's implicit synchronisation).  Its
kernel keeps its scratch in the library's fixed device array; the results
must equal those of the allocating device entry point, call after call.

Collected last on purpose; it creates its own context and buffers so it also
passes alone in a fresh process."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SLOTS = 64


def _run(fn, ctx, d_q, n, params, torch):
    from c2a_gb300 import api

    d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(n * SLOTS * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    fn(d_q.data_ptr(), n, params, d_r.data_ptr(), d_c.data_ptr(), SLOTS, stream=s.cuda_stream)
    s.synchronize()
    return d_r.cpu().numpy().view(api.RESULT_DTYPE), d_c.cpu().numpy().view(api.CONTACT_DTYPE)


def test_noalloc_matches_device_entry_on_two_consecutive_calls():
    import torch
    from c2a_gb300 import api, build, workloads

    build.build()
    assert torch.cuda.is_available()
    wl = workloads.small_knots(96, seed=31)
    with api.Context(0) as ctx:
        mid = ctx.model(wl.meshes[0])
        q = wl.qint.copy()
        q[:, :2] = mid
        d_q = torch.from_numpy(api.make_queries(q, wl.poses).view(np.uint8).copy()).cuda()
        ref_r, ref_c = _run(ctx.solve_device, ctx, d_q, wl.n, wl.params, torch)
        assert (ref_r["status"] & ~(api.QUERY_ITER_CAP | api.QUERY_CONTACT_OVERFLOW) == 0).all()
        for call in range(2):
            r, c = _run(ctx.solve_noalloc, ctx, d_q, wl.n, wl.params, torch)
            # bit-exact: the tolerance every parity test of this library uses
            for f in ("status", "collisionfree", "numCA", "toc", "distance", "mint", "num_bv_tests",
                      "num_tri_tests", "num_contact", "R_toc", "T_toc", "contact_offset"):
                assert r[f].tobytes() == ref_r[f].tobytes(), (call, f)
            for i in range(wl.n):
                k = min(int(ref_r[i]["num_contact"]), SLOTS)
                a = c[i * SLOTS:i * SLOTS + k]
                b = ref_c[i * SLOTS:i * SLOTS + k]
                assert a.tobytes() == b.tobytes(), (call, i)
        assert (1 - ref_r["collisionfree"]).sum() > 0 and ref_r["num_contact"].sum() > 0
