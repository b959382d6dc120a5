"""c2a_solve_batch_noalloc: the entry point for callers that may not allocate
device memory at query time (an engine or simulator that owns the device
memory budget and forbids cudaMalloc after start-up, or a real-time loop
that cannot afford cudaMalloc/cudaFree's implicit synchronisation).  Its
kernel keeps its scratch in the library's fixed device array; the results
must equal those of the allocating device entry point and of the CPU oracle,
call after call, and a call must not change the device's free memory.

Collected last on purpose; it creates its own context and buffers so it also
passes alone in a fresh process."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SLOTS = 64
FIELDS = ("collisionfree", "numCA", "toc", "distance", "mint", "num_bv_tests", "num_tri_tests", "num_contact")


def _buffers(n, torch):
    from c2a_gb300 import api

    d_r = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    d_c = torch.zeros(n * SLOTS * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    return d_r, d_c


def _run(fn, d_q, n, params, bufs, stream):
    from c2a_gb300 import api

    d_r, d_c = bufs
    d_r.zero_()
    d_c.zero_()
    fn(d_q.data_ptr(), n, params, d_r.data_ptr(), d_c.data_ptr(), SLOTS, stream=stream.cuda_stream)
    stream.synchronize()
    return d_r.cpu().numpy().view(api.RESULT_DTYPE).copy(), d_c.cpu().numpy().view(api.CONTACT_DTYPE).copy()


def test_noalloc_matches_device_entry_and_oracle_on_two_consecutive_calls():
    import torch
    from c2a_gb300 import api, build, workloads
    from oracle.oracle import Port

    build.build()
    assert torch.cuda.is_available()
    wl = workloads.small_knots(96, seed=31, device="cpu")
    port = Port()
    pres, pcon = port.solve_batch(port.models(wl.meshes), wl.qint, wl.poses, wl.params, contacts_per_query=SLOTS)
    with api.Context(0) as ctx:
        mid = ctx.model(wl.meshes[0])
        q = wl.qint.copy()
        q[:, :2] = mid
        d_q = torch.from_numpy(api.make_queries(q, wl.poses).view(np.uint8).copy()).cuda()
        s = torch.cuda.Stream()
        ref_r, ref_c = _run(ctx.solve_device, d_q, wl.n, wl.params, _buffers(wl.n, torch), s)
        assert (ref_r["status"] & ~(api.QUERY_ITER_CAP | api.QUERY_CONTACT_OVERFLOW) == 0).all()
        bufs = _buffers(wl.n, torch)
        for call in range(2):
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            r, c = _run(ctx.solve_noalloc, d_q, wl.n, wl.params, bufs, s)
            torch.cuda.synchronize()
            if call == 1:  # the first call may upload the model table; neither allocates
                assert torch.cuda.mem_get_info()[0] == free_before
            # bit-exact: the tolerance every parity test of this library uses
            for f in FIELDS + ("status", "R_toc", "T_toc", "contact_offset"):
                assert r[f].tobytes() == ref_r[f].tobytes(), (call, f)
            for f in FIELDS:
                assert r[f].tobytes() == pres[f].tobytes(), (call, "oracle", f)
            for i in range(wl.n):
                k = min(int(ref_r[i]["num_contact"]), SLOTS)
                a = c[i * SLOTS:i * SLOTS + k]
                b = ref_c[i * SLOTS:i * SLOTS + k]
                assert a.tobytes() == b.tobytes(), (call, i)
                for f in ("tri_a", "tri_b", "distance", "pa", "pb"):
                    assert a[f].tobytes() == pcon[i][:k][f].tobytes(), (call, "oracle", i, f)
        assert (1 - ref_r["collisionfree"]).sum() > 0 and ref_r["num_contact"].sum() > 0


def test_noalloc_rejects_canonical_mode_and_too_many_models():
    import torch
    from c2a_gb300 import api, workloads

    wl = workloads.small_knots(4, seed=32, segments=8, around=4, device="cpu")
    with api.Context(0) as ctx:
        mid = ctx.model(wl.meshes[0])
        q = wl.qint.copy()
        q[:, :2] = mid
        d_q = torch.from_numpy(api.make_queries(q, wl.poses).view(np.uint8).copy()).cuda()
        bufs = _buffers(wl.n, torch)
        s = torch.cuda.Stream()
        with pytest.raises(api.C2AError) as e:
            _run(ctx.solve_noalloc, d_q, wl.n, dict(wl.params, mode=api.MODE_CANONICAL), bufs, s)
        assert e.value.status == api.ERR_INVALID_ARGUMENT
        for _ in range(api.NOALLOC_MAX_MODELS):  # 121 models in all
            ctx.model(wl.meshes[0])
        with pytest.raises(api.C2AError) as e:
            _run(ctx.solve_noalloc, d_q, wl.n, wl.params, bufs, s)
        assert e.value.status == api.ERR_NOALLOC_CAPACITY
