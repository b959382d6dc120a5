"""Python binding of the C ABI (include/c2a_gb300.h) of libc2a_gb300.so.

Mirrors the reference's query interface for batches: build a model from a
triangle soup (C2A_Model::AddTri/EndModel), then run C2A_Solve-style queries
(C2A_QueryTimeOfContact + C2A_QueryContact), single CA steps
(C2A_TimeOfContactStep) or contact queries (C2A_QueryContactOnly) on the GPU.
There is no CPU fallback: without the compiled library or a CUDA device the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

QUERY_DTYPE = np.dtype([("model_a", np.int32), ("model_b", np.int32), ("seed_a", np.int32), ("seed_b", np.int32),
                        ("pose", np.float64, (48,))], align=True)
RESULT_DTYPE = np.dtype([("collisionfree", np.int32), ("numCA", np.int32), ("translation", np.int32),
                         ("num_contact", np.int32), ("toc", np.float64), ("distance", np.float64),
                         ("mint", np.float64), ("num_bv_tests", np.int64), ("num_tri_tests", np.int64),
                         ("R_toc", np.float64, (2, 9)), ("T_toc", np.float64, (2, 3)), ("seed_a", np.int32),
                         ("seed_b", np.int32), ("status", np.int32), ("contact_offset", np.int32)], align=True)
CONTACT_DTYPE = np.dtype([("type_a", np.int32), ("type_b", np.int32), ("fid_a", np.int32, (3,)),
                          ("fid_b", np.int32, (3,)), ("tri_a", np.int32), ("tri_b", np.int32),
                          ("query", np.int32), ("pad", np.int32), ("pa", np.float64, (3,)),
                          ("pb", np.float64, (3,)), ("distance", np.float64)], align=True)
DISTANCE_DTYPE = np.dtype([("distance", np.float64), ("p1", np.float64, (3,)), ("p2", np.float64, (3,)),
                           ("tri_a", np.int32), ("tri_b", np.int32), ("status", np.int32), ("pad", np.int32)],
                          align=True)
TOLERANCE_DTYPE = np.dtype([("closer", np.int32), ("status", np.int32), ("distance", np.float64),
                            ("p1", np.float64, (3,)), ("p2", np.float64, (3,)), ("num_bv_tests", np.int64),
                            ("num_tri_tests", np.int64)], align=True)
COLLIDE_DTYPE = np.dtype([("num_pairs", np.int32), ("status", np.int32), ("num_bv_tests", np.int64),
                          ("num_tri_tests", np.int64)], align=True)
assert TOLERANCE_DTYPE.itemsize == 80 and COLLIDE_DTYPE.itemsize == 24
assert QUERY_DTYPE.itemsize == 400 and RESULT_DTYPE.itemsize == 264 and CONTACT_DTYPE.itemsize == 104
assert DISTANCE_DTYPE.itemsize == 72

C2A_OK = 0
QUERY_BAD_INPUT, QUERY_STACK_OVERFLOW, QUERY_CONTACT_OVERFLOW, QUERY_ITER_CAP = 1, 2, 4, 8
(OK, ERR_INVALID_ARGUMENT, ERR_NO_DEVICE, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_EMPTY_MODEL, ERR_BAD_MODEL,
 ERR_TREE_TOO_DEEP, ERR_QUERY_FAILED, ERR_NOALLOC_CAPACITY) = range(10)
NOALLOC_MAX_MODELS = 120  # C2A_NOALLOC_MAX_MODELS

# every extern "C" symbol of include/c2a_gb300.h
ABI_SYMBOLS = ["c2a_create", "c2a_destroy", "c2a_status_str", "c2a_launch_count", "c2a_model_build",
               "c2a_model_build_many", "c2a_model_build_async", "c2a_model_wait", "c2a_model_info", "c2a_model_download", "c2a_model_download_obb", "c2a_model_free",
               "c2a_solve_batch",
               "c2a_solve_batch_device", "c2a_solve_batch_noalloc", "c2a_toc_step_batch", "c2a_contact_only_batch",
               "c2a_distance_batch", "c2a_solve_batch_hinted", "c2a_solve_batch_ordered",
               "c2a_solve_batch_ordered_host", "c2a_tolerance_batch", "c2a_collide_batch",
               "c2a_motion_setup", "c2a_motion_integrate"]

# include/c2a_probe.h
PROBE_SYMBOLS = ["c2a_probe_fp64_peak"]


class Params(C.Structure):
    _fields_ = [("tol_d", C.c_double), ("tol_t", C.c_double), ("toc_delta", C.c_double),
                ("contact_abs", C.c_double), ("with_contacts", C.c_int32), ("max_iters", C.c_int32),
                ("qsize", C.c_int32), ("contacts_per_query", C.c_int32), ("mode", C.c_int32),
                ("engine", C.c_int32), ("warps_per_sm", C.c_int32), ("heavy_prefix", C.c_int32)]


MODE_REFERENCE, MODE_CANONICAL = 0, 1
ENGINE_AUTO, ENGINE_WARP, ENGINE_BATCHED, ENGINE_THREAD, ENGINE_SPEC = 0, 1, 2, 3, 4


class Contacts:
    """Per-query view of a contact buffer: ``contacts[q]`` are query q's
    contacts in visiting order (at most contacts_per_query of them)."""

    def __init__(self, buf: np.ndarray, results: np.ndarray, slots: int):
        self.buf, self.results, self.slots = buf, results, slots

    def __len__(self):
        return len(self.results)

    def __getitem__(self, q):
        r = self.results[q]
        n = min(int(r["num_contact"]), self.slots)
        off = int(r["contact_offset"])
        return self.buf[off:off + n]

    def total(self) -> int:
        return int(np.minimum(self.results["num_contact"], self.slots).sum())


class C2AError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {status_str(status)} ({status})")
        self.status = status


_LIB = None


def load(build_if_missing: bool = False) -> C.CDLL:
    """Loads the in-tree library (builds it first when asked)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.environ.get("C2A_GB300_LIB") or _build.LIB  # a variant build (profiling) when set
    if not os.path.exists(path):
        if not build_if_missing or path != _build.LIB:
            raise FileNotFoundError(f"{path} is missing: run c2a_gb300.build.build() first")
        _build.build()
    lib = C.CDLL(path)
    vp, i32, dbl = C.c_void_p, C.c_int32, C.c_double
    sig = {
        "c2a_create": ([C.c_int, C.POINTER(vp)], i32),
        "c2a_destroy": ([vp], i32),
        "c2a_status_str": ([i32], C.c_char_p),
        "c2a_launch_count": ([vp, C.POINTER(C.c_int64)], i32),
        "c2a_model_build": ([vp, i32, vp, vp, vp, C.POINTER(i32)], i32),
        "c2a_model_build_many": ([vp, i32, vp, vp, vp, vp, i32, vp], i32),
        "c2a_model_build_async": ([vp, i32, vp, vp, vp, C.POINTER(vp)], i32),
        "c2a_model_wait": ([vp, C.POINTER(i32)], i32),
        "c2a_model_info": ([vp, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)], i32),
        "c2a_model_download": ([vp, i32, vp, vp, vp, vp, vp], i32),
        "c2a_model_download_obb": ([vp, i32, vp], i32),
        "c2a_model_free": ([vp, i32], i32),
        "c2a_solve_batch": ([vp, vp, i32, C.POINTER(Params), vp, vp], i32),
        "c2a_solve_batch_device": ([vp, vp, i32, C.POINTER(Params), vp, vp, vp], i32),
        "c2a_solve_batch_noalloc": ([vp, vp, i32, C.POINTER(Params), vp, vp, vp], i32),
        "c2a_toc_step_batch": ([vp, vp, i32, vp, vp, vp, C.POINTER(Params), vp], i32),
        "c2a_contact_only_batch": ([vp, vp, i32, vp, i32, vp, vp], i32),
        "c2a_distance_batch": ([vp, vp, i32, vp], i32),
        "c2a_solve_batch_ordered": ([vp, vp, i32, C.POINTER(Params), vp, vp, vp, vp], i32),
        "c2a_solve_batch_ordered_host": ([vp, vp, i32, C.POINTER(Params), vp, vp, vp], i32),
        "c2a_tolerance_batch": ([vp, vp, i32, vp, vp], i32),
        "c2a_collide_batch": ([vp, vp, i32, i32, i32, vp, vp], i32),
        "c2a_probe_fp64_peak": ([C.c_int, C.c_int, C.POINTER(dbl), C.POINTER(dbl)], i32),
        "c2a_motion_setup": ([vp, vp, vp, vp, vp], i32),
        "c2a_motion_integrate": ([vp, vp, vp, vp, dbl, vp, vp, vp], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _LIB = lib
    return lib


def fp64_peak(device: int = 0, repeats: int = 5) -> tuple[float, float]:
    """The FP64 pipe's measured peak on ``device``: (fused multiply-add flop/s,
    plain-addition flop/s), the best of ``repeats`` launches each."""
    lib = load()
    f, a = C.c_double(), C.c_double()
    _check(lib.c2a_probe_fp64_peak(device, repeats, C.byref(f), C.byref(a)), "c2a_probe_fp64_peak")
    return f.value, a.value


def status_str(s: int) -> str:
    return load().c2a_status_str(int(s)).decode()


def _ptr(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


def make_params(p: dict, contacts_per_query: int = 64) -> Params:
    return Params(float(p["tol_d"]), float(p["tol_t"]), float(p["toc_delta"]), float(p.get("contact_abs", 0.001)),
                  int(p.get("with_contacts", 1)), int(p.get("max_iters", 150)), int(p.get("qsize", 64)),
                  int(contacts_per_query), int(p.get("mode", MODE_REFERENCE)), int(p.get("engine", ENGINE_AUTO)),
                  int(p.get("warps_per_sm", 0)), int(p.get("heavy_prefix", 0)))


def make_queries(qint: np.ndarray, poses: np.ndarray) -> np.ndarray:
    q = np.zeros(len(qint), dtype=QUERY_DTYPE)
    q["model_a"], q["model_b"], q["seed_a"], q["seed_b"] = (qint[:, i] for i in range(4))
    q["pose"] = poses
    return q


def motion_setup(R0, T0, R1, T1) -> np.ndarray:
    """CInterpMotion_Linear constants: axis (3), angVel, cv (3), begin quaternion (x, y, z, w)."""
    a = [np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (R0, T0, R1, T1)]
    out = np.zeros(11)
    _check(load().c2a_motion_setup(*[_ptr(x) for x in a], _ptr(out)), "c2a_motion_setup")
    return out


def motion_integrate(R0, T0, R1, T1, t: float):
    a = [np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (R0, T0, R1, T1)]
    R, T, qua = np.zeros(9), np.zeros(3), np.zeros(7)
    _check(load().c2a_motion_integrate(*[_ptr(x) for x in a], float(t), _ptr(R), _ptr(T), _ptr(qua)),
           "c2a_motion_integrate")
    return R, T, qua


def _check(s: int, what: str):
    if s != C2A_OK:
        raise C2AError(s, what)


class Context:
    """A GPU context (device >= 0) or a host-only one (device -1: builds models only)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        _check(self.lib.c2a_create(int(device), C.byref(h)), "c2a_create")
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            self.lib.c2a_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- models ------------------------------------------------------------
    def model(self, mesh) -> int:
        tv = mesh.tri_verts()
        vidx = np.ascontiguousarray(mesh.faces, dtype=np.int32)
        mid = C.c_int32()
        _check(self.lib.c2a_model_build(self.h, mesh.num_tris, _ptr(tv), None, _ptr(vidx), C.byref(mid)),
               "c2a_model_build")
        return mid.value

    def models(self, meshes, threads: int = 0) -> list:
        """Builds every mesh at once on parallel host threads (c2a_model_build_many); ids in the order given."""
        meshes = list(meshes)
        if not meshes:
            return []
        tvs = [mesh.tri_verts() for mesh in meshes]
        vidxs = [np.ascontiguousarray(mesh.faces, dtype=np.int32) for mesh in meshes]
        n = len(meshes)
        counts = np.array([mesh.num_tris for mesh in meshes], dtype=np.int32)
        tv_ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in tvs])
        vidx_ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in vidxs])
        ids = np.full(n, -1, dtype=np.int32)
        _check(self.lib.c2a_model_build_many(self.h, n, _ptr(counts), C.cast(tv_ptrs, C.c_void_p), None,
                                             C.cast(vidx_ptrs, C.c_void_p), int(threads), _ptr(ids)),
               "c2a_model_build_many")
        return [int(i) for i in ids]

    def model_async(self, mesh) -> "C.c_void_p":
        """Starts building ``mesh`` on host threads (c2a_model_build_async); pass
        the handle to model_wait for the id."""
        tv = mesh.tri_verts()
        vidx = np.ascontiguousarray(mesh.faces, dtype=np.int32)
        h = C.c_void_p()
        _check(self.lib.c2a_model_build_async(self.h, mesh.num_tris, _ptr(tv), None, _ptr(vidx), C.byref(h)),
               "c2a_model_build_async")
        return h

    def model_wait(self, handle) -> int:
        """Finishes an asynchronous build, uploads the model and returns its id."""
        mid = C.c_int32()
        _check(self.lib.c2a_model_wait(handle, C.byref(mid)), "c2a_model_wait")
        return mid.value

    def model_info(self, mid: int) -> tuple[int, int, int]:
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        _check(self.lib.c2a_model_info(self.h, mid, C.byref(a), C.byref(b), C.byref(c)), "c2a_model_info")
        return a.value, b.value, c.value

    def download(self, mid: int):
        nt, nn, _ = self.model_info(mid)
        f = np.zeros((nn, 25))
        fc = np.zeros(nn, dtype=np.int32)
        tv = np.zeros((nt, 9))
        tid = np.zeros(nt, dtype=np.int32)
        tidx = np.zeros((nt, 3), dtype=np.int32)
        _check(self.lib.c2a_model_download(self.h, mid, _ptr(f), _ptr(fc), _ptr(tv), _ptr(tid), _ptr(tidx)),
               "c2a_model_download")
        return f, fc, tv, tid, tidx

    def download_obb(self, mid: int) -> np.ndarray:
        """(nodes, 6): each node's OBB centre in its parent's frame and half extents."""
        _, nn, _ = self.model_info(mid)
        o = np.zeros((nn, 6))
        _check(self.lib.c2a_model_download_obb(self.h, mid, _ptr(o)), "c2a_model_download_obb")
        return o

    def free_model(self, mid: int):
        _check(self.lib.c2a_model_free(self.h, mid), "c2a_model_free")

    def launches(self) -> int:
        n = C.c_int64()
        _check(self.lib.c2a_launch_count(self.h, C.byref(n)), "c2a_launch_count")
        return n.value

    # -- queries -----------------------------------------------------------
    def solve(self, qint: np.ndarray, poses: np.ndarray, params: dict, contacts_per_query: int = 64,
              check: bool = True):
        """C2A_Solve over a batch (host buffers in and out)."""
        q = make_queries(qint, poses)
        n = len(q)
        res = np.zeros(n, dtype=RESULT_DTYPE)
        con = np.zeros(max(1, n * contacts_per_query), dtype=CONTACT_DTYPE)
        prm = make_params(params, contacts_per_query)
        s = self.lib.c2a_solve_batch(self.h, _ptr(q), n, C.byref(prm), _ptr(res),
                                     _ptr(con) if contacts_per_query > 0 else None)
        if check:
            _check(s, "c2a_solve_batch")
        return res, Contacts(con, res, contacts_per_query)

    def distance(self, qint: np.ndarray, poses: np.ndarray, check: bool = True) -> np.ndarray:
        """C2A_Distance (rel_err = abs_err = 0) for a batch: model_a at pose[0:12],
        model_b at pose[24:36], seeded with (seed_a, seed_b); DISTANCE_DTYPE rows."""
        q = make_queries(qint, poses)
        res = np.zeros(len(q), dtype=DISTANCE_DTYPE)
        s = self.lib.c2a_distance_batch(self.h, _ptr(q), len(q), _ptr(res))
        if check:
            _check(s, "c2a_distance_batch")
        return res

    def tolerance(self, qint: np.ndarray, poses: np.ndarray, tolerance, check: bool = True) -> np.ndarray:
        """C2A_Tolerance (qsize 2) for a batch: model_a at pose[0:12], model_b at
        pose[24:36]; tolerance is a scalar or one per query; TOLERANCE_DTYPE rows."""
        q = make_queries(qint, poses)
        n = len(q)
        tol = np.ascontiguousarray(np.broadcast_to(np.asarray(tolerance, dtype=np.float64), (n,)))
        res = np.zeros(n, dtype=TOLERANCE_DTYPE)
        s = self.lib.c2a_tolerance_batch(self.h, _ptr(q), n, _ptr(tol), _ptr(res))
        if check:
            _check(s, "c2a_tolerance_batch")
        return res

    def collide(self, qint: np.ndarray, poses: np.ndarray, flag: int = 1, pairs_per_query: int = 256,
                check: bool = True):
        """C2A_Collide for a batch: (COLLIDE_DTYPE rows, pairs (n, pairs_per_query,
        2) caller triangle ids in visiting order, the first min(num_pairs, slots)
        of each row valid)."""
        q = make_queries(qint, poses)
        n = len(q)
        res = np.zeros(n, dtype=COLLIDE_DTYPE)
        pairs = np.zeros((n, max(1, pairs_per_query), 2), dtype=np.int32)
        s = self.lib.c2a_collide_batch(self.h, _ptr(q), n, int(flag), int(pairs_per_query), _ptr(res),
                                       _ptr(pairs) if pairs_per_query > 0 else None)
        if check:
            _check(s, "c2a_collide_batch")
        return res, pairs[:, :pairs_per_query]

    def solve_ordered_host(self, qint: np.ndarray, poses: np.ndarray, params: dict, d_order: int,
                           contacts_per_query: int = 64, check: bool = True):
        """c2a_solve_batch_ordered_host: as solve(), with the queries taken in the order of
        the device int32 permutation at d_order (REFERENCE mode)."""
        q = make_queries(qint, poses)
        n = len(q)
        res = np.zeros(n, dtype=RESULT_DTYPE)
        con = np.zeros(max(1, n * contacts_per_query), dtype=CONTACT_DTYPE)
        prm = make_params(params, contacts_per_query)
        s = self.lib.c2a_solve_batch_ordered_host(self.h, _ptr(q), n, C.byref(prm), C.c_void_p(d_order), _ptr(res),
                                                  _ptr(con) if contacts_per_query > 0 else None)
        if check:
            _check(s, "c2a_solve_batch_ordered_host")
        return res, Contacts(con, res, contacts_per_query)

    def solve_device(self, d_queries: int, n: int, params: dict, d_results: int, d_contacts: int | None,
                     contacts_per_query: int, stream: int | None = None):
        """C2A_Solve over a batch already in device memory (raw device pointers), async on ``stream``."""
        prm = make_params(params, contacts_per_query)
        _check(self.lib.c2a_solve_batch_device(self.h, C.c_void_p(d_queries), n, C.byref(prm),
                                               C.c_void_p(d_results),
                                               C.c_void_p(d_contacts) if d_contacts else None,
                                               C.c_void_p(stream) if stream else None), "c2a_solve_batch_device")

    def solve_ordered(self, d_queries: int, n: int, params: dict, d_order: int, d_results: int,
                      d_contacts: int | None, contacts_per_query: int, stream: int | None = None):
        """c2a_solve_batch_ordered: REFERENCE mode, queries taken in the order of the
        device int32 permutation at d_order (results as for solve_device)."""
        prm = make_params(params, contacts_per_query)
        _check(self.lib.c2a_solve_batch_ordered(self.h, C.c_void_p(d_queries), n, C.byref(prm), C.c_void_p(d_order),
                                                C.c_void_p(d_results),
                                                C.c_void_p(d_contacts) if d_contacts else None,
                                                C.c_void_p(stream) if stream else None), "c2a_solve_batch_ordered")

    def solve_noalloc(self, d_queries: int, n: int, params: dict, d_results: int, d_contacts: int | None,
                      contacts_per_query: int, stream: int | None = None):
        """c2a_solve_batch_noalloc: as solve_device, with the kernel's scratch in the
        library's fixed device array instead of context allocations."""
        prm = make_params(params, contacts_per_query)
        _check(self.lib.c2a_solve_batch_noalloc(self.h, C.c_void_p(d_queries), n, C.byref(prm),
                                                C.c_void_p(d_results),
                                                C.c_void_p(d_contacts) if d_contacts else None,
                                                C.c_void_p(stream) if stream else None), "c2a_solve_batch_noalloc")

    def step(self, qint, poses, lam, num_ca, prev_mint, params: dict):
        """C2A_TimeOfContactStep per query at time lam."""
        q = make_queries(qint, poses)
        n = len(q)
        res = np.zeros(n, dtype=RESULT_DTYPE)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        num_ca = np.ascontiguousarray(num_ca, dtype=np.int32)
        prev_mint = np.ascontiguousarray(prev_mint, dtype=np.float64)
        prm = make_params(params, 0)
        _check(self.lib.c2a_toc_step_batch(self.h, _ptr(q), n, _ptr(lam), _ptr(num_ca), _ptr(prev_mint),
                                           C.byref(prm), _ptr(res)), "c2a_toc_step_batch")
        return res

    def contact_only(self, qint, poses, threshold, contacts_per_query: int = 256):
        """C2A_QueryContactOnly at poses[:, 0:12] (A) and poses[:, 24:36] (B)."""
        q = make_queries(qint, poses)
        n = len(q)
        res = np.zeros(n, dtype=RESULT_DTYPE)
        con = np.zeros(max(1, n * contacts_per_query), dtype=CONTACT_DTYPE)
        thr = np.ascontiguousarray(threshold, dtype=np.float64)
        _check(self.lib.c2a_contact_only_batch(self.h, _ptr(q), n, _ptr(thr), contacts_per_query, _ptr(res),
                                               _ptr(con)), "c2a_contact_only_batch")
        return res, Contacts(con, res, contacts_per_query)
