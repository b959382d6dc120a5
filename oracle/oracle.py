"""ctypes front end of the CPU oracle (test infrastructure only).

Two checkers, both built by ``oracle/Makefile``:

* ``Port`` -- ``oracle/_build/libc2a_port.so``, the plain-C restatement of
  the C2A CA path.  Available wherever gcc is (this container and the GPU
  box); the bench's CPU-baseline leg times it.
* ``Ref``  -- ``oracle/_ref/libc2a_ref.so``, the reference's own C2A sources
  compiled against the PQP-interface restatement.  Buildable only where the
  reference sources are; it pins ``Port`` and generates the golden fixtures.

Only tests, ``__graft_entry__.smoke`` and ``bench.py``'s CPU leg import this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libc2a_port.so")
REF_SO = os.path.join(HERE, "_ref", "libc2a_ref.so")

RESULT_DTYPE = np.dtype([("collisionfree", np.int32), ("numCA", np.int32), ("translation", np.int32),
                         ("num_contact", np.int32), ("toc", np.float64), ("distance", np.float64),
                         ("mint", np.float64), ("num_bv_tests", np.int64), ("num_tri_tests", np.int64),
                         ("R_toc", np.float64, (2, 9)), ("T_toc", np.float64, (2, 3)),
                         ("seed_a", np.int32), ("seed_b", np.int32)], align=True)
CONTACT_DTYPE = np.dtype([("type_a", np.int32), ("type_b", np.int32), ("fid_a", np.int32, (3,)),
                          ("fid_b", np.int32, (3,)), ("tri_a", np.int32), ("tri_b", np.int32),
                          ("pa", np.float64, (3,)), ("pb", np.float64, (3,)), ("distance", np.float64)],
                         align=True)
assert RESULT_DTYPE.itemsize == 256 and CONTACT_DTYPE.itemsize == 96


def build(ref: bool | None = None) -> None:
    """Builds the port (always) and the reference library (when its sources exist)."""
    target = "all" if ref is None else ("ref" if ref else "port")
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


class _Params(C.Structure):
    _fields_ = [("tol_d", C.c_double), ("tol_t", C.c_double), ("toc_delta", C.c_double),
                ("contact_abs", C.c_double), ("with_contacts", C.c_int), ("max_iters", C.c_int),
                ("mode", C.c_int), ("reserved", C.c_int)]

MODE_REFERENCE, MODE_CANONICAL = 0, 1


class _PortModel(C.Structure):
    _fields_ = [("num_tris", C.c_int), ("num_nodes", C.c_int), ("tris", C.c_void_p), ("nodes", C.c_void_p)]


NODE_DTYPE = np.dtype([("R", np.float64, (9,)), ("Tr", np.float64, (3,)), ("l", np.float64, (2,)),
                       ("r", np.float64), ("angR", np.float64), ("Rloc", np.float64, (9,)),
                       ("To", np.float64, (3,)), ("d", np.float64, (3,)),
                       ("first_child", np.int32), ("pad", np.int32)], align=True)
TRI_DTYPE = np.dtype([("v", np.float64, (9,)), ("id", np.int32), ("idx", np.int32, (3,))], align=True)


def _params(p: dict) -> _Params:
    return _Params(float(p["tol_d"]), float(p["tol_t"]), float(p["toc_delta"]), float(p["contact_abs"]),
                   int(p.get("with_contacts", 1)), int(p.get("max_iters", 150)), int(p.get("mode", 0)), 0)


def _dptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Port:
    """The plain-C oracle port."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build(ref=False)
        self.lib = C.CDLL(path)
        L = self.lib
        L.c2a_port_model_build.argtypes = [C.POINTER(_PortModel), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.c2a_port_model_build.restype = C.c_int
        L.c2a_port_model_free.argtypes = [C.POINTER(_PortModel)]
        L.c2a_port_solve_batch.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                           C.POINTER(_Params), C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.c2a_port_solve_batch.restype = C.c_int
        L.c2a_port_rectdist.argtypes = [C.c_void_p] * 7
        L.c2a_port_rectdist.restype = C.c_double
        L.c2a_port_tridist.argtypes = [C.c_void_p] * 9
        L.c2a_port_tridist.restype = C.c_double
        L.c2a_port_contact_only.argtypes = [C.POINTER(_PortModel), C.POINTER(_PortModel)] + [C.c_void_p] * 4 + \
                                           [C.c_double, C.c_void_p, C.c_int]
        L.c2a_port_contact_only.restype = C.c_int
        L.c2a_port_distance.argtypes = [C.POINTER(_PortModel), C.POINTER(_PortModel), C.c_void_p, C.c_void_p,
                                        C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.c2a_port_distance.restype = C.c_double
        L.c2a_port_tolerance.argtypes = [C.POINTER(_PortModel), C.POINTER(_PortModel), C.c_void_p, C.c_void_p,
                                         C.c_double] + [C.c_void_p] * 5
        L.c2a_port_tolerance.restype = C.c_int
        L.c2a_port_collide.argtypes = [C.POINTER(_PortModel), C.POINTER(_PortModel), C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.c2a_port_collide.restype = C.c_int

    def models(self, meshes) -> C.Array:
        """Builds every mesh's hierarchy; returns a ctypes array of models."""
        arr = (_PortModel * len(meshes))()
        for i, m in enumerate(meshes):
            tv = m.tri_verts()
            vidx = np.ascontiguousarray(m.faces, dtype=np.int32)
            rc = self.lib.c2a_port_model_build(C.byref(arr[i]), m.num_tris, _dptr(tv), None, _dptr(vidx))
            if rc != 0:
                raise RuntimeError(f"port model build failed ({rc})")
        return arr

    def dump(self, models, i: int) -> tuple[np.ndarray, np.ndarray]:
        m = models[i]
        nodes = np.ctypeslib.as_array((C.c_char * (m.num_nodes * NODE_DTYPE.itemsize)).from_address(m.nodes))
        tris = np.ctypeslib.as_array((C.c_char * (m.num_tris * TRI_DTYPE.itemsize)).from_address(m.tris))
        return nodes.view(NODE_DTYPE).copy(), tris.view(TRI_DTYPE).copy()

    def solve_batch(self, models, qint: np.ndarray, poses: np.ndarray, params: dict, threads: int = 1,
                    contacts_per_query: int = 64):
        n = len(qint)
        qint = np.ascontiguousarray(qint, dtype=np.int32)
        poses = np.ascontiguousarray(poses, dtype=np.float64)
        res = np.zeros(n, dtype=RESULT_DTYPE)
        con = np.zeros(n * max(contacts_per_query, 1), dtype=CONTACT_DTYPE)
        prm = _params(params)
        bad = self.lib.c2a_port_solve_batch(models, len(models), _dptr(qint), _dptr(poses), n, C.byref(prm),
                                            _dptr(res), _dptr(con) if contacts_per_query > 0 else None,
                                            contacts_per_query, threads)
        if bad:
            raise RuntimeError(f"{bad} queries rejected by the oracle port")
        return res, con.reshape(n, max(contacts_per_query, 1))

    def count_flops(self, models, qint: np.ndarray, poses: np.ndarray, params: dict) -> dict:
        """FP64 operation counts of the port's CA path over a batch
        (flop_count.cpp): per bucket (other, expansion, triangle test,
        contacts) the add/sub, mul, div, sqrt and compare counts, and the
        summed num_bv_tests / num_tri_tests."""
        lib = C.CDLL(os.path.join(HERE, "_build", "libc2a_flops.so"))
        lib.c2a_fc_solve.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                     C.c_void_p, C.c_void_p]
        lib.c2a_fc_solve.restype = C.c_int
        qint = np.ascontiguousarray(qint, dtype=np.int32)
        poses = np.ascontiguousarray(poses, dtype=np.float64)
        ops = np.zeros((4, 5), dtype=np.int64)
        cnt = np.zeros(2, dtype=np.int64)
        prm = _params(params)
        bad = lib.c2a_fc_solve(C.cast(models, C.c_void_p), len(models), _dptr(qint), _dptr(poses), len(qint),
                               C.byref(prm), _dptr(ops), _dptr(cnt))
        if bad:
            raise RuntimeError(f"{bad} queries rejected by the counting port")
        return {"ops": ops, "num_bv_tests": int(cnt[0]), "num_tri_tests": int(cnt[1])}

    def distance(self, models, ia: int, ib: int, R, T, seed_a: int, seed_b: int):
        """C2A_Distance (rel_err = abs_err = 0) with B placed in A's frame by (R, T):
        (distance, tri_a, tri_b) in the reference's order and tie rule."""
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(9)
        T = np.ascontiguousarray(T, dtype=np.float64).reshape(3)
        t = np.zeros(2, dtype=np.int32)
        d = self.lib.c2a_port_distance(C.byref(models[ia]), C.byref(models[ib]), _dptr(R), _dptr(T), int(seed_a),
                                       int(seed_b), _dptr(t[0:1]), _dptr(t[1:2]), None, None)
        return d, int(t[0]), int(t[1])

    def tolerance(self, models, ia: int, ib: int, R, T, tol: float):
        """C2A_Tolerance (qsize 2): (closer, distance, p1, p2, num_bv_tests, num_tri_tests)."""
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(9)
        T = np.ascontiguousarray(T, dtype=np.float64).reshape(3)
        d = np.zeros(1)
        p1, p2 = np.zeros(3), np.zeros(3)
        n = np.zeros(2, dtype=np.int64)
        c = self.lib.c2a_port_tolerance(C.byref(models[ia]), C.byref(models[ib]), _dptr(R), _dptr(T), float(tol),
                                        _dptr(d), _dptr(p1), _dptr(p2), _dptr(n[0:1]), _dptr(n[1:2]))
        return c, float(d[0]), p1, p2, int(n[0]), int(n[1])

    def collide(self, models, ia: int, ib: int, R, T, flag: int = 1, cap: int = 1 << 16):
        """C2A_Collide: (pairs (k, 2) caller ids in the order found, num_bv_tests, num_tri_tests)."""
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(9)
        T = np.ascontiguousarray(T, dtype=np.float64).reshape(3)
        pairs = np.zeros((cap, 2), dtype=np.int32)
        n = np.zeros(2, dtype=np.int64)
        k = self.lib.c2a_port_collide(C.byref(models[ia]), C.byref(models[ib]), _dptr(R), _dptr(T), int(flag),
                                      _dptr(pairs), cap, _dptr(n[0:1]), _dptr(n[1:2]))
        return pairs[:min(k, cap)].copy(), int(n[0]), int(n[1])

    def rectdist(self, Rab, Tab, a, b):
        Rab = np.ascontiguousarray(Rab, dtype=np.float64).reshape(9)
        Tab, a, b = (np.ascontiguousarray(x, dtype=np.float64) for x in (Tab, a, b))
        P, Q, S = np.zeros(3), np.zeros(3), np.full(3, np.nan)
        d = self.lib.c2a_port_rectdist(_dptr(Rab), _dptr(Tab), _dptr(a), _dptr(b), _dptr(P), _dptr(Q), _dptr(S))
        return d, P, Q, S

    def tridist(self, S9, T9):
        S9 = np.ascontiguousarray(S9, dtype=np.float64).reshape(9)
        T9 = np.ascontiguousarray(T9, dtype=np.float64).reshape(9)
        P, Q = np.zeros(3), np.zeros(3)
        i = np.full(5, -1, dtype=np.int32)
        i[4] = 0
        d = self.lib.c2a_port_tridist(_dptr(P), _dptr(Q), _dptr(S9), _dptr(T9), _dptr(i[0:1]), _dptr(i[1:2]),
                                      _dptr(i[2:3]), _dptr(i[3:4]), _dptr(i[4:5]))
        return d, P, Q, tuple(int(x) for x in i)


class Ref:
    """The reference's own C2A sources (only where they were compiled)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        L.c2a_ref_model_build.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.c2a_ref_model_build.restype = C.c_void_p
        L.c2a_ref_model_num_nodes.argtypes = [C.c_void_p]
        L.c2a_ref_model_num_tris.argtypes = [C.c_void_p]
        L.c2a_ref_model_last_tri.argtypes = [C.c_void_p]
        L.c2a_ref_model_dump.argtypes = [C.c_void_p] * 6
        L.c2a_ref_solve.argtypes = [C.c_void_p, C.c_void_p] + [C.c_void_p] * 8 + [C.c_int, C.c_int] + \
                                   [C.c_double] * 4 + [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        L.c2a_ref_solve_canonical.argtypes = L.c2a_ref_solve.argtypes
        L.c2a_ref_solve_shipped.argtypes = [C.c_void_p, C.c_void_p] + [C.c_void_p] * 8 + [C.c_int, C.c_int] + \
                                           [C.c_void_p, C.c_void_p, C.c_int]
        L.c2a_ref_rectdist.argtypes = [C.c_void_p] * 7
        L.c2a_ref_rectdist.restype = C.c_double
        L.c2a_ref_tridist.argtypes = [C.c_void_p] * 9
        L.c2a_ref_tridist.restype = C.c_double
        L.c2a_ref_motion.argtypes = [C.c_void_p] * 4 + [C.c_double] + [C.c_void_p] * 3
        L.c2a_ref_distance.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_int] + [C.c_void_p] * 4
        L.c2a_ref_distance.restype = C.c_double
        L.c2a_ref_tolerance.argtypes = [C.c_void_p] * 4 + [C.c_double, C.c_void_p]
        L.c2a_ref_tolerance.restype = C.c_int
        L.c2a_ref_collide.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_void_p, C.c_int, C.c_void_p]
        L.c2a_ref_collide.restype = C.c_int

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_SO)

    def last_tri(self, h) -> int:
        """The model's last_tri (post-build index): the seed the demo passes next."""
        return int(self.lib.c2a_ref_model_last_tri(h))

    def model(self, mesh):
        tv = mesh.tri_verts()
        vidx = np.ascontiguousarray(mesh.faces, dtype=np.int32)
        h = self.lib.c2a_ref_model_build(mesh.num_tris, _dptr(tv), None, _dptr(vidx))
        if not h:
            raise RuntimeError("reference model build failed")
        return C.c_void_p(h)

    def dump(self, h):
        nn = self.lib.c2a_ref_model_num_nodes(h)
        nt = self.lib.c2a_ref_model_num_tris(h)
        f = np.zeros((nn, 25))
        fc = np.zeros(nn, dtype=np.int32)
        tv = np.zeros((nt, 9))
        tid = np.zeros(nt, dtype=np.int32)
        tidx = np.zeros((nt, 3), dtype=np.int32)
        self.lib.c2a_ref_model_dump(h, _dptr(f), _dptr(fc), _dptr(tv), _dptr(tid), _dptr(tidx))
        return f, fc, tv, tid, tidx

    def solve(self, ha, hb, pose: np.ndarray, seed_a: int, seed_b: int, params: dict, max_contacts: int = 4096,
              shipped: bool = False):
        p = np.ascontiguousarray(pose, dtype=np.float64)
        res = np.zeros(1, dtype=RESULT_DTYPE)
        con = np.zeros(max_contacts, dtype=CONTACT_DTYPE)
        ptrs = [C.c_void_p(p.ctypes.data + 8 * o) for o in (0, 9, 12, 21, 24, 33, 36, 45)]
        if shipped:
            self.lib.c2a_ref_solve_shipped(ha, hb, *ptrs, seed_a, seed_b, _dptr(res), _dptr(con), max_contacts)
        else:
            fn = self.lib.c2a_ref_solve_canonical if params.get("mode", 0) == MODE_CANONICAL else self.lib.c2a_ref_solve
            fn(ha, hb, *ptrs, seed_a, seed_b, float(params["tol_d"]), float(params["tol_t"]),
                                   float(params["toc_delta"]), float(params["contact_abs"]),
                                   int(params.get("with_contacts", 1)), int(params.get("max_iters", 150)),
                                   _dptr(res), _dptr(con), max_contacts)
        nc = int(res["num_contact"][0])
        return res[0], con[:min(nc, max_contacts)]

    def rectdist(self, Rab, Tab, a, b):
        Rab = np.ascontiguousarray(Rab, dtype=np.float64).reshape(9)
        Tab, a, b = (np.ascontiguousarray(x, dtype=np.float64) for x in (Tab, a, b))
        P, Q, S = np.zeros(3), np.zeros(3), np.full(3, np.nan)
        d = self.lib.c2a_ref_rectdist(_dptr(Rab), _dptr(Tab), _dptr(a), _dptr(b), _dptr(P), _dptr(Q), _dptr(S))
        return d, P, Q, S

    def tridist(self, S9, T9):
        S9 = np.ascontiguousarray(S9, dtype=np.float64).reshape(9)
        T9 = np.ascontiguousarray(T9, dtype=np.float64).reshape(9)
        P, Q = np.zeros(3), np.zeros(3)
        i = np.full(5, -1, dtype=np.int32)
        i[4] = 0
        d = self.lib.c2a_ref_tridist(_dptr(P), _dptr(Q), _dptr(S9), _dptr(T9), _dptr(i[0:1]), _dptr(i[1:2]),
                                     _dptr(i[2:3]), _dptr(i[3:4]), _dptr(i[4:5]))
        return d, P, Q, tuple(int(x) for x in i)

    def distance(self, ha, hb, R, T, seed_a: int, seed_b: int):
        """The reference's C2A_Distance (rel_err = abs_err = 0, qsize 2): (distance, tri_a, tri_b).
        ha and hb must be distinct model objects (the query sets each one's last_tri)."""
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(9)
        T = np.ascontiguousarray(T, dtype=np.float64).reshape(3)
        t = np.zeros(2, dtype=np.int32)
        d = self.lib.c2a_ref_distance(ha, hb, _dptr(R), _dptr(T), int(seed_a), int(seed_b), _dptr(t[0:1]),
                                      _dptr(t[1:2]), None, None)
        return d, int(t[0]), int(t[1])

    def tolerance(self, ha, hb, R, T, tol: float):
        """The reference's C2A_Tolerance (qsize 2): (closer, distance, p1, p2, num_bv_tests, num_tri_tests)."""
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(9)
        T = np.ascontiguousarray(T, dtype=np.float64).reshape(3)
        out = np.zeros(9)
        c = self.lib.c2a_ref_tolerance(ha, hb, _dptr(R), _dptr(T), float(tol), _dptr(out))
        return c, float(out[0]), out[1:4].copy(), out[4:7].copy(), int(out[7]), int(out[8])

    def collide(self, ha, hb, R, T, flag: int = 1, cap: int = 1 << 16):
        """The reference's C2A_Collide: (pairs (k, 2) caller ids in order, num_bv_tests, num_tri_tests)."""
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(9)
        T = np.ascontiguousarray(T, dtype=np.float64).reshape(3)
        pairs = np.zeros((cap, 2), dtype=np.int32)
        n = np.zeros(2, dtype=np.int64)
        k = self.lib.c2a_ref_collide(ha, hb, _dptr(R), _dptr(T), int(flag), _dptr(pairs), cap, _dptr(n))
        return pairs[:min(k, cap)].copy(), int(n[0]), int(n[1])

    def motion(self, R0, T0, R1, T1, t):
        args = [np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (R0, T0, R1, T1)]
        out = np.zeros(7)
        R = np.zeros(9)
        T = np.zeros(3)
        self.lib.c2a_ref_motion(*[_dptr(a) for a in args], float(t), _dptr(out), _dptr(R), _dptr(T))
        return out[:3], out[3], out[4:7], R, T
