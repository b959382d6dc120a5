"""Learned seeding of the CANONICAL closest-pair search.

A small network looks at a query's relative pose and velocity and at the two
meshes (a learned 16-float embedding each) and proposes the leaf-cluster
pairs most likely to hold the closest triangle pair.  A cluster is a node of
a model's BVH at depth 6 (or a shallower leaf): at most 64 per model, so a
pair is one of 64 x 64 = 4,096 classes.  At the first CA step, a descent
towards each of the top-8 proposals gives an exact triangle-pair distance
that can tighten the search's first bound (c2a_solve_batch_hinted).  The
search is exact, so the results are those of the plain engine bit for bit;
only the pruning changes.

Training data come from the library itself: the label of a query is the
cluster pair of its exact closest triangle pair at the start pose
(c2a_distance_batch, the reference's C2A_Distance with rel_err = abs_err = 0).

The network (include/c2a_mlp.h): x (18 pose/velocity features, two 16-float
embeddings, zero padding to 128) -> 256 -> 256 -> 256 -> 4,096 logits, GELU,
BF16 weights and activations, FP32 accumulation on the tensor cores, softmax
cross-entropy, Adam with FP32 master weights.  Every forward and backward
operation is one of the library's kernels; torch only allocates device
memory and passes pointers.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import api

CLUSTER_DEPTH = 6
NCLUSTER = 64
IN_FEATURES = 18
EMBED = 16
IN_WIDTH = 128  # 18 + 16 + 16 = 50 inputs, zero-padded to the GEMM's 128
HIDDEN = 256
OUT = NCLUSTER * NCLUSTER
TOPK = 8
ROW_ALIGN = 128

MLP_SYMBOLS = ["c2a_mlp_adam", "c2a_mlp_assemble", "c2a_mlp_check", "c2a_mlp_colsum", "c2a_mlp_embed_backward",
               "c2a_mlp_expect",
               "c2a_mlp_gelu_backward", "c2a_mlp_gemm", "c2a_mlp_order_desc", "c2a_mlp_softmax_xent",
               "c2a_mlp_topk", "c2a_mlp_transpose"]
ORDER_BINS = 1024  # C2A_ORDER_BINS


def order_scratch(n: int) -> int:
    """int32 scratch of c2a_mlp_order_desc (C2A_ORDER_SCRATCH)."""
    return (n + 1023) // 1024 * ORDER_BINS

BIAS, GELU = 1, 2


def bind(lib=None):
    lib = lib or api.load()
    vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    sig = {
        "c2a_mlp_gemm": [vp, vp, vp, i32, i32, i32, i32, vp, vp, vp],
        "c2a_mlp_transpose": [vp, i32, i32, vp, vp],
        "c2a_mlp_gelu_backward": [vp, vp, i64, vp, vp],
        "c2a_mlp_softmax_xent": [vp, vp, i32, i32, f32, vp, vp, vp],
        "c2a_mlp_colsum": [vp, i32, i32, vp, vp],
        "c2a_mlp_adam": [vp, vp, vp, vp, i64, f32, f32, f32, f32, i32, vp, vp, i32, i32, vp],
        "c2a_mlp_assemble": [vp, vp, vp, vp, i32, i32, i32, vp, vp],
        "c2a_mlp_embed_backward": [vp, vp, vp, i32, i32, vp, vp],
        "c2a_mlp_topk": [vp, i32, i32, i32, vp, vp],
        "c2a_mlp_expect": [vp, i32, i32, vp, vp],
        "c2a_mlp_order_desc": [vp, i32, f32, vp, vp, vp],
        "c2a_mlp_check": [vp],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = i32
    lib.c2a_solve_batch_hinted.argtypes = [vp, vp, i32, C.POINTER(api.Params), vp, i32, vp, vp, vp]
    lib.c2a_solve_batch_hinted.restype = i32
    return lib


def _p(t) -> C.c_void_p | None:
    return None if t is None else C.c_void_p(t.data_ptr())


def _ok(s: int, what: str):
    if s != 0:
        raise api.C2AError(s, what)


# ------------------------------------------------------------ clusters


@dataclass
class ClusterTable:
    """A model's leaf clusters: hint[c] encodes cluster c's node as its path
    from the root (low 16 bits; bit k = the child taken at depth k) and its
    depth (high 16 bits); of_tri[t] is the cluster of post-build triangle t."""
    hint: np.ndarray     # (64,) uint32
    of_tri: np.ndarray   # (num_tris,) int32
    count: int


def cluster_table(first_child: np.ndarray, num_tris: int, depth: int = CLUSTER_DEPTH) -> ClusterTable:
    """Cuts the hierarchy (children of node i at first_child[i] and + 1,
    leaves first_child < 0 holding triangle -first_child - 1) at ``depth``."""
    hint = np.zeros(NCLUSTER, dtype=np.uint32)
    of_tri = np.full(num_tris, -1, dtype=np.int32)
    level = [(0, 0)]  # (node, path)
    clusters = []
    for d in range(depth + 1):
        nxt = []
        for node, path in level:
            fc = int(first_child[node])
            if fc < 0 or d == depth:
                clusters.append((node, path, d))
            else:
                nxt.append((fc, path))
                nxt.append((fc + 1, path | (1 << d)))
        level = nxt
    assert len(clusters) <= NCLUSTER
    for c, (node, path, d) in enumerate(clusters):
        hint[c] = np.uint32(path | (d << 16))
        stack = [node]
        while stack:  # the cluster's triangles
            n = stack.pop()
            fc = int(first_child[n])
            if fc < 0:
                of_tri[-fc - 1] = c
            else:
                stack += [fc, fc + 1]
    assert (of_tri >= 0).all()
    return ClusterTable(hint, of_tri, len(clusters))


def cluster_tables(ctx: api.Context, model_ids) -> list[ClusterTable]:
    out = []
    for mid in model_ids:
        nt, _, _ = ctx.model_info(mid)
        _, fc, _, _, _ = ctx.download(mid)
        out.append(cluster_table(fc, nt))
    return out


# ------------------------------------------------------------ features


def _rotvec(R: np.ndarray) -> np.ndarray:
    from scipy.spatial.transform import Rotation

    return Rotation.from_matrix(R).as_rotvec()


def features(poses: np.ndarray, diag_a: np.ndarray, diag_b: np.ndarray) -> np.ndarray:
    """(n, 18) float32: B's start pose in A's start frame (R 9, T 3 over the
    mean diagonal), the relative linear velocity (3, same scale) and the
    relative angular velocity (3, radians over the motion), in A's frame."""
    n = len(poses)
    R0a, T0a = poses[:, 0:9].reshape(n, 3, 3), poses[:, 9:12]
    R1a, T1a = poses[:, 12:21].reshape(n, 3, 3), poses[:, 21:24]
    R0b, T0b = poses[:, 24:33].reshape(n, 3, 3), poses[:, 33:36]
    R1b, T1b = poses[:, 36:45].reshape(n, 3, 3), poses[:, 45:48]
    s = 0.5 * (np.asarray(diag_a) + np.asarray(diag_b))
    Rt = np.transpose(R0a, (0, 2, 1))
    R = Rt @ R0b
    T = np.einsum("nij,nj->ni", Rt, T0b - T0a) / s[:, None]
    v = np.einsum("nij,nj->ni", Rt, (T1b - T0b) - (T1a - T0a)) / s[:, None]
    wa = np.einsum("nij,nj->ni", R0a, _rotvec(np.transpose(R0a, (0, 2, 1)) @ R1a))
    wb = np.einsum("nij,nj->ni", R0b, _rotvec(np.transpose(R0b, (0, 2, 1)) @ R1b))
    w = np.einsum("nij,nj->ni", Rt, wb - wa)
    return np.ascontiguousarray(np.concatenate([R.reshape(n, 9), T, v, w], axis=1), dtype=np.float32)


def labels(ctx: api.Context, qint: np.ndarray, poses: np.ndarray, tables: list[ClusterTable],
           chunk: int = 65536) -> np.ndarray:
    """Cluster-pair class (64 ca + cb) of each query's exact closest triangle
    pair at the start pose; qint holds context model ids, ``tables`` is
    indexed by model id."""
    out = np.empty(len(qint), dtype=np.int32)
    for s in range(0, len(qint), chunk):
        r = ctx.distance(qint[s:s + chunk], poses[s:s + chunk])
        a, b = qint[s:s + chunk, 0], qint[s:s + chunk, 1]
        ca = np.array([tables[x].of_tri[t] for x, t in zip(a, r["tri_a"])], dtype=np.int32)
        cb = np.array([tables[x].of_tri[t] for x, t in zip(b, r["tri_b"])], dtype=np.int32)
        out[s:s + chunk] = ca * NCLUSTER + cb
    return out


def hints_of(top: np.ndarray, qint: np.ndarray, tables: list[ClusterTable]) -> np.ndarray:
    """(n, k, 2) uint32 hint codes of the proposed classes ``top`` (n, k)."""
    n, k = top.shape
    out = np.zeros((n, k, 2), dtype=np.uint32)
    ha = np.stack([t.hint if t is not None else np.zeros(NCLUSTER, np.uint32) for t in tables])  # (models, 64)
    out[:, :, 0] = ha[qint[:, 0][:, None], top // NCLUSTER]
    out[:, :, 1] = ha[qint[:, 1][:, None], top % NCLUSTER]
    return out


# ------------------------------------------------------------ network


class SeedNet:
    """The proposal network and its training state on one device."""

    def __init__(self, num_meshes: int, seed: int = 0, device: str = "cuda"):
        import torch

        self.torch = torch
        self.dev = torch.device(device)
        self.lib = bind()
        rng = np.random.default_rng(seed)
        dims = [(HIDDEN, IN_WIDTH), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (OUT, HIDDEN)]
        fan_in = [IN_FEATURES + 2 * EMBED, HIDDEN, HIDDEN, HIDDEN]
        self.W, self.b = [], []
        for (o, i), f in zip(dims, fan_in):
            w = np.zeros((o, i), dtype=np.float32)
            lim = 1.0 / math.sqrt(f)
            w[:, :f] = rng.uniform(-lim, lim, (o, f))
            self.W.append(torch.tensor(w, device=self.dev))
            self.b.append(torch.zeros(o, dtype=torch.float32, device=self.dev))
        self.E = torch.tensor(rng.normal(0.0, 0.5, (num_meshes, EMBED)).astype(np.float32), device=self.dev)
        self.params = self.W + self.b + [self.E]
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.g = [torch.zeros_like(p) for p in self.params]
        self.Wb = [w.to(torch.bfloat16) for w in self.W]
        self.WbT = [w.t().contiguous().to(torch.bfloat16) for w in self.W]
        self.t = 0
        self.stream = None  # torch's current stream

    # -- kernels -----------------------------------------------------------
    def _s(self):
        return C.c_void_p(self.torch.cuda.current_stream(self.dev).cuda_stream)

    def gemm(self, A, B, bias=None, flags=0, out_f32=None, out_bf16=None):
        M, K = A.shape
        N = B.shape[0]
        _ok(self.lib.c2a_mlp_gemm(_p(A), _p(B), _p(bias), M, N, K, flags, _p(out_f32), _p(out_bf16), self._s()),
            "c2a_mlp_gemm")

    def transpose(self, x):
        out = self.torch.empty((x.shape[1], x.shape[0]), dtype=x.dtype, device=self.dev)
        _ok(self.lib.c2a_mlp_transpose(_p(x), x.shape[0], x.shape[1], _p(out), self._s()), "c2a_mlp_transpose")
        return out

    def assemble(self, feat, ia, ib, M):
        x = self.torch.empty((M, IN_WIDTH), dtype=self.torch.bfloat16, device=self.dev)
        _ok(self.lib.c2a_mlp_assemble(_p(feat), _p(ia), _p(ib), _p(self.E), feat.shape[0], M, IN_WIDTH, _p(x),
                                      self._s()), "c2a_mlp_assemble")
        return x

    # -- passes ------------------------------------------------------------
    def forward(self, x):
        """logits (FP32) of the bf16 input rows x; keeps what backward needs."""
        torch = self.torch
        M = x.shape[0]
        acts, pres = [x], []
        h = x
        for layer in range(3):
            pre = torch.empty((M, HIDDEN), dtype=torch.float32, device=self.dev)
            out = torch.empty((M, HIDDEN), dtype=torch.bfloat16, device=self.dev)
            self.gemm(h, self.Wb[layer], self.b[layer], BIAS | GELU, pre, out)
            pres.append(pre)
            acts.append(out)
            h = out
        logits = torch.empty((M, OUT), dtype=torch.float32, device=self.dev)
        self.gemm(h, self.Wb[3], self.b[3], BIAS, logits, None)
        self._cache = (acts, pres)
        return logits

    def backward(self, logits, lab, ia, ib, n_valid):
        """Gradients of the mean cross-entropy over the first n_valid rows into
        self.g; returns the per-row losses."""
        torch = self.torch
        acts, pres = self._cache
        M = logits.shape[0]
        loss = torch.empty(M, dtype=torch.float32, device=self.dev)
        d = torch.empty((M, OUT), dtype=torch.bfloat16, device=self.dev)
        _ok(self.lib.c2a_mlp_softmax_xent(_p(logits), _p(lab), M, OUT, 1.0 / max(n_valid, 1), _p(loss), _p(d),
                                          self._s()), "c2a_mlp_softmax_xent")
        for layer in (3, 2, 1, 0):
            h_in = acts[layer]
            gW, gb = self.g[layer], self.g[4 + layer]
            self.gemm(self.transpose(d), self.transpose(h_in), out_f32=gW)
            _ok(self.lib.c2a_mlp_colsum(_p(d), M, d.shape[1], _p(gb), self._s()), "c2a_mlp_colsum")
            dh = torch.empty((M, h_in.shape[1]), dtype=torch.float32, device=self.dev)
            self.gemm(d, self.WbT[layer], out_f32=dh)
            if layer > 0:
                d = torch.empty((M, HIDDEN), dtype=torch.bfloat16, device=self.dev)
                _ok(self.lib.c2a_mlp_gelu_backward(_p(dh), _p(pres[layer - 1]), dh.numel(), _p(d), self._s()),
                    "c2a_mlp_gelu_backward")
            else:
                self.g[8].zero_()
                _ok(self.lib.c2a_mlp_embed_backward(_p(dh), _p(ia), _p(ib), n_valid, IN_WIDTH, _p(self.g[8]),
                                                    self._s()), "c2a_mlp_embed_backward")
        return loss

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.t += 1
        for i, p in enumerate(self.params):
            wb = self.Wb[i] if i < 4 else None
            wbt = self.WbT[i] if i < 4 else None
            rows, cols = (p.shape[0], p.shape[1]) if p.dim() == 2 else (1, p.shape[0])
            _ok(self.lib.c2a_mlp_adam(_p(p), _p(self.m[i]), _p(self.v[i]), _p(self.g[i]), p.numel(), lr, beta1,
                                      beta2, eps, self.t, _p(wb), _p(wbt), rows, cols, self._s()), "c2a_mlp_adam")

    # -- training and inference ---------------------------------------------
    def train(self, feat: np.ndarray, ia: np.ndarray, ib: np.ndarray, lab: np.ndarray, epochs: int = 4,
              batch: int = 1024, lr: float = 1e-3, seed: int = 0, log=None) -> list[float]:
        torch = self.torch
        assert batch % ROW_ALIGN == 0
        F = torch.tensor(feat, device=self.dev)
        A = torch.tensor(ia, dtype=torch.int32, device=self.dev)
        B = torch.tensor(ib, dtype=torch.int32, device=self.dev)
        Y = torch.tensor(lab, dtype=torch.int32, device=self.dev)
        g = torch.Generator(device="cpu")
        g.manual_seed(seed)
        n = len(feat)
        history = []
        for ep in range(epochs):
            perm = torch.randperm(n, generator=g).to(self.dev)
            tot = torch.zeros((), dtype=torch.float64, device=self.dev)
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                fa, aa, bb, yy = F[idx].contiguous(), A[idx].contiguous(), B[idx].contiguous(), Y[idx].contiguous()
                x = self.assemble(fa, aa, bb, batch)
                logits = self.forward(x)
                loss = self.backward(logits, yy, aa, bb, batch)
                self.adam(lr)
                tot += loss.double().sum()
            history.append(float(tot) / (n // batch * batch))
            if log:
                log(f"epoch {ep}: mean cross-entropy {history[-1]:.4f}")
        return history

    def logits(self, feat: np.ndarray, ia: np.ndarray, ib: np.ndarray, chunk: int = 16384):
        torch = self.torch
        out = []
        for s in range(0, len(feat), chunk):
            f = torch.tensor(feat[s:s + chunk], device=self.dev)
            m = f.shape[0]
            M = (m + ROW_ALIGN - 1) // ROW_ALIGN * ROW_ALIGN
            x = self.assemble(f, torch.tensor(ia[s:s + chunk], dtype=torch.int32, device=self.dev),
                              torch.tensor(ib[s:s + chunk], dtype=torch.int32, device=self.dev), M)
            out.append(self.forward(x)[:m])
        return torch.cat(out)

    def topk(self, feat: np.ndarray, ia: np.ndarray, ib: np.ndarray, k: int = TOPK) -> np.ndarray:
        torch = self.torch
        lg = self.logits(feat, ia, ib)
        idx = torch.empty((lg.shape[0], k), dtype=torch.int32, device=self.dev)
        _ok(self.lib.c2a_mlp_topk(_p(lg), lg.shape[0], OUT, k, _p(idx), self._s()), "c2a_mlp_topk")
        return idx.cpu().numpy()

    def state(self) -> dict:
        """Weights, biases and mesh embeddings (float32), then the Adam moments
        and step: everything training needs to resume."""
        st = {f"p{i}": p.cpu().numpy() for i, p in enumerate(self.params)}
        st.update({f"m{i}": m.cpu().numpy() for i, m in enumerate(self.m)})
        st.update({f"v{i}": v.cpu().numpy() for i, v in enumerate(self.v)})
        st["t"] = np.int64(self.t)
        return st

    def save(self, path: str) -> None:
        """Checkpoint to one .npz (state())."""
        np.savez(path, **self.state())

    def load_state(self, st) -> None:
        """Restores state() (shapes must match); the BF16 weight copies the
        GEMMs read are re-derived from the FP32 weights."""
        torch = self.torch
        for name, group in (("p", self.params), ("m", self.m), ("v", self.v)):
            for i, t in enumerate(group):
                a = np.asarray(st[f"{name}{i}"], dtype=np.float32)
                if a.shape != tuple(t.shape):
                    raise ValueError(f"checkpoint {name}{i} has shape {a.shape}, the network {tuple(t.shape)}")
                t.copy_(torch.from_numpy(a))
        self.t = int(st["t"])
        for i, w in enumerate(self.W):
            self.Wb[i].copy_(w.to(torch.bfloat16))
            self.WbT[i].copy_(w.t().contiguous().to(torch.bfloat16))

    @classmethod
    def load(cls, path: str, device: str = "cuda") -> "SeedNet":
        """A network rebuilt from save()'s checkpoint (its mesh count read from it)."""
        with np.load(path) as z:
            st = {k: z[k] for k in z.files}
        net = cls(int(st["p8"].shape[0]), device=device)
        net.load_state(st)
        return net


def solve_hinted(ctx: api.Context, qint: np.ndarray, poses: np.ndarray, params: dict, hints: np.ndarray,
                 contacts_per_query: int = 64, stream=None):
    """c2a_solve_batch_hinted on host arrays (CANONICAL mode); returns (results, contact buffer)."""
    import torch

    lib = bind(ctx.lib)
    q = api.make_queries(qint, poses)
    n = len(q)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    dh = torch.from_numpy(np.ascontiguousarray(hints, dtype=np.uint32).view(np.int32).copy()).cuda()
    dr = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    dc = torch.zeros(max(1, n * contacts_per_query) * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    prm = api.make_params(params, contacts_per_query)
    s = stream or torch.cuda.current_stream()
    _ok(lib.c2a_solve_batch_hinted(ctx.h, _p(dq), n, C.byref(prm), _p(dh), hints.shape[1], _p(dr),
                                   _p(dc) if contacts_per_query else None, C.c_void_p(s.cuda_stream)),
        "c2a_solve_batch_hinted")
    torch.cuda.synchronize()  # a null stream handle runs the batch on the context's own stream
    return dr.cpu().numpy().view(api.RESULT_DTYPE), dc.cpu().numpy().view(api.CONTACT_DTYPE)


# ------------------------------------------------------------ experiment


def _timed_solve(ctx, q, poses, prm, hints, cpq: int):
    """One CANONICAL batch through the device entry points (plain or hinted),
    timed with CUDA events on its stream; returns (ms, results, contacts)."""
    import torch

    lib = bind(ctx.lib)
    qs = api.make_queries(q, poses)
    n = len(qs)
    dq = torch.from_numpy(qs.view(np.uint8).copy()).cuda()
    dr = torch.zeros(n * api.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    dc = torch.zeros(max(1, n * cpq) * api.CONTACT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    dh = None
    if hints is not None:
        dh = torch.from_numpy(np.ascontiguousarray(hints, dtype=np.uint32).view(np.int32).copy()).cuda()
    prm_c = api.make_params(prm, cpq)
    s = torch.cuda.Stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(s)
    if dh is None:
        _ok(ctx.lib.c2a_solve_batch_device(ctx.h, _p(dq), n, C.byref(prm_c), _p(dr), _p(dc), C.c_void_p(s.cuda_stream)),
            "c2a_solve_batch_device")
    else:
        _ok(lib.c2a_solve_batch_hinted(ctx.h, _p(dq), n, C.byref(prm_c), _p(dh), hints.shape[1], _p(dr), _p(dc),
                                       C.c_void_p(s.cuda_stream)), "c2a_solve_batch_hinted")
    b.record(s)
    s.synchronize()
    return a.elapsed_time(b), dr.cpu().numpy().view(api.RESULT_DTYPE), dc.cpu().numpy().view(api.CONTACT_DTYPE)


def experiment(n_train: int = 2_000_000, n_eval: int = 65536, epochs: int = 4, pool: int = 12,
               tri_range=(1000, 200000), engine: int = api.ENGINE_BATCHED, batch: int = 1024, k: int = TOPK,
               seed: int = 3, log=print) -> dict:
    """Trains the proposal network on the uneven pool (labels from the
    library's exact distance query at the start pose) and measures the
    hinted CANONICAL solve against the plain one on held-out queries of the
    same pool: results must agree bit for bit, the queries/s may not."""
    import time

    from . import workloads

    t0 = time.time()
    wl = workloads.config3(n=n_train + n_eval, seed=seed, pool=pool, tri_range=tri_range)
    log(f"workload: {wl.n} queries over {pool} meshes ({[m.num_tris for m in wl.meshes]}) in {time.time() - t0:.1f} s")
    out = {"pool_tris": [m.num_tris for m in wl.meshes], "n_train": n_train, "n_eval": n_eval}
    with api.Context(0) as ctx:
        ids = np.array(ctx.models(wl.meshes))
        q = wl.qint.copy()
        q[:, 0], q[:, 1] = ids[wl.qint[:, 0]], ids[wl.qint[:, 1]]
        tabs = cluster_tables(ctx, ids)
        tab = [None] * (int(ids.max()) + 1)
        for i, t in zip(ids, tabs):
            tab[int(i)] = t
        t1 = time.time()
        lab = labels(ctx, q, wl.poses, tab)
        out["label_s"] = time.time() - t1
        log(f"labels: {wl.n} exact closest pairs in {out['label_s']:.1f} s")
        diag = np.array([m.bbox_diag() for m in wl.meshes])
        feat = features(wl.poses, diag[wl.qint[:, 0]], diag[wl.qint[:, 1]])
        tr, ev = slice(0, n_train), slice(n_train, n_train + n_eval)
        net = SeedNet(pool, seed=seed)
        t2 = time.time()
        hist = net.train(feat[tr], wl.qint[tr, 0], wl.qint[tr, 1], lab[tr], epochs=epochs, batch=batch, log=log)
        out["train_s"] = time.time() - t2
        out["loss"] = hist
        top = net.topk(feat[ev], wl.qint[ev, 0], wl.qint[ev, 1], k)
        out["top1"] = float(np.mean(top[:, 0] == lab[ev]))
        out["topk"] = float(np.mean([lab[ev][i] in top[i] for i in range(n_eval)]))
        log(f"held-out: top-1 {out['top1']:.3f}, top-{k} {out['topk']:.3f}; trained in {out['train_s']:.1f} s")
        hints = hints_of(top, q[ev], tab)
        prm = dict(wl.params, mode=api.MODE_CANONICAL, engine=engine)
        cpq = 64
        _timed_solve(ctx, q[ev][:256], wl.poses[ev][:256], prm, None, cpq)  # warm-up
        ms_plain, rp, cp = _timed_solve(ctx, q[ev], wl.poses[ev], prm, None, cpq)
        ms_hint, rh, ch = _timed_solve(ctx, q[ev], wl.poses[ev], prm, hints, cpq)
        # the ceiling: the true closest cluster pair as the only hint
        ms_oracle, ro, _ = _timed_solve(ctx, q[ev], wl.poses[ev], prm, hints_of(lab[ev][:, None], q[ev], tab), cpq)
        out["oracle_hint_ms"] = ms_oracle
        out["oracle_identical"] = all(ro[f].tobytes() == rp[f].tobytes() for f in ("collisionfree", "numCA", "toc",
                                                                                   "distance", "mint", "seed_a",
                                                                                   "seed_b"))
        log(f"true-pair hints: {ms_oracle:.1f} ms")
        fields = ("collisionfree", "numCA", "toc", "distance", "mint", "num_contact", "seed_a", "seed_b",
                  "num_bv_tests", "num_tri_tests", "R_toc", "T_toc")
        differ = [f for f in fields if rp[f].tobytes() != rh[f].tobytes()]
        used = np.minimum(rp["num_contact"], cpq)
        cfields = ("type_a", "type_b", "fid_a", "fid_b", "tri_a", "tri_b", "pa", "pb", "distance")
        for i in range(n_eval):
            if rp["num_contact"][i] > cpq:
                continue  # more contacts than slots: which ones are stored is unspecified in CANONICAL mode
            a, b = cp[i * cpq:i * cpq + used[i]], ch[i * cpq:i * cpq + used[i]]
            differ += [f"contact.{f}" for f in cfields if a[f].tobytes() != b[f].tobytes()]
        out["differ"] = sorted(set(differ))
        same = same_c = not differ
        out["contact_overflow_queries"] = int(np.sum(rp["num_contact"] > cpq))
        out.update(plain_ms=ms_plain, hinted_ms=ms_hint, plain_qps=n_eval / ms_plain * 1e3,
                   hinted_qps=n_eval / ms_hint * 1e3, speedup=ms_plain / ms_hint, identical=bool(same and same_c),
                   colliding=float(np.mean(rp["collisionfree"] == 0)),
                   bv_tests_plain=int(rp["num_bv_tests"].sum()), bv_tests_hinted=int(rh["num_bv_tests"].sum()))
        log(f"CANONICAL engine {engine}: plain {ms_plain:.1f} ms, hinted {ms_hint:.1f} ms "
            f"({out['speedup']:.3f}x), identical results: {out['identical']}")
        # end to end from host arrays: pose features on the host, the network's top-k on the device, the
        # hint codes, then the hinted solve (queries and hints H2D, results and contacts D2H)
        launches0 = ctx.launches()
        t3 = time.perf_counter()
        f_ev = features(wl.poses[ev], diag[wl.qint[ev, 0]], diag[wl.qint[ev, 1]])
        top_e = net.topk(f_ev, wl.qint[ev, 0], wl.qint[ev, 1], k)
        re, _ = solve_hinted(ctx, q[ev], wl.poses[ev], prm, hints_of(top_e, q[ev], tab), cpq)
        out["e2e_s"] = time.perf_counter() - t3
        out["e2e_launches"] = ctx.launches() - launches0
        out["e2e_identical"] = all(re[f].tobytes() == rp[f].tobytes() for f in fields)
        out["e2e_h2d_bytes"] = n_eval * (api.QUERY_DTYPE.itemsize + 18 * 4 + 2 * 4 + k * 8)
        out["e2e_d2h_bytes"] = n_eval * (api.RESULT_DTYPE.itemsize + cpq * api.CONTACT_DTYPE.itemsize + k * 4)
        out["eval_results"] = rp
        out["eval_workload"] = wl.subset(np.arange(n_train, n_train + n_eval))
    return out


# ------------------------------------------------------------ learned schedule

COST_BUCKETS = 64
LEAF_COST = 1.6  # a leaf pair (TriDist on the warp) against an expansion, from the profiling build's cycle counters


def query_cost(results: np.ndarray) -> np.ndarray:
    """A REFERENCE query's work in expansions: num_bv_tests / 2 node-pair
    expansions plus the triangle tests weighted by their relative cost."""
    return results["num_bv_tests"] / 2.0 + LEAF_COST * results["num_tri_tests"]


class CostOrder:
    """Learned schedule for REFERENCE batches: the same network, trained to
    classify a query's log-cost into 64 buckets from its pose features;
    queries are then taken in decreasing expected bucket (the costliest
    first), which shortens a batch whose length is set by its heaviest
    queries.  The order never changes a result (c2a_solve_batch_ordered)."""

    def __init__(self, num_meshes: int = 1, seed: int = 0, device: str = "cuda"):
        self.net = SeedNet(num_meshes, seed=seed, device=device)
        self.top = 1.0

    def save(self, path: str) -> None:
        """Checkpoint: the network's state and the cost scale of the buckets."""
        np.savez(path, top=np.float64(self.top), **self.net.state())

    @classmethod
    def load(cls, path: str, device: str = "cuda") -> "CostOrder":
        with np.load(path) as z:
            st = {k: z[k] for k in z.files}
        co = cls(int(st["p8"].shape[0]), device=device)
        co.net.load_state(st)
        co.top = float(st["top"])
        return co

    def fit(self, feat, ia, ib, cost, epochs: int = 10, batch: int = 1024, log=None) -> list[float]:
        y = np.log1p(np.asarray(cost, dtype=np.float64))
        self.top = float(y.max()) if y.max() > 0 else 1.0
        lab = np.minimum((y / self.top * (COST_BUCKETS - 1)).astype(np.int32), COST_BUCKETS - 1)
        return self.net.train(feat, ia, ib, lab, epochs=epochs, batch=batch, log=log)

    def expected(self, feat_dev, ia_dev, ib_dev):
        """Expected cost bucket of each query (device FP32); inputs on the device."""
        torch = self.net.torch
        n = feat_dev.shape[0]
        M = (n + ROW_ALIGN - 1) // ROW_ALIGN * ROW_ALIGN
        x = self.net.assemble(feat_dev, ia_dev, ib_dev, M)
        logits = self.net.forward(x)
        out = torch.empty(M, dtype=torch.float32, device=self.net.dev)
        _ok(self.net.lib.c2a_mlp_expect(_p(logits), M, OUT, _p(out), self.net._s()), "c2a_mlp_expect")
        return out[:n]

    def order(self, feat_dev, ia_dev, ib_dev):
        """The schedule: query indices by decreasing expected cost (device int32),
        the library's stable counting sort over the expected bucket quantised to
        1/16 of a bucket (c2a_mlp_order_desc)."""
        torch = self.net.torch
        e = self.expected(feat_dev, ia_dev, ib_dev)
        n = e.shape[0]
        if getattr(self, "_scratch", None) is None or self._scratch.numel() < order_scratch(n):
            self._scratch = torch.empty(order_scratch(n), dtype=torch.int32, device=self.net.dev)
        out = torch.empty(n, dtype=torch.int32, device=self.net.dev)
        _ok(self.net.lib.c2a_mlp_order_desc(_p(e), n, float(COST_BUCKETS - 1), _p(out), _p(self._scratch),
                                            self.net._s()), "c2a_mlp_order_desc")
        return out
