"""Continuous-batching solve server on one GPU.

Requests -- rigid-body resistance solves and free-swimmer instants of uneven
size -- are submitted as they arrive and served by `slots` workers, each a host
thread with its own CUDA stream, so the work of concurrent requests overlaps
on the device.  Scheduling is continuous: whenever a slot finishes, it admits
the next pending request (preferring one of the bucket it already has a plan
for) provided the HBM budget allows; nothing waits for a batch to fill.

Resistance requests are padded to a size bucket (N rounded up on a ~19 %
geometric grid of multiples of 128 points).  Each slot keeps one *bucket plan*:
fixed device buffers and a CUDA graph capturing, for that bucket size,
``flg_assemble_bucket`` (real block + identity padding) -> FP32 copy ->
``flg_lu_factor_lowp_async`` (tensor-core LU, no host sync).  A request copies
its points into the plan's buffers, replays the graph and runs FP64 GMRES-IR
on the padded system; padded rows are identity and padded right-hand sides
zero, so the solution is exactly that of the unpadded system (the forces
agree with a solve of the request alone to rounding).  The per-bucket choice
of tensor-core precision (TF32 or BF16) and of the trailing updates' tile
width (128 x 128, 128 x 256, or chosen per update from its shape) is made by a
small autotuner that times the candidates on the first request of the bucket and
keeps the fastest one that converges.  Swimmer requests run on pooled swimmer
plans, one per shape size: a captured graph of the nearest map, the nearest-
neighbour assembly, the constraint rows, the FP32 copies and the tensor-core LU,
replayed with the request's points, then FP64 GMRES-IR.
"""
from __future__ import annotations

import ctypes
import math
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _device as dv
from ._lib import F64, LU_MODE, check, load, lu_mode
from .kernels import Stokeslet3D, kernel_params

BUCKET_BASE = 128
# LU modes the autotuner times per bucket: precision, and the tile width of the trailing updates
# (no suffix: chosen per update from its shape); "fp32" factors on the CUDA cores, which can win
# for the smallest buckets, where the tensor-core updates are too small to fill the GPU
TUNE_CANDIDATES = ("tf32", "tf32:128", "tf32:256", "bf16", "bf16:128", "bf16:256", "fp32")


def _uniform(eps) -> bool:
    """One blob width for every point (a scalar, or an array of equal entries)."""
    a = np.asarray(eps, dtype=np.float64)
    return a.ndim == 0 or a.size == 0 or bool(np.all(a == a.reshape(-1)[0]))


def bucket_of(n_points: int) -> int:
    """Smallest bucket >= n_points: multiples of 128 on a 2^(1/4) geometric grid."""
    b = BUCKET_BASE
    while b < n_points:
        b = int(math.ceil(b * 2 ** 0.25 / BUCKET_BASE)) * BUCKET_BASE
    return b


@dataclass
class ResistanceRequest:
    kernel: object
    points: np.ndarray
    velocities: np.ndarray
    eps: float
    mu: float = 1.0


@dataclass
class SwimmerRequest:
    shape: object
    x0: np.ndarray
    B: np.ndarray
    eps: float
    mu: float = 1.0
    kernel: object = None


@dataclass
class Result:
    value: object               # forces (N, 3) or a SwimState
    residual: float
    t_arrival: float
    t_start: float
    t_done: float
    slot: int
    bucket: int = 0
    lu: str = ""
    ir_steps: int = 0
    batch: int = 1              # requests factored together with this one (one batched graph)

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival


def plan_bytes(nb_points: int) -> int:
    n = 3 * nb_points
    ld32 = (n + 31) // 32 * 32
    return 8 * n * n + 8 * n * ld32 + 64 * n * 128 + 128 * n * 8 + (64 << 20)


class BucketPlan:
    """Device buffers and captured graphs of one bucket size for up to `cap` systems.

    System z of a group has its own slice of every buffer (points, blob widths, real count,
    K, the FP32 copies, the block inverses, flags, right-hand side, solution).  A group of
    k <= cap requests of the bucket replays one captured graph of k systems: one batched
    assembly launch, one FP32 conversion pass, and the batched tensor-core LU, whose steps
    each cover all k systems.  Each system is then refined by its own captured FP64
    refinement graph.  cap = 1 (and the FP32 LU, which is not batched) captures the
    single-system graph."""

    def __init__(self, kernel, nb_points: int, mu: float, lu: str, stream, uniform: bool = False, cap: int = 1):
        L = load()
        self.kernel, self.mu, self.lu, self.nbp = kernel, mu, lu, nb_points
        self.uniform = uniform  # one blob width for every point: the symmetric assembly, half the pairs
        self.kind, self.are, self.aim = kernel_params(kernel)
        self.cap = 1 if lu.startswith("fp32") else max(1, int(cap))
        dev = torch.device("cuda", torch.cuda.current_device())
        n = 3 * nb_points
        c = self.cap
        self.n = n
        self.ld32 = (n + 31) // 32 * 32
        self.pts = torch.zeros((c, nb_points, 3), dtype=torch.float64, device=dev)
        self.eps = torch.ones((c, nb_points), dtype=torch.float64, device=dev)
        self.n_real = torch.zeros(c, dtype=torch.int64, device=dev)
        self.K = torch.empty((c, n, n), dtype=torch.float64, device=dev)
        self.K32 = torch.empty((c, n, self.ld32), dtype=torch.float32, device=dev)
        self.A32 = torch.empty((c, n, self.ld32), dtype=torch.float32, device=dev)  # inner GMRES matvecs
        self.dinv = torch.empty((c, L.flg_lu_lowp_dinv_elems(n)), dtype=torch.float32, device=dev)
        self.flags = torch.zeros((c, 2), dtype=torch.int32, device=dev)
        mode = lu_mode(lu)
        # sized for either tensor-core precision, so the autotuner can switch modes on one plan
        if c == 1:
            self.lu_bytes = max(L.flg_lu_factor_lowp_workspace(n, LU_MODE[m]) for m in ("tf32", "bf16"))
        else:
            self.lu_bytes = max(L.flg_lu_factor_lowp_batched_workspace(n, c, LU_MODE[m]) for m in ("tf32", "bf16"))
        self.lu_ws = dv.workspace(self.lu_bytes)
        self.b = torch.zeros((c, n), dtype=torch.float64, device=dev)
        self.x = torch.zeros((c, n), dtype=torch.float64, device=dev)
        self.graphs = {}  # systems in the group -> captured graph
        self.irs = []     # per system: the captured refinement (after capture())
        self.rtol_ir = 1e-12  # the refinement's target: rtol / 100 for the server's rtol 1e-10
        self.stream = stream
        self.mode = mode
        self.count = 0    # systems of the current group

    @property
    def graph(self):
        """The graph of a single system (None before capture() or when capture failed)."""
        return self.graphs.get(1)

    def _st(self):
        return ctypes.c_void_p(self.stream.cuda_stream)

    def _run(self, k: int):
        L = load()
        st = self._st()
        n = self.n
        if self.cap == 1:
            asm = L.flg_assemble_bucket_uniform if self.uniform else L.flg_assemble_bucket
            check(asm(self.kind, self.are, self.aim, dv.ptr(self.pts), dv.ptr(self.eps), dv.ptr(self.n_real),
                      self.nbp, float(self.mu), dv.ptr(self.K), F64, n, st), "bucket assembly")
        else:
            check(L.flg_assemble_bucket_batched(self.kind, self.are, self.aim, dv.ptr(self.pts), dv.ptr(self.eps),
                                                int(self.uniform), dv.ptr(self.n_real), self.nbp, k, float(self.mu),
                                                dv.ptr(self.K), F64, n, n * n, st), "bucket assembly")
        check(L.flg_convert_f64_f32x2(k * n, n, dv.ptr(self.K), n, dv.ptr(self.K32), dv.ptr(self.A32), self.ld32,
                                      st), "convert")
        if self.cap == 1:
            check(L.flg_lu_factor_lowp_async(n, dv.ptr(self.K32), self.ld32, self.mode, dv.ptr(self.dinv),
                                             dv.ptr(self.flags), dv.ptr(self.lu_ws), self.lu_bytes, st), "LU")
        else:
            check(L.flg_lu_factor_lowp_batched_async(n, k, dv.ptr(self.K32), self.ld32, n * self.ld32, self.mode,
                                                     dv.ptr(self.dinv), dv.ptr(self.flags), dv.ptr(self.lu_ws),
                                                     self.lu_bytes, st), "batched LU")

    def set_lu(self, lu: str):
        """Switch the LU mode of an uncaptured plan (the autotuner's candidates)."""
        if self.graphs:
            raise RuntimeError("the LU mode of a captured plan is fixed")
        if self.cap > 1 and lu.startswith("fp32"):
            raise ValueError("the FP32 LU is not batched")
        self.lu, self.mode = lu, lu_mode(lu)

    def _capture_group(self, k: int):
        L = load()
        h = ctypes.c_void_p(0)
        args = (self.kind, self.are, self.aim, dv.ptr(self.pts), dv.ptr(self.eps), int(self.uniform),
                dv.ptr(self.n_real), self.nbp)
        tail = (float(self.mu), dv.ptr(self.K), dv.ptr(self.A32), dv.ptr(self.K32), self.ld32, self.mode,
                dv.ptr(self.dinv), dv.ptr(self.flags), dv.ptr(self.lu_ws), self.lu_bytes, self._st(), ctypes.byref(h))
        if self.cap == 1:
            st = L.flg_bucket_graph_create(*args, *tail)
        else:
            st = L.flg_bucket_batch_graph_create(*args, k, *tail)
        if st != 0 or not h.value:
            raise RuntimeError(L.flg_last_error().decode(errors="replace"))
        self.graphs[k] = h.value

    def capture(self):
        """Capture assembly -> FP32 copy -> tensor-core LU as a CUDA graph (in the library,
        thread-local capture mode) for every group size up to cap, and each system's
        refinement.  On failure the plan stays eager."""
        try:
            for k in range(1, self.cap + 1):
                self._capture_group(k)
        except RuntimeError as e:
            self.capture_error = str(e)
            for h in self.graphs.values():
                load().flg_graph_destroy(ctypes.c_void_p(h))
            self.graphs = {}
            return
        # the refinement as a second graph over the same buffers (conditional loops steered
        # on the device): a request then costs one host synchronization, at the end
        from .core import IrGraph

        try:
            self.irs = [IrGraph(self.K[z], self.A32[z], self.K32[z], self.ld32, self.dinv[z], self.b[z], self.x[z],
                                self.rtol_ir, stream=self.stream) for z in range(self.cap)]
        except (RuntimeError, ValueError) as e:
            for ir in self.irs:
                ir.close()
            self.irs = []
            self.capture_error = str(e)

    def __del__(self):
        for ir in getattr(self, "irs", []):
            ir.close()
        for h in getattr(self, "graphs", {}).values():
            try:
                load().flg_graph_destroy(ctypes.c_void_p(h))
            except Exception:  # noqa: BLE001 - interpreter shutdown
                pass

    def factor(self, X: torch.Tensor, eps: torch.Tensor):
        self.factor_group([(X, eps)])

    def factor_group(self, items):
        """Factor the systems of a group of k <= cap requests ((points, blob widths) each):
        one replay of the k-system graph (captured on first use), or the eager sequence."""
        k = len(items)
        if not 1 <= k <= self.cap:
            raise ValueError(f"a group of {k} systems on a plan of {self.cap}")
        Ns = []
        for z, (X, eps) in enumerate(items):
            N = X.shape[0]
            self.pts[z, :N].copy_(X)
            self.eps[z, :N].copy_(eps)
            Ns.append(N)
        if k == 1:
            self.n_real[:1].fill_(Ns[0])
        else:
            self.n_real[:k].copy_(torch.tensor(Ns, dtype=torch.int64), non_blocking=False)
        self.count = k
        if self.graph is not None:
            if k not in self.graphs:
                self._capture_group(k)
            check(load().flg_graph_launch(ctypes.c_void_p(self.graphs[k]), self._st()), "graph launch")
        else:
            self._run(k)

    def _flags(self, z):
        flags = self.flags[z].cpu()
        if int(flags[1]) or int(self.flags[0, 1]):
            raise RuntimeError("low-precision LU: a bounded device wait timed out")
        if int(flags[0]):
            raise np.linalg.LinAlgError(f"zero pivot at row {int(flags[0]) - 1} in the low-precision LU")

    def solve(self, U: torch.Tensor, rtol: float, restart: int = 60, maxiter: int = 200, z: int = 0):
        if self.irs and rtol * 1e-2 == self.rtol_ir:
            return self._solve_graph(U, rtol, z)
        L = load()
        N = U.shape[0]
        b, x = self.b[z], self.x[z]
        b.zero_()
        b[:3 * N].copy_(U.reshape(-1))
        x.zero_()
        self._flags(z)
        nbytes = L.flg_gmres_ir_dense_workspace(self.n, restart)
        ws = dv.workspace(nbytes)
        iters, outer, resid = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
        from .core import _accept

        st = L.flg_gmres_ir_dense(self.n, dv.ptr(self.K[z]), self.n, dv.ptr(self.A32[z]), self.ld32,
                                  dv.ptr(self.K32[z]), self.ld32, dv.ptr(self.dinv[z]), dv.ptr(b), dv.ptr(x),
                                  rtol * 1e-2, restart, maxiter, ctypes.byref(iters), ctypes.byref(outer),
                                  ctypes.byref(resid), dv.ptr(ws), nbytes, self._st())
        _accept(st, resid.value, rtol, "GMRES-IR")
        return x[:3 * N].reshape(N, 3).clone(), iters.value, outer.value, resid.value

    def _solve_graph(self, U: torch.Tensor, rtol: float, z: int):
        """The captured refinement of system z: one replay, then the LU's flags and the
        refinement's outcome."""
        self.launch_refinement(U, z)
        return self.refinement_result(U.shape[0], rtol, z)

    def launch_refinement(self, U: torch.Tensor, z: int):
        N = U.shape[0]
        b = self.b[z]
        b.zero_()
        b[:3 * N].copy_(U.reshape(-1))
        self.irs[z].launch(self.stream)

    def refinement_result(self, N: int, rtol: float, z: int):
        from .core import _accept

        st, it, outer, resid = self.irs[z].result(self.stream)
        self._flags(z)
        _accept(st, resid, rtol, "GMRES-IR")
        return self.x[z, :3 * N].reshape(N, 3).clone(), it, outer, resid


class SolveServer:
    """Continuous-batching server: submit() returns a Future of a Result.

    Bucket plans live in a shared pool, counted against the HBM budget: a
    plan is checked out by one slot for one group of requests and then
    returned; free plans are evicted least-recently-used when a new plan or a
    swimmer system needs the memory.  The scheduler takes the oldest request,
    preferring, within a look-ahead window, one whose bucket has a free plan,
    and adds up to `batch` - 1 pending requests of the same plan key (kernel,
    bucket, mu, LU mode, one blob width or not) for buckets of at most
    `batch_points` points: the group is factored by one replay of the batched
    graph.  Nothing waits for a group to fill."""

    def __init__(self, slots: int = 6, hbm_budget_gb: float = 150.0, rtol: float = 1e-10, graphs: bool = True,
                 lu: str = "auto", lookahead: int = 16, batch: int = 4, batch_points: int = 1280):
        self.slots = slots
        self.budget = int(hbm_budget_gb * 2**30)
        self.rtol = rtol
        self.graphs = graphs
        self.lu = lu
        self.lookahead = lookahead
        if not 1 <= int(batch) <= 64:
            raise ValueError(f"batch must lie in [1, 64] (systems per batched factorization), got {batch}")
        self.batch = int(batch)
        self.batch_points = batch_points
        self._pending = []            # [(request, future, t_arrival, bucket, group key)]
        self._cv = threading.Condition()
        self._used = 0                # bytes of pooled plans + in-flight swimmer systems
        self._free = {}               # plan key -> [free BucketPlan], most recently used last
        self._lru = []                # free plans, least recently used first
        self._busy = [False] * slots
        self._tuned = {}              # (kernel kind, bucket) -> LU mode name, e.g. "tf32:256"
        self._closed = False
        self.stats = {"graph_replays": 0, "eager_factors": 0, "captures": 0, "capture_errors": [], "plans_built": 0,
                      "plans_evicted": 0, "tuned": {}, "groups": {}}
        self._dev = self._device()
        self._threads = [threading.Thread(target=self._worker, args=(s,), daemon=True) for s in range(slots)]
        for t in self._threads:
            t.start()

    # ---- public -----------------------------------------------------------------
    def submit(self, req, t_arrival: float | None = None) -> Future:
        fut = Future()
        t = time.perf_counter() if t_arrival is None else t_arrival
        b = bucket_of(len(req.points)) if isinstance(req, ResistanceRequest) else 0
        g = self._group_key(req, b)
        with self._cv:
            self._pending.append((req, fut, t, b, g))
            self._cv.notify_all()
        return fut

    def close(self):
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- plan pool (lock held) ----------------------------------------------------------
    def _key(self, req, b):
        """Pool key of the plan a request runs on: resistance plans per (kernel, bucket, mu, LU
        mode); swimmer plans per (kernel, force and quadrature point counts, eps, mu)."""
        if isinstance(req, ResistanceRequest):
            lu = self._lu_for(req, b) or "tune"
            return ("res", kernel_params(req.kernel)[0], b, float(req.mu), lu, _uniform(req.eps))
        kind = kernel_params(req.kernel if req.kernel is not None else Stokeslet3D())[0]
        return ("swim", kind, len(req.shape.x), len(req.shape.X), float(req.eps), float(req.mu))

    @staticmethod
    def _group_key(req, b):
        """Requests with equal group keys run on the same plan key (the LU mode is tuned per
        kernel and bucket; swimmers of one shape size, blob width and viscosity share one), so
        they can share a batched plan."""
        if not isinstance(req, ResistanceRequest):
            kind = kernel_params(req.kernel if req.kernel is not None else Stokeslet3D())[0]
            return ("swim", kind, len(req.shape.x), len(req.shape.X), float(req.eps), float(req.mu))
        return (kernel_params(req.kernel)[0], b, float(req.mu), _uniform(req.eps))

    def _cap(self, key, b):
        """Systems per plan of this key: `batch` for swimmer plans (captured graphs) and for
        tuned tensor-core resistance plans of at most `batch_points` points, else 1."""
        if self.batch == 1:
            return 1
        if key[0] == "swim":
            return self.batch if self.graphs else 1
        if b > self.batch_points:
            return 1
        lu = key[4]
        return 1 if lu == "tune" or lu.startswith("fp32") else self.batch

    @staticmethod
    def _need(req, b):
        if isinstance(req, ResistanceRequest):
            return plan_bytes(b)
        n = 3 * len(req.shape.x) + 6
        return 16 * n * n + (64 << 20)

    def _evict_free(self, need):
        """Free least-recently-used idle plans until `need` more bytes fit the budget."""
        while self._used + need > self.budget and self._lru:
            plan = self._lru.pop(0)
            self._free[plan.key].remove(plan)
            self._used -= plan.nbytes
            self.stats["plans_evicted"] += 1

    def _pick(self, slot):
        """Oldest admissible request, preferring one with a free plan within the look-ahead window,
        plus pending requests of its group key up to the plan's capacity.  A new plan holds as
        many systems as the key allows (_cap) and the budget leaves room for.
        Returns ([(request, future, t_arrival)], bucket, plan or None, reserved bytes, systems per
        plan) or None."""
        cand = None
        for k, (req, fut, t, b, g) in enumerate(self._pending[: self.lookahead]):
            if self._free.get(self._key(req, b)):
                cand = k
                break
        if cand is None:
            cand = 0
        req, fut, t, b, g = self._pending[cand]
        key = self._key(req, b)
        plan, reserved = None, 0
        if self._free.get(key):
            plan = max(self._free[key], key=lambda p: getattr(p, "cap", 1))
            self._free[key].remove(plan)
            self._lru.remove(plan)
            cap = getattr(plan, "cap", 1)
        else:
            cap, need1 = self._cap(key, b), self._need(req, b)
            while cap > 1 and self._used + need1 * cap > self.budget:
                cap -= 1
            need = need1 * cap
            if self._used + need > self.budget:
                self._evict_free(need)
                if self._used + need > self.budget and any(self._busy):
                    return None  # wait until running requests release memory
            self._used += need
            reserved = need
        group = [self._pending.pop(cand)[:3]]
        k = 0
        while len(group) < cap and k < len(self._pending):
            if self._pending[k][4] == g:
                group.append(self._pending.pop(k)[:3])
            else:
                k += 1
        self._busy[slot] = True
        return group, b, plan, reserved, cap

    # ---- device hooks (overridden by the scheduler's CPU test) ---------------------------
    def _device(self):
        return torch.cuda.current_device()

    def _make_stream(self):
        torch.cuda.set_device(self._dev)
        return torch.cuda.Stream()

    def _run_group(self, slot, stream, reqs, b, plan, cap=1):
        """A group of requests of one plan key (one request, or up to the plan's capacity; a new
        plan holds `cap` systems): ([Result or exception per request], plan)."""
        with torch.cuda.stream(stream):
            if isinstance(reqs[0], ResistanceRequest):
                res, plan = self._resistance(slot, stream, reqs, b, plan, cap)
            else:
                res, plan = self._swimmers(stream, reqs, plan, cap)
            stream.synchronize()
        return res, plan

    def _worker(self, slot):
        stream = self._make_stream()
        while True:
            with self._cv:
                while True:
                    if self._pending:
                        item = self._pick(slot)
                        if item is not None:
                            break
                    elif self._closed:
                        return
                    self._cv.wait(timeout=0.05)
            group, b, plan, reserved, cap = item
            reqs = [r for r, _, _ in group]
            t0 = time.perf_counter()
            try:
                res, plan = self._run_group(slot, stream, reqs, b, plan, cap)
                t1 = time.perf_counter()
                for (req, fut, t_arr), r in zip(group, res):
                    if isinstance(r, Exception):
                        fut.set_exception(r)
                        continue
                    r.t_arrival, r.t_start, r.t_done, r.slot, r.batch = t_arr, t0, t1, slot, len(group)
                    fut.set_result(r)
                with self._cv:
                    self.stats["groups"][len(group)] = self.stats["groups"].get(len(group), 0) + 1
                    if plan is not None:  # back into the pool, counted against the budget
                        if reserved:  # built for this group: count what it holds
                            nb = getattr(plan, "nbytes", None) or reserved
                            self._used += nb - reserved
                            plan.nbytes = nb
                        plan.key = self._key(reqs[0], b)
                        self._free.setdefault(plan.key, []).append(plan)
                        self._lru.append(plan)
                    else:
                        self._used -= reserved
            except Exception as e:  # noqa: BLE001 - delivered to the caller
                with self._cv:
                    self._used -= reserved if reserved else getattr(plan, "nbytes", 0)
                for _, fut, _ in group:
                    if not fut.done():
                        fut.set_exception(e)
            finally:
                with self._cv:
                    self._busy[slot] = False
                    self._cv.notify_all()

    # ---- request pipelines ------------------------------------------------------------
    def _lu_for(self, req, b):
        if self.lu != "auto":
            return self.lu
        return self._tuned.get((kernel_params(req.kernel)[0], b))

    def _resistance(self, slot, stream, reqs, b, plan, cap=1):
        """Resistance requests of one plan key: one (batched) factorization of the group, then
        each system's refinement.  A request whose system fails gets its exception in place of
        a Result."""
        dev = torch.device("cuda", self._dev)
        items, Us = [], []
        for req in reqs:
            X = torch.as_tensor(np.ascontiguousarray(req.points, dtype=np.float64)).to(dev, non_blocking=True)
            U = torch.as_tensor(np.ascontiguousarray(req.velocities, dtype=np.float64)).to(dev, non_blocking=True)
            N = X.shape[0]
            e = torch.full((N,), float(req.eps), dtype=torch.float64, device=dev) if np.ndim(req.eps) == 0 else \
                torch.as_tensor(np.asarray(req.eps, dtype=np.float64)).to(dev)
            items.append((X, e))
            Us.append(U)
        req = reqs[0]
        if plan is None:
            lu = self._lu_for(req, b)
            if lu is None:  # autotune this bucket (precision x tile width), keep the fastest that converges
                lu = self._autotune(req, b, stream, items[0][0], items[0][1], Us[0])
                with self._cv:
                    self._tuned[(kernel_params(req.kernel)[0], b)] = lu
            uniform = _uniform(req.eps)
            plan = BucketPlan(req.kernel, b, req.mu, lu, stream, uniform=uniform, cap=max(cap, len(reqs)))
            plan.nbytes = self._need(req, b) * plan.cap
            with self._cv:
                self.stats["plans_built"] += 1
            if self.graphs:
                plan.stream = stream
                plan.rtol_ir = self.rtol * 1e-2
                plan.capture()
                with self._cv:
                    self.stats["captures"] += 1
                    if plan.graph is None:
                        self.stats["capture_errors"].append(getattr(plan, "capture_error", "?"))
        plan.stream = stream  # a pooled plan runs on the stream of the slot that checked it out
        plan.factor_group(items)
        with self._cv:
            self.stats["graph_replays" if plan.graph is not None else "eager_factors"] += 1
        outs = []
        if plan.irs and self.rtol * 1e-2 == plan.rtol_ir:
            for z, U in enumerate(Us):  # every refinement queued, then the results in order
                plan.launch_refinement(U, z)
            for z, U in enumerate(Us):
                try:
                    outs.append(plan.refinement_result(U.shape[0], self.rtol, z))
                except Exception as e:  # noqa: BLE001 - this request's own failure
                    outs.append(e)
        else:
            for z, U in enumerate(Us):
                try:
                    outs.append(plan.solve(U, self.rtol, z=z))
                except Exception as e:  # noqa: BLE001
                    outs.append(e)
        # resid: the refinement's last ||U - K F|| / ||U|| with the FP64 K (padding rows are identity
        # with zero right-hand side, so this is the residual of the unpadded system)
        res = [o if isinstance(o, Exception) else Result(o[0].cpu().numpy(), o[3], 0, 0, 0, slot, b, plan.lu, o[2])
               for o in outs]
        return res, plan

    def _autotune(self, req, b, stream, X, e, U):
        """Time factor + solve of this request for every candidate LU mode on one eager plan
        (one untimed run each first); the fastest whose residual meets rtol wins."""
        p = BucketPlan(req.kernel, b, req.mu, "tf32", stream, uniform=_uniform(req.eps))
        best = None
        for lu in TUNE_CANDIDATES:
            p.set_lu(lu)
            dt = math.inf
            for rep in range(2):
                stream.synchronize()  # only this slot's stream: another slot may be capturing a graph
                t0 = time.perf_counter()
                p.factor(X, e)
                x, it, outer, resid = p.solve(U, self.rtol)
                stream.synchronize()
                if rep:
                    dt = time.perf_counter() - t0
            if resid <= self.rtol and (best is None or dt < best[0]):
                best = (dt, lu)
        del p
        lu = best[1] if best else "tf32"
        with self._cv:
            self.stats["tuned"][f"{kernel_params(req.kernel)[0]}:{b}"] = lu
        return lu

    def _swimmers(self, stream, reqs, plan, cap=1):
        """Free-swimmer instants of one shape size on a pooled SwimmerPlan: one captured graph
        of the group's systems (nearest maps -> nearest-neighbour assemblies -> constraint rows
        -> FP32 copies -> batched tensor-core LU) replayed with the requests' points, then each
        system's FP64 GMRES-IR.  A request whose system fails gets its exception."""
        from .swimming import SwimmerPlan, SwimState, swimming_problem

        if not self.graphs:  # eager: the mixed-precision swimmer solve, no plan (groups of one)
            out = []
            for req in reqs:
                st = swimming_problem(req.shape, req.x0, req.B, req.eps, req.mu, req.kernel, precision="mixed",
                                      rtol=self.rtol)
                out.append(Result(st, float("nan"), 0, 0, 0, 0, 0, "tf32", 0))
            return out, None
        req = reqs[0]
        kernel = Stokeslet3D() if req.kernel is None else req.kernel
        items, geo = [], []
        for r in reqs:
            x0 = np.asarray(r.x0, float)
            B = np.asarray(r.B, float)
            x = x0 + np.asarray(r.shape.x, float) @ B.T
            X = x0 + np.asarray(r.shape.X, float) @ B.T
            v = np.asarray(r.shape.v, float) @ B.T
            rhs = np.zeros(3 * len(x) + 6)
            rhs[:3 * len(x)] = v.ravel()
            items.append((x, X, x0, rhs))
            geo.append((x, X))
        N = len(items[0][0])
        if plan is None:
            plan = SwimmerPlan(kernel, N, len(items[0][1]), req.eps, req.mu, stream=stream, cap=max(cap, len(reqs)))
            plan.nbytes = self._need(req, 0) * plan.cap
            with self._cv:
                self.stats["plans_built"] += 1
                self.stats["captures"] += 1
        outs = plan.solve_group(items, rtol=self.rtol, stream=stream)
        with self._cv:
            self.stats["graph_replays"] += 1
        res = [o if isinstance(o, Exception) else
               Result(SwimState(o[0], o[1], o[2], x, X, o[3]), o[4], 0, 0, 0, 0, 0, "tf32", 0)
               for o, (x, X) in zip(outs, geo)]
        return res, plan


# ---- the served mixed workload ------------------------------------------------------
def make_requests(n_requests=4096, seed=0):
    """Synthetic mixed workload: 75 % rigid bodies (sphere, or prolate spheroid with aspect ratio
    U[1, 5] and random orientation; N log-uniform in [256, 6144]; free space or a wall at gap
    U[0.05, 2]; eps / spacing U[0.15, 0.4]; translation or rotation), 25 % biflagellate swimmers."""
    from .geometry import biflagellate_shape, fibonacci_sphere, mean_nn_spacing

    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(n_requests):
        if rng.random() < 0.25:
            t = rng.uniform(0, 1)
            shape = biflagellate_shape(t)
            B = np.linalg.qr(rng.normal(size=(3, 3)))[0]
            B *= np.sign(np.linalg.det(B))
            reqs.append(SwimmerRequest(shape, np.zeros(3), B, 0.02))
            continue
        N = int(round(math.exp(rng.uniform(math.log(256), math.log(6144)))))
        unit = fibonacci_sphere(N)
        if rng.random() < 0.5:
            a = rng.uniform(1, 5)
            R = np.linalg.qr(rng.normal(size=(3, 3)))[0]
            pts = (unit * np.array([a, 1.0, 1.0])) @ R.T
        else:
            pts = unit
        wall = rng.random() < 0.5
        if wall:
            pts = pts + np.array([0, 0, -pts[:, 2].min() + rng.uniform(0.05, 2.0)])
        sp = mean_nn_spacing(pts)
        eps = rng.uniform(0.15, 0.4) * sp
        if rng.random() < 0.5:
            U = np.tile(rng.normal(size=3), (N, 1))
        else:
            w = rng.normal(size=3)
            U = np.cross(w, pts - pts.mean(0))
        from .kernels import WallStokeslet3D

        reqs.append(ResistanceRequest(WallStokeslet3D() if wall else Stokeslet3D(), pts, U, eps))
    return reqs


def _warm(srv, reqs):
    """One request per (type, bucket, kernel) in use: builds and autotunes their plans."""
    warm = {}
    for r in reqs:
        key = (type(r).__name__, bucket_of(len(r.points)) if isinstance(r, ResistanceRequest) else 0,
               type(getattr(r, "kernel", None)).__name__)
        warm.setdefault(key, r)
    for f in [srv.submit(r) for r in warm.values()]:
        f.result()


def _poisson_run(srv, reqs, rate, seed):
    """Submit reqs at Poisson arrival times (rate per second); latency percentiles and throughput."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(reqs))
    t0 = time.perf_counter()
    arrivals = t0 + np.cumsum(gaps)
    futs = []
    for r, ta in zip(reqs, arrivals):
        now = time.perf_counter()
        if ta > now:
            time.sleep(ta - now)
        futs.append(srv.submit(r, t_arrival=ta))
    res = [f.result() for f in futs]
    t_end = max(x.t_done for x in res)
    lat = np.array([x.latency for x in res]) * 1e3
    resid = np.array([x.residual for x in res if np.isfinite(x.residual)])
    return {"rate_per_s": rate, "requests": len(res), "solves_per_s": len(res) / (t_end - t0),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_residual": float(resid.max()) if len(resid) else None}


def serve_run(n_requests=512, rate=200.0, slots=6, seed=0, batch=4, warm_pass=True):
    """A served run of the mixed workload at one arrival rate: p50 / p99 latency, solves/s and the
    server's counters.  Untimed first: one request per bucket in use (plans built, LU modes
    autotuned) and, with warm_pass, the same arrival stream once, which builds the plan pool that
    concurrent requests need, so that the timed pass measures steady-state serving."""
    reqs = make_requests(n_requests, seed=seed)
    with SolveServer(slots=slots, batch=batch) as srv:
        _warm(srv, reqs)
        if warm_pass:
            _poisson_run(srv, reqs, rate, int(rate) + 1)
        built = srv.stats["plans_built"]
        line = _poisson_run(srv, reqs, rate, int(rate))
        stats = dict(srv.stats)
        stats["plans_built_timed"] = stats["plans_built"] - built
    line["workload"] = (f"served mixed workload: {n_requests} requests (75% rigid bodies N log-uniform [256, 6144], "
                        f"25% biflagellate swimmers), Poisson arrivals at {rate:g}/s, {slots} slots, groups of up to "
                        f"{batch} same-bucket requests, HBM budget 150 GB"
                        + (", steady state (plan pool built by an untimed pass of the same stream)" if warm_pass else ""))
    line["server_stats"] = {k: (v if not isinstance(v, list) else len(v)) for k, v in stats.items()}
    return line


def bench_serving(args):
    """Poisson arrivals at rates {50, 200, 800}/s over the mixed workload, served with continuous
    batching; p50 / p99 latency and solves/s, and the one-solve-at-a-time FP64 GPU service time on a
    sample of the same requests."""
    import json

    import fluidlets_gb300 as fl

    n_req = getattr(args, "n_points", None) or 4096
    reqs = make_requests(n_req)
    out = {"workload": f"served mixed workload: {n_req} requests (75% rigid bodies N log-uniform [256, 6144], "
                       "25% biflagellate swimmers), Poisson arrivals, HBM budget 150 GB, steady state (plan pool "
                       "built by an untimed pass of the stream)", "rates": []}
    slots = getattr(args, "slots", 6)
    batch = getattr(args, "batch", 4)
    rates = [float(r) for r in str(getattr(args, "rates", "50,200,800")).split(",")]
    out["slots"], out["batch"] = slots, batch
    with SolveServer(slots=slots, batch=batch) as srv:
        srv_stats = srv.stats
        # warm-up and autotuning of the buckets in use, then one untimed pass of the stream at the
        # first rate (it builds the plan pool), outside the timed runs: steady-state serving
        _warm(srv, reqs)
        _poisson_run(srv, reqs, rates[0], int(rates[0]) + 1)
        for rate in rates:
            line = _poisson_run(srv, reqs, rate, int(rate))
            out["rates"].append(line)
            print(json.dumps(line), flush=True)
    out["server_stats"] = {k: (v if not isinstance(v, list) else len(v)) for k, v in srv_stats.items()}
    if getattr(args, "no_extras", False):
        print(json.dumps(out), flush=True)
        return
    # one-solve-at-a-time FP64 GPU service times on a stratified sample
    sample = reqs[:: max(1, len(reqs) // 48)]
    times = []
    for r in sample:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if isinstance(r, ResistanceRequest):
            fl.resistance(r.kernel, r.points, r.velocities, r.eps, method="lu")
        else:
            fl.swimming_problem(r.shape, r.x0, r.B, r.eps)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    mean_fp64 = float(np.mean(times))
    out["fp64_one_at_a_time"] = {"sample_requests": len(sample), "mean_service_ms": 1e3 * mean_fp64,
                                 "max_solves_per_s": 1.0 / mean_fp64}
    print(json.dumps(out), flush=True)
