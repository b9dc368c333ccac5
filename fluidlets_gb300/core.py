"""The reference's operator API on the GPU: evaluate, assemble, resistance.

Signatures, defaults, dtype rules and exceptions follow the reference package
``fluidlets`` (``core/_common.py``, ``core/matvec.py``, ``core/assemble.py``,
``core/solve.py``); the O(MN) loops, the dense LU and GMRES run in
``libfluidlets_gb300.so`` on the current CUDA device.

NumPy in gives NumPy out (host <-> device copies at this boundary); torch CUDA
tensors in give torch CUDA tensors out with no host round trip.

Extensions, all keyword-only with defaults that reproduce the reference:
``precision="fp64" | "mixed"`` (FP32 far field + FP64 near field for sums;
TF32/BF16 tensor-core LU + FP64 GMRES iterative refinement for solves).
"""
from __future__ import annotations

import ctypes
import threading
from dataclasses import dataclass

import numpy as np
import torch

from . import _device as dv
from ._lib import BF16, C128, F32, F64, FLG_ERR_NOT_CONVERGED, KIND, PREC, LinAlgError, check, load, lu_mode
from .kernels import kernel_params

#: above this many unknowns, method="auto" switches from dense LU to GMRES (core/solve.py:20)
DENSE_MAX = 6000


# ---- input normalization (core/_common.py:7-23) ---------------------------
def _points(a, dim=3) -> torch.Tensor:
    if isinstance(a, torch.Tensor):
        t = a.to(dtype=torch.float64)
        if t.dim() == 1:
            t = t.reshape(1, -1)
        if t.dim() != 2 or t.shape[1] != dim:
            raise ValueError(f"expected points of shape (N, {dim}), got {tuple(a.shape)}")
        return dv.to_dev(t, torch.float64)
    arr = np.atleast_2d(np.asarray(a, dtype=np.float64))
    if arr.ndim != 2 or arr.shape[1] != dim:
        raise ValueError(f"expected points of shape (N, {dim}), got {arr.shape}")
    return dv.to_dev(arr, torch.float64)


def _blob_widths(eps, n) -> torch.Tensor:
    if isinstance(eps, torch.Tensor):
        e = eps.to(dtype=torch.float64)
        return dv.to_dev(torch.broadcast_to(e, (n,)), torch.float64)
    e = np.asarray(eps, dtype=np.float64)
    return dv.to_dev(np.broadcast_to(e, (n,)), torch.float64)


def _prec(precision) -> int:
    if precision not in PREC:
        raise ValueError(f"unknown precision {precision!r} (expected 'fp64' or 'mixed')")
    return PREC[precision]


def _mu(mu):
    m = complex(mu.item() if isinstance(mu, torch.Tensor) else mu)
    if m == 0:
        raise ValueError("mu must be non-zero")
    return m, dv.is_complex_value(mu)


def _out(t: torch.Tensor, where):
    """NumPy for NumPy callers; a torch tensor on the inputs' device otherwise."""
    if where is None:
        return dv.to_host(t)
    return t if where == "cuda" else t.cpu()


# ---- core/matvec.py:24-49 ---------------------------------------------------
def _evaluate_dev(kernel, X, Y, f, e, mu, precision, out=None):
    """Device-level sum: X (M,3), Y (N,3), f (N,3) f64/c128, e (N,) -> (M,3)."""
    kind, are, aim = kernel_params(kernel)
    m, mu_c = _mu(mu)
    M, N = X.shape[0], Y.shape[0]
    fc = f.is_complex()
    lib_complex = fc or aim != 0.0 or m.imag != 0.0
    want_complex = lib_complex or mu_c
    if out is None:
        out = torch.empty((M, 3), dtype=torch.complex128 if lib_complex else torch.float64, device=X.device)
    prec = _prec(precision)
    L = load()
    nbytes = L.flg_evaluate_workspace(kind, M, N, int(fc), aim, prec)
    ws = dv.workspace(nbytes)
    st = L.flg_evaluate(kind, are, aim, dv.ptr(X), M, dv.ptr(Y), dv.ptr(e), N, dv.ptr(f), int(fc), m.real, m.imag,
                        dv.ptr(out), prec, dv.ptr(ws), nbytes, dv.stream())
    check(st, "evaluate")
    if want_complex and not out.is_complex():
        out = out.to(torch.complex128)
    return out


def evaluate(kernel, targets, sources, strengths, eps, mu=1.0, *, precision="fp64"):
    """Field at targets from regularized sources, without storing the matrix.

    Same contract as the reference's ``fluidlets.evaluate``
    (``core/matvec.py:24-49``): (M, 3) array, complex if mu, the strengths or
    the kernel (complex Brinkman alpha) are complex.
    """
    as_torch = dv.home(targets, sources, strengths)
    X = _points(targets, kernel.dim)
    Y = _points(sources, kernel.dim)
    N = Y.shape[0]
    e = _blob_widths(eps, N)
    fc = dv.is_complex_value(strengths)
    f = dv.to_dev(strengths, torch.complex128 if fc else torch.float64).reshape(N, 3)
    return _out(_evaluate_dev(kernel, X, Y, f, e, mu, precision), as_torch)


def evaluate_grid(kernel, axes, sources, strengths, eps, mu=1.0, *, precision="fp64", field=False):
    """Field on the structured grid ``axes = (x, y, z)`` (1-D coordinate arrays).

    Equal to ``evaluate(kernel, grid, ...)`` with the grid the reference's examples build,
    ``np.meshgrid(z, y, x, indexing="ij")`` raveled into ``c_[X, Y, Z]``
    (``examples/glycocalyx_towers/run.py:48-51``): rows in VTK point order, x fastest.  The
    grid points are generated on the device (no host grid array); ``field=True`` returns the
    result shaped (nz, ny, nx, 3).
    """
    as_torch = dv.home(sources, strengths)
    ax = [dv.to_dev(np.asarray(a, float) if not isinstance(a, torch.Tensor) else a, torch.float64).reshape(-1)
          for a in axes]
    if len(ax) != 3:
        raise ValueError("axes must be three 1-D coordinate arrays (x, y, z)")
    nx, ny, nz = (a.shape[0] for a in ax)
    G = torch.empty((nx * ny * nz, 3), dtype=torch.float64, device=ax[0].device)
    check(load().flg_grid_points(dv.ptr(ax[0]), nx, dv.ptr(ax[1]), ny, dv.ptr(ax[2]), nz, dv.ptr(G), dv.stream()),
          "grid points")
    Y = _points(sources, kernel.dim)
    N = Y.shape[0]
    e = _blob_widths(eps, N)
    fc = dv.is_complex_value(strengths)
    f = dv.to_dev(strengths, torch.complex128 if fc else torch.float64).reshape(N, 3)
    u = _evaluate_dev(kernel, G, Y, f, e, mu, precision)
    if field:
        u = u.reshape(nz, ny, nx, 3)
    return _out(u, as_torch)


# ---- core/assemble.py:27-101 ------------------------------------------------
def _uniform_eps(eps):
    """The blob width when it is one number (a scalar, or an array of equal entries on the
    host), else None."""
    if isinstance(eps, torch.Tensor):
        return float(eps) if eps.numel() == 1 else None
    a = np.asarray(eps, dtype=np.float64)
    if a.size == 1:
        return float(a.reshape(-1)[0])
    return float(a.reshape(-1)[0]) if a.size and np.all(a == a.reshape(-1)[0]) else None


def _assemble_dev(kernel, X, Y, e, mu, out_dtype=torch.float64, out=None, ld=None, sym_eps=None, reciprocal=False):
    """sym_eps: the one blob width, when Y is X -- half the pair evaluations (bit-identical for
    the free kernels; for the wall kernel only with reciprocal=True, equal to rounding)."""
    kind, are, aim = kernel_params(kernel)
    m, mu_c = _mu(mu)
    M, N = X.shape[0], Y.shape[0]
    complex_out = aim != 0.0 or m.imag != 0.0
    if complex_out:
        out_dtype = torch.complex128
    code = {torch.float64: F64, torch.complex128: C128, torch.float32: F32, torch.bfloat16: BF16}[out_dtype]
    if out is None:
        out = torch.empty((3 * M, 3 * N), dtype=out_dtype, device=X.device)
        ld = 3 * N
    if sym_eps is not None and Y is X and (kind != KIND["wall"] or reciprocal):
        st = load().flg_assemble_self_uniform(kind, are, aim, dv.ptr(X), N, sym_eps, m.real, m.imag, dv.ptr(out),
                                              code, ld, dv.stream())
    else:
        st = load().flg_assemble(kind, are, aim, dv.ptr(X), M, dv.ptr(Y), dv.ptr(e), N, m.real, m.imag,
                                 dv.ptr(out), code, ld, dv.stream())
    check(st, "assemble")
    if mu_c and not out.is_complex():
        out = out.to(torch.complex128)
    return out


def assemble(kernel, targets, sources, eps, mu=1.0):
    """Dense (3M) x (3N) matrix of ``kernel`` from N sources to M targets (``core/assemble.py:27-46``)."""
    as_torch = dv.home(targets, sources)
    X = _points(targets, kernel.dim)
    Y = _points(sources, kernel.dim)
    e = _blob_widths(eps, Y.shape[0])
    return _out(_assemble_dev(kernel, X, Y, e, mu), as_torch)


def _nearest_dev(Xq: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    out = torch.empty(Xq.shape[0], dtype=torch.int64, device=Xq.device)
    check(load().flg_nearest_neighbors(dv.ptr(Xq), Xq.shape[0], dv.ptr(x), x.shape[0], dv.ptr(out), dv.stream()),
          "nearest_neighbors")
    return out


def nearest_neighbors(quad_points, force_points):
    """Index of the nearest force point for every quadrature point, shape (Q,) (``core/assemble.py:61-65``).

    The reference queries a SciPy k-d tree on the host; here an exhaustive FP64 search on the
    device gives the same indices (the first one on exact ties).
    """
    as_torch = dv.home(quad_points, force_points)
    Xq = _points(quad_points, 3)
    x = _points(force_points, 3)
    if Xq.shape[0] and not x.shape[0]:
        raise ValueError("no force points to search")
    return _out(_nearest_dev(Xq, x), as_torch)


def _assemble_nearest_dev(kernel, X, Xq, nn, n_force, e, mu, out_dtype=torch.float64, out=None, ld=None):
    kind, are, aim = kernel_params(kernel)
    m, mu_c = _mu(mu)
    M, Q = X.shape[0], Xq.shape[0]
    if aim != 0.0 or m.imag != 0.0:
        out_dtype = torch.complex128
    code = {torch.float64: F64, torch.complex128: C128, torch.float32: F32}[out_dtype]
    if out is None:
        out = torch.empty((3 * M, 3 * n_force), dtype=out_dtype, device=X.device)
        ld = 3 * n_force
    L = load()
    nbytes = L.flg_assemble_nearest_workspace(Q, n_force)
    ws = dv.workspace(nbytes)
    st = L.flg_assemble_nearest(kind, are, aim, dv.ptr(X), M, dv.ptr(Xq), dv.ptr(nn), dv.ptr(e), Q, n_force,
                                m.real, m.imag, dv.ptr(out), code, ld, dv.ptr(ws), nbytes, dv.stream())
    check(st, "assemble_nearest")
    if mu_c and not out.is_complex():
        out = out.to(torch.complex128)
    return out


def assemble_nearest(kernel, targets, quad_points, nearest, n_force, eps, mu=1.0):
    """Nearest-neighbour kernel matrix of Gallagher & Smith (2018) (``core/assemble.py:68-101``).

    K[:, j] = sum over k with nearest[k] = j of G(x_i, X_k) / mu.
    """
    as_torch = dv.home(targets, quad_points)
    X = _points(targets, kernel.dim)
    Xq = _points(quad_points, kernel.dim)
    e = _blob_widths(eps, Xq.shape[0])
    nn = dv.to_dev(np.asarray(nearest) if not isinstance(nearest, torch.Tensor) else nearest, torch.int64)
    if nn.numel() != Xq.shape[0]:
        raise ValueError("nearest must have one entry per quadrature point")
    n_force = int(n_force)
    if nn.numel() and (int(nn.min()) < 0 or int(nn.max()) >= n_force):
        raise ValueError("nearest indices must lie in [0, n_force)")
    return _out(_assemble_nearest_dev(kernel, X, Xq, nn, n_force, e, mu), as_torch)


# ---- core/solve.py:23-84 ----------------------------------------------------
@dataclass
class SolveInfo:
    """``core/solve.py:23-27``, plus how the solve was computed."""

    method: str
    iterations: int
    residual: float          # ||K f - U|| / ||U||, FP64 operator
    precision: str = "fp64"
    ir_steps: int = 0        # FP64 refinement steps of the mixed-precision path


def _lu_solve_dev(K: torch.Tensor, U: torch.Tensor) -> torch.Tensor:
    """Dense FP64 LU with partial pivoting (getrf + getrs) on the device; K is overwritten.
    U holds one right-hand side (n values, returned flat) or several as the columns of (n, k)."""
    n = K.shape[0]
    L = load()
    if K.is_complex():
        # complex system through its real 2n x 2n form [[Re, -Im], [Im, Re]]
        R = torch.empty((2 * n, 2 * n), dtype=torch.float64, device=K.device)
        R[:n, :n] = K.real
        R[:n, n:] = -K.imag
        R[n:, :n] = K.imag
        R[n:, n:] = K.real
        b = torch.cat([U.real, U.imag]).to(torch.float64).contiguous() if U.is_complex() else \
            torch.cat([U, torch.zeros_like(U)]).contiguous()
        x = _lu_solve_dev(R, b)
        return torch.complex(x[:n], x[n:])
    piv = torch.empty(n, dtype=torch.int32, device=K.device)
    nbytes = L.flg_lu_factor_f64_workspace(n)
    ws = dv.workspace(nbytes)
    info = ctypes.c_int(0)
    check(L.flg_lu_factor_f64(n, dv.ptr(K), n, dv.ptr(piv), ctypes.byref(info), dv.ptr(ws), nbytes, dv.stream()),
          "LU factorization")
    # the solve overwrites its right-hand side: always work on a copy of U
    B = U.reshape(n, -1).to(torch.float64).clone() if not U.is_complex() else None
    if B is None:  # real matrix, complex right-hand side: two real columns
        B = torch.stack([U.real, U.imag], 1).contiguous()
        check(L.flg_lu_solve_f64(n, 2, dv.ptr(K), n, dv.ptr(piv), dv.ptr(B), 2, dv.stream()), "LU solve")
        return torch.complex(B[:, 0], B[:, 1])
    nrhs = B.shape[1]
    check(L.flg_lu_solve_f64(n, nrhs, dv.ptr(K), n, dv.ptr(piv), dv.ptr(B), nrhs, dv.stream()), "LU solve")
    return B.reshape(-1) if nrhs == 1 else B


def _lowp_factor_dev(K: torch.Tensor, lu_name: str):
    """FP32 copy of K (leading dimension padded to 32) factored without pivoting
    on the tensor cores; returns (K32, ld32, dinv, A32) with A32 an unfactored FP32
    copy of K for the inner matvecs of GMRES-IR."""
    n = K.shape[0]
    L = load()
    ld32 = (n + 31) // 32 * 32
    K32 = torch.empty((n, ld32), dtype=torch.float32, device=K.device)
    A32 = torch.empty_like(K32)
    check(L.flg_convert_f64_f32x2(n, n, dv.ptr(K), K.stride(0), dv.ptr(K32), dv.ptr(A32), ld32, dv.stream()),
          "convert")
    dinv = torch.empty(L.flg_lu_lowp_dinv_elems(n), dtype=torch.float32, device=K.device)
    mode = lu_mode(lu_name)
    nbytes = L.flg_lu_factor_lowp_workspace(n, mode)
    ws = dv.workspace(nbytes)
    info = ctypes.c_int(0)
    check(L.flg_lu_factor_lowp(n, dv.ptr(K32), ld32, mode, dv.ptr(dinv), ctypes.byref(info), dv.ptr(ws), nbytes,
                               dv.stream()), "low-precision LU")
    return K32, ld32, dinv, A32


def _accept(status, resid, required, what):
    """Iterative refinement aims below the requested tolerance; if it stalls at the FP64 floor
    after already meeting `required`, the solve is accepted."""
    if status == FLG_ERR_NOT_CONVERGED and resid <= required:
        return
    check(status, what)


def _gmres_ir_dense_dev(K, K32, ld32, dinv, b, rtol, restart, maxiter, required=None, A32=None):
    """FP64 GMRES-IR on the dense FP64 K, preconditioned by the low-precision factors
    (inner matvecs on the FP32 copy A32 when given)."""
    n = K.shape[0]
    L = load()
    x = torch.zeros_like(b)
    nbytes = L.flg_gmres_ir_dense_workspace(n, restart)
    ws = dv.workspace(nbytes)
    iters, outer, resid = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
    st = L.flg_gmres_ir_dense(n, dv.ptr(K), K.stride(0), dv.ptr(A32), ld32, dv.ptr(K32), ld32, dv.ptr(dinv), dv.ptr(b),
                              dv.ptr(x), rtol,
                              restart, maxiter, ctypes.byref(iters), ctypes.byref(outer), ctypes.byref(resid),
                              dv.ptr(ws), nbytes, dv.stream())
    _accept(st, resid.value, rtol if required is None else required, "GMRES-IR")
    return x, iters.value, outer.value, resid.value


class IrGraph:
    """The FP64 GMRES-IR of K x = b (low-precision factors K32/dinv as preconditioner, inner
    matvecs on the FP32 copy A32) as one replayable CUDA graph over fixed buffers: the loops run
    as conditional graph nodes steered on the device, so ``launch`` costs no host round trip and
    ``result`` reads the outcome once.  b and x are fixed device vectors; write a new right-hand
    side into b before a replay."""

    def __init__(self, K, A32, K32, ld32, dinv, b, x, rtol, m=30, max_outer=60, stream=None):
        L = load()
        n = K.shape[0]
        self.nbytes = L.flg_gmres_ir_graph_workspace(n, m)
        self.ws = dv.workspace(self.nbytes)
        self.graph = ctypes.c_void_p(0)
        st = stream if stream is not None else torch.cuda.current_stream()
        if st.cuda_stream == 0:
            raise ValueError("IrGraph needs a non-default stream")
        check(L.flg_gmres_ir_graph_create(n, dv.ptr(K), K.stride(0), dv.ptr(A32), ld32, dv.ptr(K32), ld32, dv.ptr(dinv),
                                          dv.ptr(b), dv.ptr(x), float(rtol), int(m), int(max_outer), dv.ptr(self.ws),
                                          self.nbytes, ctypes.c_void_p(st.cuda_stream), ctypes.byref(self.graph)),
              "GMRES-IR graph")
        self._keep = (K, A32, K32, dinv, b, x)

    def launch(self, stream):
        check(load().flg_graph_launch(self.graph, ctypes.c_void_p(stream.cuda_stream)), "GMRES-IR graph replay")

    def result(self, stream):
        """(status, inner iterations, refinement steps, final FP64 residual) of the last replay."""
        it, outer, resid = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
        st = load().flg_gmres_ir_graph_result(dv.ptr(self.ws), ctypes.byref(it), ctypes.byref(outer),
                                              ctypes.byref(resid), ctypes.c_void_p(stream.cuda_stream))
        return st, it.value, outer.value, resid.value

    def close(self):
        if self.graph:
            load().flg_graph_destroy(self.graph)
            self.graph = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


class _DensePlan:
    """Device buffers of a mixed-precision dense solve of one size n (K, its two FP32 copies, the
    diagonal-block inverses, the LU workspace, b, x) and the refinement captured over them as an
    IrGraph.  resistance() keeps the last one per host thread, so repeated solves of one size
    reuse both the buffers and the graph (release_plans() frees them)."""

    def __init__(self, n, dev, rtol_ir, m):
        L = load()
        self.n, self.dev, self.rtol_ir, self.m = n, dev, rtol_ir, m
        self.ld32 = (n + 31) // 32 * 32
        self.K = torch.empty((n, n), dtype=torch.float64, device=dev)
        self.K32 = torch.empty((n, self.ld32), dtype=torch.float32, device=dev)
        self.A32 = torch.empty_like(self.K32)
        self.dinv = torch.empty(L.flg_lu_lowp_dinv_elems(n), dtype=torch.float32, device=dev)
        self.lu_bytes = max(L.flg_lu_factor_lowp_workspace(n, lu_mode(x)) for x in ("tf32", "bf16", "fp32"))
        self.lu_ws = dv.workspace(self.lu_bytes)
        self.b = torch.zeros(n, dtype=torch.float64, device=dev)
        self.x = torch.zeros(n, dtype=torch.float64, device=dev)
        self.flags = torch.zeros(2, dtype=torch.int32, device=dev)
        self.factor_graphs = {}  # LU mode -> captured FP32 copies + tensor-core LU
        self.stream = torch.cuda.Stream(device=dev)  # graph capture needs a non-default stream
        torch.cuda.current_stream(dev).synchronize()
        self.ir = IrGraph(self.K, self.A32, self.K32, self.ld32, self.dinv, self.b, self.x, rtol_ir, m=m,
                          stream=self.stream)
        self.stream.synchronize()

    def factor_graph(self, mode):
        """The captured copies + LU for one LU mode (made on first use, on the plan's stream)."""
        g = self.factor_graphs.get(mode)
        if g is None:
            L = load()
            torch.cuda.current_stream(self.dev).synchronize()
            h = ctypes.c_void_p(0)
            check(L.flg_lowp_factor_graph_create(self.n, dv.ptr(self.K), self.n, dv.ptr(self.K32), dv.ptr(self.A32),
                                                 self.ld32, mode, dv.ptr(self.dinv), dv.ptr(self.flags),
                                                 dv.ptr(self.lu_ws), self.lu_bytes,
                                                 ctypes.c_void_p(self.stream.cuda_stream), ctypes.byref(h)),
                  "factor graph")
            self.stream.synchronize()
            g = self.factor_graphs[mode] = h
        return g

    def close(self):
        self.ir.close()
        for g in self.factor_graphs.values():
            load().flg_graph_destroy(g)
        self.factor_graphs = {}


_plans = threading.local()


def release_plans():
    """Free the device buffers that resistance() keeps for repeated mixed-precision solves."""
    p = getattr(_plans, "plan", None)
    if p is not None:
        p.close()
        _plans.plan = None


def _dense_plan(n, dev, rtol_ir, m):
    p = getattr(_plans, "plan", None)
    if p is None or (p.n, p.dev, p.rtol_ir, p.m) != (n, dev, rtol_ir, m):
        release_plans()
        p = _plans.plan = _DensePlan(n, dev, rtol_ir, m)
    return p


def _mixed_lu_planned(kernel, X, e, mu, eps, U, rtol_ir, restart, lu_name, required):
    """The mixed dense solve on the cached plan of its size: assembly into the plan's K, the two
    FP32 copies, the tensor-core LU, then one replay of the captured refinement."""
    L = load()
    n = 3 * X.shape[0]
    p = _dense_plan(n, X.device, rtol_ir, min(restart, 64))
    fg = p.factor_graph(lu_mode(lu_name))
    cur = torch.cuda.current_stream(X.device)
    _assemble_dev(kernel, X, X, e, mu, out=p.K, ld=n, sym_eps=_uniform_eps(eps), reciprocal=True)
    check(L.flg_graph_launch(fg, ctypes.c_void_p(cur.cuda_stream)), "factor graph replay")
    p.b.copy_(U.reshape(-1))
    p.ir.launch(cur)
    st, iters, outer, resid = p.ir.result(cur)  # synchronizes
    flags = p.flags.cpu()
    if int(flags[1]):
        raise RuntimeError("low-precision LU: a bounded device wait timed out")
    if int(flags[0]):
        raise LinAlgError(f"zero or non-finite pivot at row {int(flags[0]) - 1} in the low-precision LU")
    _accept(st, resid, required, "GMRES-IR")
    return p.x.clone(), iters, outer, resid


def _mixed_lu_solve_dev(K: torch.Tensor, U: torch.Tensor, rtol, restart, maxiter, lu_name, required=None):
    """TF32/BF16 tensor-core LU of K (no pivoting) + FP64 GMRES iterative refinement."""
    K32, ld32, dinv, A32 = _lowp_factor_dev(K, lu_name)
    b = U.reshape(-1).to(torch.float64).contiguous()
    return _gmres_ir_dense_dev(K, K32, ld32, dinv, b, rtol, restart, maxiter, required, A32=A32)


def _gmres_dev(kernel, X, e, mu, b, rtol, restart, maxiter, precision, inner_rtol=1e-6, required=None):
    kind, are, aim = kernel_params(kernel)
    m, _ = _mu(mu)
    N = X.shape[0]
    is_c = b.is_complex()
    prec = _prec(precision)
    L = load()
    x = torch.zeros_like(b)
    nbytes = L.flg_gmres_workspace(N, restart, int(is_c), prec)
    ws = dv.workspace(nbytes)
    iters, outer, resid = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
    st = L.flg_gmres(kind, are, aim, dv.ptr(X), dv.ptr(e), N, m.real, m.imag, dv.ptr(b), dv.ptr(x), int(is_c), rtol,
                     restart, maxiter, prec, inner_rtol, ctypes.byref(iters), ctypes.byref(outer),
                     ctypes.byref(resid), dv.ptr(ws), nbytes, dv.stream())
    if required is not None:
        _accept(st, resid.value, required, "GMRES")
    else:
        check(st, "GMRES")
    return x, iters.value, outer.value, resid.value


def resistance(kernel, points, velocities, eps, mu=1.0, method="auto", rtol=1e-10, restart=60, maxiter=200, *,
               precision="fp64", lu="tf32"):
    """Forces that produce the given velocities at the given points (``core/solve.py:30-84``).

    Returns ``(forces (N, 3), SolveInfo)``.  ``method`` is "auto" (LU up to
    ``DENSE_MAX`` unknowns, GMRES above), "lu" or "gmres"; GMRES follows
    ``scipy.sparse.linalg.gmres`` (rtol relative to ||U||, atol 0, ``restart``
    inner iterations per cycle, ``maxiter`` cycles) and raises RuntimeError if
    it does not converge.

    ``precision="mixed"``: LU runs as a TF32 (``lu="tf32"``) or BF16
    (``lu="bf16"``) tensor-core factorization refined by FP64 GMRES to
    ``rtol``; GMRES runs FP32-far/FP64-near matvecs inside FP64 iterative
    refinement.  The residual reported is always that of the FP64 operator.
    """
    as_torch = dv.home(points, velocities)
    X = _points(points, kernel.dim)
    n = X.shape[0]
    e = _blob_widths(eps, n)
    Uc = dv.is_complex_value(velocities)
    m, mu_c = _mu(mu)
    kc = kernel_params(kernel)[2] != 0.0
    cplx = Uc or mu_c or kc
    U = dv.to_dev(velocities, torch.complex128 if Uc else torch.float64).reshape(-1)
    if method == "auto":
        method = "lu" if U.numel() <= DENSE_MAX else "gmres"
    prec = _prec(precision)
    ir_steps = 0
    # mixed precision refines to rtol / 100 so that the FORCE error against the FP64 solve,
    # not only the residual, is within rtol (error <= condition number x residual)
    rtol_ir = rtol * 1e-2 if prec == PREC["mixed"] else rtol
    resid = None
    if method == "lu" and prec == PREC["mixed"] and not kc and not mu_c and not Uc and restart <= 64:
        # real mixed dense solve: the cached plan of this size and its captured refinement
        f, iterations, ir_steps, resid = _mixed_lu_planned(kernel, X, e, mu, eps, U, rtol_ir, restart, lu, rtol)
    elif method == "lu":
        K = _assemble_dev(kernel, X, X, e, mu, sym_eps=_uniform_eps(eps), reciprocal=prec == PREC["mixed"])
        if prec == PREC["mixed"] and not K.is_complex() and not Uc:
            # the refinement's last residual is ||U - K f|| / ||U|| with the FP64 K: reported as is
            f, iterations, ir_steps, resid = _mixed_lu_solve_dev(K, U, rtol_ir, restart, maxiter, lu, required=rtol)
        else:
            f = _lu_solve_dev(K, U.to(K.dtype) if K.is_complex() else U)
            iterations = 1
        del K
    elif method == "gmres":
        b = U.to(torch.complex128) if cplx else U
        f, iterations, ir_steps, resid = _gmres_dev(kernel, X, e, mu, b, rtol_ir, restart, maxiter, precision,
                                                    required=rtol if prec == PREC["mixed"] else None)
    else:
        raise ValueError(f"unknown method {method!r}")
    if cplx and not f.is_complex():
        f = f.to(torch.complex128)
    F = f.reshape(n, -1)
    if resid is None:
        # final FP64 residual, one more O(N^2) sum as in core/solve.py:83 (the GMRES solvers
        # return exactly this quantity, ||b - A x|| / ||b|| with the FP64 operator, already)
        Kf = _evaluate_dev(kernel, X, X, F.contiguous(), e, mu, "fp64").reshape(-1)
        resid = float(torch.linalg.vector_norm(Kf - U) / torch.linalg.vector_norm(U))
    return _out(F, as_torch), SolveInfo(method, int(iterations), resid, precision, int(ir_steps))
