"""Free swimming in Stokes flow (the reference's ``swimming.py``).

Gallagher & Smith, Phys. Rev. Fluids 3, 053101 (2018): at every instant the
forces on N force points, the frame velocity U and angular velocity Omega
solve the (3N + 6)^2 system (``swimming.py:66-102``)

    [ K_nn      | -I   | r x ] [ f     ]   [ B xi_dot ]
    [ count x I |  0   |  0  ] [ U     ] = [ 0        ]
    [ [Xsum x]  |  0   |  0  ] [ Omega ]   [ 0        ]

assembled on the device (``flg_assemble_nearest`` writes K_nn in place,
``flg_swimmer_constraints`` the rest) and solved by the FP64 LU, or by the
tensor-core LU + FP64 GMRES-IR with ``precision="mixed"``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Callable

import numpy as np
import torch

from . import _device as dv
from ._lib import F64, check, load, lu_mode
from .core import _assemble_nearest_dev, _gmres_ir_dense_dev, _lowp_factor_dev, _lu_solve_dev, _prec, nearest_neighbors
from .kernels import Stokeslet3D, kernel_params


@dataclass
class SwimmerShape:
    """Swimmer geometry at one instant, in the body frame: x (N,3) force points,
    v (N,3) their body-frame velocities, X (Q,3) quadrature points."""

    x: np.ndarray
    v: np.ndarray
    X: np.ndarray


@dataclass
class SwimState:
    U: np.ndarray
    Omega: np.ndarray
    forces: np.ndarray
    x: np.ndarray
    X: np.ndarray
    nearest: np.ndarray


def _system_dev(kernel, x, X, nearest, x0, eps, mu):
    """(3N+6)^2 FP64 system on the device."""
    N, Q = len(x), len(X)
    n = 3 * N + 6
    xd = dv.to_dev(x, torch.float64)
    Xd = dv.to_dev(X, torch.float64)
    nn = dv.to_dev(np.asarray(nearest, dtype=np.int64), torch.int64)
    e = dv.to_dev(np.broadcast_to(np.asarray(eps, dtype=np.float64), (Q,)), torch.float64)
    A = torch.empty((n, n), dtype=torch.float64, device=xd.device)
    _assemble_nearest_dev(kernel, xd, Xd, nn, N, e, mu, out=A, ld=n)
    x0c = (ctypes.c_double * 3)(*np.asarray(x0, float))
    check(load().flg_swimmer_constraints(dv.ptr(xd), N, x0c, dv.ptr(Xd), dv.ptr(nn), Q, dv.ptr(A), F64, n,
                                         dv.stream()), "swimmer system")
    return A


def swimming_problem(shape: SwimmerShape, x0, B, eps, mu=1.0, kernel=None, nearest=None, *, precision="fp64",
                     lu="tf32", rtol=1e-10) -> SwimState:
    """Solve the instantaneous free-swimming problem (``swimming.py:66-102``)."""
    kernel = Stokeslet3D() if kernel is None else kernel
    if complex(mu).imag != 0.0:
        raise ValueError("swimming_problem needs a real viscosity")
    x0 = np.asarray(x0, float)
    B = np.asarray(B, float)
    x = x0 + np.asarray(shape.x, float) @ B.T
    X = x0 + np.asarray(shape.X, float) @ B.T
    v = np.asarray(shape.v, float) @ B.T
    if nearest is None:
        nearest = nearest_neighbors(X, x)
    nearest = np.asarray(nearest)
    N = len(x)
    A = _system_dev(kernel, x, X, nearest, x0, eps, mu)
    rhs = torch.zeros(3 * N + 6, dtype=torch.float64, device=A.device)
    rhs[:3 * N] = torch.from_numpy(v.ravel()).to(A.device)
    if _prec(precision) == 1:
        K32, ld32, dinv, A32 = _lowp_factor_dev(A, lu)
        sol, *_ = _gmres_ir_dense_dev(A, K32, ld32, dinv, rhs, rtol * 1e-2, 60, 200, required=rtol, A32=A32)
    else:
        sol = _lu_solve_dev(A, rhs)
    sol = dv.to_host(sol)
    return SwimState(sol[3 * N:3 * N + 3], sol[3 * N + 3:], sol[:3 * N].reshape(N, 3), x, X, nearest)


class SwimmerPlan:
    """Device buffers and captured CUDA graphs of the mixed-precision swimmer system for one
    shape size (N force points, Q quadrature points): nearest map -> nearest-neighbour
    assembly -> constraint rows -> FP32 copies -> tensor-core LU (``flg_swimmer_graph_create``).
    Each ``solve`` writes the stage's points into the buffers, replays the graph and refines
    with FP64 GMRES-IR; ``swim(..., precision="mixed")`` keeps one plan for all stages.

    With cap > 1 the plan holds that many systems and replays, for a group of k <= cap
    swimmers, one graph of k systems (``flg_swimmer_batch_graph_create``: each system's small
    assembly stages, then one FP32 conversion and the batched tensor-core LU); each system is
    then refined by its own captured refinement (``solve_group``)."""

    def __init__(self, kernel, N, Q, eps, mu=1.0, lu="tf32", nearest=None, stream=None, cap=1):
        L = load()
        dev = dv.require_cuda()
        if complex(mu).imag != 0.0:
            raise ValueError("swimming needs a real viscosity")
        self.N, self.Q, self.n = N, Q, 3 * N + 6
        n = self.n
        self.cap = c = 1 if lu.startswith("fp32") else max(1, int(cap))
        self.stream = torch.cuda.Stream(device=dev) if stream is None else stream
        self.last_residual = float("nan")
        f64 = dict(dtype=torch.float64, device=dev)
        self.x = torch.zeros((c, N, 3), **f64)
        self.X = torch.zeros((c, Q, 3), **f64)
        self.x0 = torch.zeros((c, 3), **f64)
        self.e = torch.from_numpy(np.broadcast_to(np.asarray(eps, float), (c, Q)).copy()).to(dev)
        self.fixed = nearest is not None
        self.nn = (torch.from_numpy(np.broadcast_to(np.asarray(nearest, np.int64), (c, Q)).copy()).to(dev)
                   if self.fixed else torch.zeros((c, Q), dtype=torch.int64, device=dev))
        self.A = torch.empty((c, n, n), **f64)
        self.ld32 = (n + 31) // 32 * 32
        self.K32 = torch.empty((c, n, self.ld32), dtype=torch.float32, device=dev)
        self.A32 = torch.empty((c, n, self.ld32), dtype=torch.float32, device=dev)
        self.dinv = torch.empty((c, L.flg_lu_lowp_dinv_elems(n)), dtype=torch.float32, device=dev)
        self.flags = torch.zeros(3 * c, dtype=torch.int32, device=dev)
        mode = lu_mode(lu)
        wb = (L.flg_swimmer_graph_workspace(N, Q, mode) if c == 1
              else L.flg_swimmer_batch_graph_workspace(N, Q, c, mode))
        self.ws = dv.workspace(wb)
        kind, are, aim = kernel_params(kernel)
        self.graphs = {}
        st = ctypes.c_void_p(self.stream.cuda_stream)
        with torch.cuda.stream(self.stream):
            for k in range(1, c + 1):
                h = ctypes.c_void_p(0)
                head = (kind, are, aim, dv.ptr(self.x), N, dv.ptr(self.x0), dv.ptr(self.X), dv.ptr(self.e), Q,
                        dv.ptr(self.nn), 0 if self.fixed else 1)
                tail = (float(complex(mu).real), dv.ptr(self.A), dv.ptr(self.A32), dv.ptr(self.K32), self.ld32, mode,
                        dv.ptr(self.dinv), dv.ptr(self.flags), dv.ptr(self.ws), wb, st, ctypes.byref(h))
                if c == 1:
                    check(L.flg_swimmer_graph_create(*head, *tail), "swimmer graph")
                else:
                    check(L.flg_swimmer_batch_graph_create(*head, k, *tail), "batched swimmer graph")
                self.graphs[k] = h
        self.stream.synchronize()
        # the refinement of each system captured over fixed buffers (right-hand side b, solution sol)
        from .core import IrGraph

        self.b = torch.zeros((c, n), **f64)
        self.sol = torch.zeros((c, n), **f64)
        self.rtol = 1e-10
        self.irs = [IrGraph(self.A[z], self.A32[z], self.K32[z], self.ld32, self.dinv[z], self.b[z], self.sol[z],
                            self.rtol * 1e-2, stream=self.stream) for z in range(c)]
        self.stream.synchronize()

    @property
    def graph(self):
        return self.graphs.get(1)

    def solve(self, x, X, x0, rhs, rtol=1e-10, stream=None):
        """(U, Omega, forces, nearest) for world-frame force points x, quadrature points X,
        origin x0 and right-hand side rhs (3N + 6), on `stream` (default: the plan's own);
        the refinement's final FP64 residual is left in last_residual."""
        out = self.solve_group([(x, X, x0, rhs)], rtol, stream)[0]
        if isinstance(out, Exception):
            raise out
        U, Om, F, nn, self.last_residual = out
        return U, Om, F, nn

    def solve_group(self, items, rtol=1e-10, stream=None):
        """Solve a group of k <= cap swimmer systems ((x, X, x0, rhs) each): one replay of the
        k-system graph, then each system's refinement.  Returns, per system, (U, Omega, forces,
        nearest, residual) or the exception of that system."""
        L = load()
        k = len(items)
        if not 1 <= k <= self.cap:
            raise ValueError(f"a group of {k} swimmers on a plan of {self.cap}")
        st = self.stream if stream is None else stream
        N = self.N
        out = []
        with torch.cuda.stream(st):
            bs = []
            for z, (x, X, x0, rhs) in enumerate(items):
                self.x[z].copy_(torch.from_numpy(np.ascontiguousarray(x, float)))
                self.X[z].copy_(torch.from_numpy(np.ascontiguousarray(X, float)))
                self.x0[z].copy_(torch.from_numpy(np.asarray(x0, float)))
                bs.append(torch.from_numpy(np.ascontiguousarray(rhs, float)).to(self.x.device))
            check(L.flg_graph_launch(self.graphs[k], ctypes.c_void_p(st.cuda_stream)), "swimmer graph replay")
            graph_ir = rtol == self.rtol
            if graph_ir:  # every refinement queued, then one synchronization per result
                for z in range(k):
                    self.b[z].copy_(bs[z])
                    self.irs[z].launch(st)
            fl = self.flags.cpu().numpy()
            for z in range(k):
                try:
                    if fl[2 * k + z]:
                        raise ValueError("nearest indices must lie in [0, n_force)")
                    if fl[2 * z + 1] or fl[1]:
                        raise RuntimeError("low-precision LU: a bounded device wait timed out")
                    if fl[2 * z]:
                        raise np.linalg.LinAlgError(
                            f"zero or non-finite pivot at row {int(fl[2 * z]) - 1} in the low-precision LU")
                    if graph_ir:
                        from .core import _accept

                        status, _, _, resid = self.irs[z].result(st)
                        _accept(status, resid, rtol, "GMRES-IR")
                        sol = self.sol[z]
                    else:
                        sol, _, _, resid = _gmres_ir_dense_dev(self.A[z], self.K32[z], self.ld32, self.dinv[z], bs[z],
                                                               rtol * 1e-2, 60, 200, required=rtol, A32=self.A32[z])
                    sol = dv.to_host(sol)
                    nn = self.nn[z].cpu().numpy()
                    out.append((sol[3 * N:3 * N + 3], sol[3 * N + 3:], sol[:3 * N].reshape(N, 3), nn, resid))
                except Exception as e:  # noqa: BLE001 - this system's own failure
                    out.append(e)
        return out

    def close(self):
        for ir in getattr(self, "irs", []):
            ir.close()
        self.irs = []
        for h in getattr(self, "graphs", {}).values():
            if h:
                load().flg_graph_destroy(h)
        self.graphs = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Trajectory:
    t: np.ndarray
    x0: np.ndarray
    B: np.ndarray


def swim(shape_at: Callable[[float], SwimmerShape], t_span, eps, mu=1.0, x0=(0, 0, 0), B0=None, kernel=None,
         t_eval=None, rtol=1e-6, atol=1e-9, fixed_nearest=False, *, precision="fp64") -> Trajectory:
    """Integrate a free swimmer's position and orientation (``swimming.py:112-148``): RK45
    (SciPy ``solve_ivp``, as the reference) over instantaneous solves on the device; with
    ``precision="mixed"`` every stage replays one captured system graph (SwimmerPlan)."""
    from scipy.integrate import solve_ivp

    B0 = np.eye(3) if B0 is None else np.asarray(B0, float)
    nearest = None
    if fixed_nearest:
        s0 = shape_at(t_span[0])
        nearest = nearest_neighbors(s0.X, s0.x)
    mixed = _prec(precision) == 1
    plans = {}  # (N, Q) -> SwimmerPlan: one captured system graph reused by every stage

    def rhs(t, z):
        b1, b2 = z[3:6], z[6:9]
        Bm = np.c_[b1, b2, np.cross(b1, b2)]
        shape = shape_at(t)
        if not mixed:
            st = swimming_problem(shape, z[:3], Bm, eps, mu, kernel, nearest, precision=precision)
            U, Om = st.U, st.Omega
        else:
            key = (len(shape.x), len(shape.X))
            if key not in plans:
                plans[key] = SwimmerPlan(Stokeslet3D() if kernel is None else kernel, key[0], key[1], eps, mu,
                                         nearest=nearest)
            x0 = z[:3]
            xw = x0 + np.asarray(shape.x, float) @ Bm.T
            Xw = x0 + np.asarray(shape.X, float) @ Bm.T
            r = np.zeros(3 * key[0] + 6)
            r[:3 * key[0]] = (np.asarray(shape.v, float) @ Bm.T).ravel()
            U, Om, _, _ = plans[key].solve(xw, Xw, x0, r)
        return np.concatenate([U, np.cross(Om, b1), np.cross(Om, b2)])

    z0 = np.concatenate([np.asarray(x0, float), B0[:, 0], B0[:, 1]])
    sol = solve_ivp(rhs, t_span, z0, t_eval=t_eval, rtol=rtol, atol=atol)
    if not sol.success:
        raise RuntimeError(sol.message)
    b1, b2 = sol.y[3:6].T, sol.y[6:9].T
    Bm = np.stack([b1, b2, np.cross(b1, b2)], axis=2)
    return Trajectory(sol.t, sol.y[:3].T, Bm)
