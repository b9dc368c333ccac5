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
from ._lib import F64, check, load
from .core import _assemble_nearest_dev, _gmres_ir_dense_dev, _lowp_factor_dev, _lu_solve_dev, _prec, nearest_neighbors
from .kernels import Stokeslet3D


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


@dataclass
class Trajectory:
    t: np.ndarray
    x0: np.ndarray
    B: np.ndarray


def swim(shape_at: Callable[[float], SwimmerShape], t_span, eps, mu=1.0, x0=(0, 0, 0), B0=None, kernel=None,
         t_eval=None, rtol=1e-6, atol=1e-9, fixed_nearest=False, *, precision="fp64") -> Trajectory:
    """Integrate a free swimmer's position and orientation (``swimming.py:112-148``): RK45
    (SciPy ``solve_ivp``) over instantaneous solves on the device."""
    from scipy.integrate import solve_ivp

    B0 = np.eye(3) if B0 is None else np.asarray(B0, float)
    nearest = None
    if fixed_nearest:
        s0 = shape_at(t_span[0])
        nearest = nearest_neighbors(s0.X, s0.x)

    def rhs(t, z):
        b1, b2 = z[3:6], z[6:9]
        Bm = np.c_[b1, b2, np.cross(b1, b2)]
        st = swimming_problem(shape_at(t), z[:3], Bm, eps, mu, kernel, nearest, precision=precision)
        return np.concatenate([st.U, np.cross(st.Omega, b1), np.cross(st.Omega, b2)])

    z0 = np.concatenate([np.asarray(x0, float), B0[:, 0], B0[:, 1]])
    sol = solve_ivp(rhs, t_span, z0, t_eval=t_eval, rtol=rtol, atol=atol)
    if not sol.success:
        raise RuntimeError(sol.message)
    b1, b2 = sol.y[3:6].T, sol.y[6:9].T
    Bm = np.stack([b1, b2, np.cross(b1, b2)], axis=2)
    return Trajectory(sol.t, sol.y[:3].T, Bm)
