"""Rigid bodies: the mobility problem and the grand resistance matrix.

The reference states both only in its tutorial (``tutorials/03_mobility_resistance_swimming.ipynb``,
the sedimenting sphere): with the surface forces f_k, the rigid velocity U and angular velocity
Omega about a centre c as unknowns,

    (1/mu) sum_j K_kj f_j - U + (x_k - c) x Omega = 0     (every point moves rigidly)
    sum_k f_k = F,    sum_k x_k x f_k = T + c x F          (given force, and torque about c)

which is the free-swimming system of ``swimming.py:66-102`` with the quadrature points equal to
the force points, no slip, and the force and torque on the right-hand side; it is assembled by the
same device kernels (``flg_assemble_nearest`` with the identity map, ``flg_swimmer_constraints``).
The grand resistance matrix R (forces and torques for unit translations and rotations) is six
resistance solves with one factorization.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _device as dv
from .core import (_assemble_dev, _blob_widths, _gmres_ir_dense_dev, _lowp_factor_dev, _lu_solve_dev, _points, _prec,
                   _uniform_eps)
from .kernels import Stokeslet3D
from .swimming import _system_dev


def _centre(X: np.ndarray, center) -> np.ndarray:
    return X.mean(axis=0) if center is None else np.asarray(center, float).reshape(3)


def rigid_body_mobility(kernel, points, eps, force, torque=(0.0, 0.0, 0.0), mu=1.0, center=None, *,
                        precision="fp64", lu="tf32", rtol=1e-10):
    """Velocity of a rigid body under a given force and torque (about ``center``, default the
    centroid of the points): returns (U, Omega, forces (N, 3))."""
    kernel = Stokeslet3D() if kernel is None else kernel
    if complex(mu).imag != 0.0:
        raise ValueError("the rigid-body problem needs a real viscosity")
    X = np.asarray(dv.to_host(_points(points, 3)), float)
    N = len(X)
    c = _centre(X, center)
    F = np.asarray(force, float).reshape(3)
    T = np.asarray(torque, float).reshape(3) + np.cross(c, F)  # torque about the origin
    A = _system_dev(kernel, X, X, np.arange(N), c, eps, mu)
    rhs = torch.zeros(3 * N + 6, dtype=torch.float64, device=A.device)
    rhs[3 * N:3 * N + 3] = torch.from_numpy(F).to(A.device)
    rhs[3 * N + 3:] = torch.from_numpy(T).to(A.device)
    if _prec(precision) == 1:
        K32, ld32, dinv, A32 = _lowp_factor_dev(A, lu)
        sol, *_ = _gmres_ir_dense_dev(A, K32, ld32, dinv, rhs, rtol * 1e-2, 60, 200, required=rtol, A32=A32)
    else:
        sol = _lu_solve_dev(A, rhs)
    sol = dv.to_host(sol)
    return sol[3 * N:3 * N + 3], sol[3 * N + 3:], sol[:3 * N].reshape(N, 3)


def resistance_matrix(kernel, points, eps, mu=1.0, center=None, *, precision="fp64", lu="tf32", rtol=1e-10):
    """Grand resistance matrix R (6, 6) of a rigid body: column j holds the total force (rows 0-2)
    and torque about ``center`` (rows 3-5) exerted on the fluid when the body translates with
    unit velocity e_j (j < 3) or rotates with unit angular velocity e_{j-3} about the centre."""
    kernel = Stokeslet3D() if kernel is None else kernel
    Xd = _points(points, 3)
    X = np.asarray(dv.to_host(Xd), float)
    N = len(X)
    c = _centre(X, center)
    r = X - c
    e = _blob_widths(eps, N)
    U = np.zeros((N, 3, 6))
    for j in range(3):
        U[:, j, j] = 1.0
        U[:, :, 3 + j] = np.cross(np.eye(3)[j], r)
    Ud = torch.from_numpy(U.reshape(3 * N, 6)).to(Xd.device)
    K = _assemble_dev(kernel, Xd, Xd, e, mu, sym_eps=_uniform_eps(eps), reciprocal=_prec(precision) == 1)
    if K.is_complex():
        raise ValueError("the resistance matrix needs a real kernel and viscosity")
    if _prec(precision) == 1:
        K32, ld32, dinv, A32 = _lowp_factor_dev(K, lu)
        cols = [_gmres_ir_dense_dev(K, K32, ld32, dinv, Ud[:, j].contiguous(), rtol * 1e-2, 60, 200,
                                    required=rtol, A32=A32)[0] for j in range(6)]
        f = torch.stack(cols, 1)
    else:
        f = _lu_solve_dev(K, Ud).reshape(3 * N, 6)
    f = dv.to_host(f).reshape(N, 3, 6)
    R = np.zeros((6, 6))
    R[:3] = f.sum(axis=0)
    R[3:] = np.cross(r[:, :, None], f, axis=1).sum(axis=0)
    return R
