"""CPU oracle for the fluidlets hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline and reference
arms) may import it; ``fluidlets_gb300`` never does, and fails loudly when its
own CUDA library is missing.

It restates the reference package ``fluidlets`` (pure Python + Numba + SciPy):

* per-pair kernel blocks and the O(MN) loops run in ``fl_oracle.c`` (C, OpenMP,
  same operation order as ``kernels/*.py`` and ``core/matvec.py:10-21``,
  ``core/assemble.py:15-58``);
* the driver functions below follow ``core/_common.py:7-23``,
  ``core/matvec.py:24-49``, ``core/assemble.py:27-101``,
  ``core/solve.py:20-84`` and ``swimming.py:33-102`` line by line, including
  the SciPy calls (``scipy.linalg.solve``, ``scipy.sparse.linalg.gmres``,
  ``cKDTree``) that the reference itself makes.

Parity is pinned against the reference's own golden data (the MATLAB
``kernels.mat`` / ``towers.mat`` vectors) and against fixtures produced by
importing the reference itself (``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
KIND = {"stokeslet": 0, "wall": 1, "brinkman": 2}
DENSE_MAX = 6000  # core/solve.py:20

_lib = None


def build(force: bool = False) -> Path:
    """Compile fl_oracle.c into oracle/_build/liboracle.so (gcc, OpenMP)."""
    src = HERE / "fl_oracle.c"
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= src.stat().st_mtime:
        return LIB_PATH
    LIB_PATH.parent.mkdir(exist_ok=True)
    tmp = LIB_PATH.with_suffix(f".so.{os.getpid()}")
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        dp = ctypes.POINTER(ctypes.c_double)
        i64 = ctypes.c_int64
        L.orc_apply.argtypes = [ctypes.c_int, dp, i64, dp, i64, dp, dp, dp, ctypes.c_int, dp, ctypes.c_int]
        L.orc_fill.argtypes = [ctypes.c_int, dp, i64, dp, i64, dp, dp, dp, ctypes.c_int]
        L.orc_fill_nearest.argtypes = [ctypes.c_int, dp, i64, dp, i64, dp, ctypes.POINTER(i64), dp, i64, dp,
                                       ctypes.c_int]
        L.orc_block.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, dp]
        L.orc_brink_f.argtypes = [ctypes.c_double, ctypes.c_double, dp, dp]
        L.orc_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# --------------------------------------------------------------------------
# kernel description: accepts either a kind string ("stokeslet" | "wall" |
# "brinkman", alpha) or any object with .kind / .alpha (the package's kernels)
# --------------------------------------------------------------------------
def kernel_spec(kernel, alpha=0.0):
    if isinstance(kernel, str):
        kind, a = kernel, alpha
    else:
        kind, a = kernel.kind, getattr(kernel, "alpha", 0.0)
    a = complex(a)
    params = np.array([a.real, a.imag], dtype=np.float64)
    return KIND[kind], params, (KIND[kind] == 2 and a.imag != 0.0)


# ---- core/_common.py:7-23 ------------------------------------------------
def points(a, dim=3):
    a = np.atleast_2d(np.asarray(a, dtype=np.float64))
    if a.shape[1] != dim:
        raise ValueError(f"expected points of shape (N, {dim}), got {a.shape}")
    return np.ascontiguousarray(a)


def blob_widths(eps, n):
    eps = np.asarray(eps, dtype=np.float64)
    return np.ascontiguousarray(np.broadcast_to(eps, (n,)))


def field_dtype(mu, *arrays):
    return np.result_type(np.asarray(mu), np.float64, *[np.asarray(a) for a in arrays])


# ---- core/matvec.py:24-49 ------------------------------------------------
def evaluate(kernel, targets, sources, strengths, eps, mu=1.0, alpha=0.0, nthreads=0):
    kind, params, kc = kernel_spec(kernel, alpha)
    targets = points(targets)
    sources = points(sources)
    eps = blob_widths(eps, sources.shape[0])
    dtype = field_dtype(mu, strengths)
    if kc:
        dtype = np.result_type(dtype, np.complex128)
    strengths = np.ascontiguousarray(np.asarray(strengths, dtype=dtype).reshape(sources.shape[0], 3))
    out = np.zeros((targets.shape[0], 3), dtype=dtype)
    fc = np.iscomplexobj(strengths)
    lib().orc_apply(kind, _p(params), targets.shape[0], _p(targets), sources.shape[0], _p(sources), _p(eps),
                    _p(strengths.view(np.float64)), int(fc), _p(out.view(np.float64)), nthreads)
    return out / mu


# ---- core/assemble.py:27-46 ----------------------------------------------
def assemble(kernel, targets, sources, eps, mu=1.0, alpha=0.0, nthreads=0):
    kind, params, kc = kernel_spec(kernel, alpha)
    targets = points(targets)
    sources = points(sources)
    eps = blob_widths(eps, sources.shape[0])
    K = np.empty((3 * targets.shape[0], 3 * sources.shape[0]), dtype=np.complex128 if kc else np.float64)
    lib().orc_fill(kind, _p(params), targets.shape[0], _p(targets), sources.shape[0], _p(sources), _p(eps),
                   _p(K.view(np.float64)), nthreads)
    return K.astype(np.result_type(field_dtype(mu), K.dtype)) / mu


# ---- core/assemble.py:61-101 ---------------------------------------------
def nearest_neighbors(quad_points, force_points):
    from scipy.spatial import cKDTree

    return cKDTree(np.asarray(force_points, float)).query(np.asarray(quad_points, float))[1]


def assemble_nearest(kernel, targets, quad_points, nearest, n_force, eps, mu=1.0, alpha=0.0, nthreads=0):
    kind, params, kc = kernel_spec(kernel, alpha)
    targets = points(targets)
    quad = points(quad_points)
    eps = blob_widths(eps, quad.shape[0])
    nearest = np.ascontiguousarray(nearest, dtype=np.int64)
    K = np.zeros((3 * targets.shape[0], 3 * n_force), dtype=np.complex128 if kc else np.float64)
    lib().orc_fill_nearest(kind, _p(params), targets.shape[0], _p(targets), quad.shape[0], _p(quad),
                           nearest.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _p(eps), n_force,
                           _p(K.view(np.float64)), nthreads)
    return K.astype(np.result_type(field_dtype(mu), K.dtype)) / mu


# ---- core/solve.py:23-84 -------------------------------------------------
@dataclass
class SolveInfo:
    method: str
    iterations: int
    residual: float


def resistance(kernel, points_, velocities, eps, mu=1.0, method="auto", rtol=1e-10, restart=60, maxiter=200,
               alpha=0.0):
    import scipy.linalg
    import scipy.sparse.linalg as spla

    X = points(points_)
    n = X.shape[0]
    eps = blob_widths(eps, n)
    U = np.asarray(velocities).reshape(-1)
    dtype = field_dtype(mu, U)
    if kernel_spec(kernel, alpha)[2]:
        dtype = np.result_type(dtype, np.complex128)
    if method == "auto":
        method = "lu" if U.size <= DENSE_MAX else "gmres"
    if method == "lu":
        K = assemble(kernel, X, X, eps, mu, alpha)
        f = scipy.linalg.solve(K, U.astype(dtype))
        iterations = 1
    elif method == "gmres":
        def matvec(v):
            return evaluate(kernel, X, X, v.reshape(n, -1), eps, mu, alpha).ravel()

        A = spla.LinearOperator((U.size, U.size), matvec=matvec, dtype=dtype)
        count = [0]
        f, flag = spla.gmres(A, U.astype(dtype), rtol=rtol, atol=0.0, restart=restart, maxiter=maxiter,
                             callback=lambda _: count.__setitem__(0, count[0] + 1), callback_type="pr_norm")
        if flag != 0:
            raise RuntimeError(f"GMRES did not converge (flag {flag})")
        iterations = count[0]
    else:
        raise ValueError(f"unknown method {method!r}")
    resid = np.linalg.norm(evaluate(kernel, X, X, f.reshape(n, -1), eps, mu, alpha).ravel() - U) / np.linalg.norm(U)
    return f.reshape(n, -1), SolveInfo(method, iterations, float(resid))


# ---- swimming.py:33-102 --------------------------------------------------
def cross_matrix(v):
    v = np.atleast_2d(v)
    C = np.zeros((len(v), 3, 3))
    C[:, 0, 1], C[:, 0, 2] = -v[:, 2], v[:, 1]
    C[:, 1, 0], C[:, 1, 2] = v[:, 2], -v[:, 0]
    C[:, 2, 0], C[:, 2, 1] = -v[:, 1], v[:, 0]
    return C


def swimming_problem(x_body, v_body, X_body, x0, B, eps, mu=1.0, kernel="stokeslet", nearest=None):
    """Returns (U, Omega, forces, x, X, nearest) as the reference's SwimState."""
    x0 = np.asarray(x0, float)
    B = np.asarray(B, float)
    x = x0 + np.asarray(x_body, float) @ B.T
    X = x0 + np.asarray(X_body, float) @ B.T
    v = np.asarray(v_body, float) @ B.T
    if nearest is None:
        nearest = nearest_neighbors(X, x)
    N = len(x)
    A = np.zeros((3 * N + 6, 3 * N + 6))
    A[:3 * N, :3 * N] = assemble_nearest(kernel, x, X, nearest, N, eps, mu)
    A[:3 * N, 3 * N:3 * N + 3] = -np.tile(np.eye(3), (N, 1))
    A[:3 * N, 3 * N + 3:] = cross_matrix(x - x0).reshape(3 * N, 3)
    count = np.bincount(nearest, minlength=N).astype(float)
    Xsum = np.zeros((N, 3))
    np.add.at(Xsum, nearest, X)
    A[3 * N:3 * N + 3, :3 * N] = np.kron(count, np.eye(3))
    A[3 * N + 3:, :3 * N] = np.hstack(list(cross_matrix(Xsum)))
    rhs = np.concatenate([v.ravel(), np.zeros(6)])
    sol = np.linalg.solve(A, rhs)
    return sol[3 * N:3 * N + 3], sol[3 * N + 3:], sol[:3 * N].reshape(N, 3), x, X, nearest


# ---- Brinkmanlet auxiliary functions (kernels/brinkmanlet3d.py:52-71) -----
def brink_f(z):
    z = complex(z)
    a = np.zeros(2)
    b = np.zeros(2)
    lib().orc_brink_f(z.real, z.imag, _p(a), _p(b))
    return complex(a[0], a[1]), complex(b[0], b[1])


def block(kernel, x, x0, eps, alpha=0.0):
    kind, params, _ = kernel_spec(kernel, alpha)
    x = np.ascontiguousarray(x, dtype=np.float64)
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    G = np.zeros(18)
    lib().orc_block(kind, _p(params), _p(x), _p(x0), float(eps), _p(G))
    return G.view(np.complex128).reshape(3, 3)


# ---- geometry (geometry/spheres.py), the checker of the device generators --
def fibonacci_sphere(n, radius=1.0, center=(0.0, 0.0, 0.0)):
    """geometry/spheres.py:7-13: golden-angle spiral, NumPy's operation order."""
    k = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * k / n)
    theta = np.pi * (1 + np.sqrt(5)) * k
    unit = np.c_[np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)]
    return radius * unit + np.asarray(center, float)


def cube_sphere(n, radius=1.0, center=(0.0, 0.0, 0.0)):
    """geometry/spheres.py:33-52: n x n cell-centred points on each cube face (faces ordered
    x = -1, x = +1, y = -1, y = +1, z = -1, z = +1; the two free coordinates in ascending axis
    order, the first one slowest), normalized onto the sphere."""
    s = np.linspace(-1.0 + 1.0 / n, 1.0 - 1.0 / n, n)
    u = np.repeat(s, n)          # slow free coordinate
    v = np.tile(s, n)            # fast free coordinate
    blocks = []
    for axis in range(3):
        for side in (-1.0, 1.0):
            P = np.empty((n * n, 3))
            free = [a for a in range(3) if a != axis]
            P[:, axis] = side
            P[:, free[0]] = u
            P[:, free[1]] = v
            blocks.append(P)
    P = np.concatenate(blocks)
    return radius * (P / np.linalg.norm(P, axis=1)[:, None]) + np.asarray(center, float)


def mean_nn_spacing(points):
    """Mean distance to the nearest other point (SciPy k-d tree)."""
    from scipy.spatial import cKDTree

    d, _ = cKDTree(points).query(points, k=2)
    return float(d[:, 1].mean())


def max_threads():
    return lib().orc_max_threads()
