"""Point sets used to build the benchmark and test workloads.

The sphere discretizations of the reference (``geometry/spheres.py``: the
golden-angle spiral and the six-patch cube sphere) and the mean
nearest-neighbour spacing that sets blob widths are generated on the GPU by
``csrc/geometry.cu``; the ``*_device`` functions return CUDA tensors, the plain
names NumPy arrays.  ``spheroid`` and the ``*_workload`` / ``*_shape``
functions build the synthetic, seeded inputs of the benchmark configurations
from them.
"""
from __future__ import annotations

import numpy as np


def fibonacci_sphere(n: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """n nearly uniform points on a sphere (golden-angle spiral), shape (n, 3), generated on the GPU."""
    return fibonacci_sphere_device(n, radius, center).cpu().numpy()


def cube_sphere(n: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Six n x n cell-centred patches of the cube projected onto the sphere: 6 n^2 points,
    generated on the GPU."""
    return cube_sphere_device(n, radius, center).cpu().numpy()


def mean_nn_spacing(points) -> float:
    """Mean nearest-neighbour distance (exhaustive search on the GPU)."""
    return mean_nn_spacing_device(points)


def spheroid(n: int, aspect: float, rotation: np.ndarray | None = None, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Prolate spheroid with semi-axes (aspect, 1, 1) from a Fibonacci lattice, rotated then shifted."""
    p = fibonacci_sphere(n) * np.array([aspect, 1.0, 1.0])
    if rotation is not None:
        p = p @ np.asarray(rotation).T
    return p + np.asarray(center, float)


def wall_sum_workload(n_src: int = 262144, n_tgt: int = 262144, n_wall: int = 16384, eps: float = 0.01,
                      seed: int = 0):
    """Wall-Stokeslet sum workload: sources and targets uniform in [-1,1]^2 x [0.02,2]
    above the wall z = 0, i.i.d. N(0,1) forces, plus n_wall targets on z = 0."""
    rng = np.random.default_rng(seed)
    lo, hi = [-1.0, -1.0, 0.02], [1.0, 1.0, 2.0]
    src = rng.uniform(lo, hi, (n_src, 3))
    tgt = rng.uniform(lo, hi, (n_tgt, 3))
    wall = np.c_[rng.uniform(-1, 1, (n_wall, 2)), np.zeros(n_wall)]
    f = rng.normal(size=(n_src, 3))
    return np.r_[tgt, wall], src, f, eps


def ellipsoid_points(n: int, axes=(0.6, 0.4, 0.4)) -> np.ndarray:
    """n points on an ellipsoid surface (a stretched Fibonacci lattice)."""
    return fibonacci_sphere(n) * np.asarray(axes, float)


def biflagellate_shape(t: float, n_body: int = 96, fine: int = 4, segments: int = 64, amplitude: float = 0.2,
                       wavelength: float = 1.0, length: float = 1.0, frequency: float = 1.0):
    """A model biflagellate swimmer in its body frame at time t.

    Body: ellipsoid with semi-axes 0.6 : 0.4 : 0.4 (3:2:2), n_body force points and fine * n_body
    quadrature points, at rest in the body frame.  Two planar flagella of `segments` segments
    attached at the front (x = 0.6, z = +-0.1), pointing along +x and beating in the x-z plane as
    travelling sine waves z = +-(0.1 + A sin(k s - w t) s/L) of amplitude A = 0.2 and wavelength 1;
    force points at the segment ends, `fine` quadrature points per segment.  Returns a SwimmerShape.
    With amplitude >= 0.1 the two mirror-image flagella cross during the beat (the system is
    near-singular at those instants): fine for instantaneous solves, but integrate a trajectory
    with amplitude < 0.1.
    """
    from .swimming import SwimmerShape

    k = 2 * np.pi / wavelength
    w = 2 * np.pi * frequency

    def flagellum(sign, s):
        env = s / length
        x = 0.6 + s
        z = sign * (0.1 + amplitude * env * np.sin(k * s - w * t))
        vz = sign * (-amplitude * env * w * np.cos(k * s - w * t))
        pos = np.c_[x, np.zeros_like(s), z]
        vel = np.c_[np.zeros_like(s), np.zeros_like(s), vz]
        return pos, vel

    s_c = np.linspace(0, length, segments + 1)[1:]
    s_f = np.linspace(0, length, fine * segments + 1)[1:]
    body_c = ellipsoid_points(n_body)
    body_f = ellipsoid_points(fine * n_body)
    xs, vs, Xs = [body_c], [np.zeros_like(body_c)], [body_f]
    for sign in (1.0, -1.0):
        p, v = flagellum(sign, s_c)
        pf, _ = flagellum(sign, s_f)
        xs.append(p)
        vs.append(v)
        Xs.append(pf)
    return SwimmerShape(x=np.vstack(xs), v=np.vstack(vs), X=np.vstack(Xs))


# ---- the same on the device -------------------------------------------------------------
def _sphere_device(fn, count, n, radius, center):
    import ctypes

    import torch

    from . import _device as dv
    from ._lib import check, load

    out = torch.empty((count, 3), dtype=torch.float64, device=dv.require_cuda())
    c = (ctypes.c_double * 3)(*np.asarray(center, float).reshape(3))
    check(getattr(load(), fn)(n, float(radius), c, dv.ptr(out), dv.stream()), fn)
    return out


def fibonacci_sphere_device(n: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """fibonacci_sphere generated on the GPU (a CUDA tensor)."""
    return _sphere_device("flg_fibonacci_sphere", n, n, radius, center)


def cube_sphere_device(n: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """cube_sphere generated on the GPU (a CUDA tensor)."""
    return _sphere_device("flg_cube_sphere", 6 * n * n, n, radius, center)


def mean_nn_spacing_device(points) -> float:
    """mean_nn_spacing on the GPU (exhaustive nearest-neighbour search)."""
    import torch

    from . import _device as dv
    from ._lib import check, load

    P = dv.to_dev(points, torch.float64).reshape(-1, 3)
    L = load()
    n = P.shape[0]
    nb = L.flg_mean_nn_spacing_workspace(n)
    ws = dv.workspace(nb)
    m = torch.empty(1, dtype=torch.float64, device=P.device)
    check(L.flg_mean_nn_spacing(dv.ptr(P), n, dv.ptr(m), dv.ptr(ws), nb, dv.stream()), "mean_nn_spacing")
    return float(m.item())
