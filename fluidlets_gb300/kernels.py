"""Kernel objects: the plugin interface of the reference, kept by name.

The reference's kernels (``kernels/base.py:14-32``) carry a Numba ``block``
function that the core loops call per pair.  Here a kernel is a *description*
-- a kind and its parameters -- that the CUDA library dispatches on; the
per-pair arithmetic lives in ``csrc/pair_math.cuh``.  ``velocity()`` keeps the
reference's pure-NumPy single-pair formula (for tests and for users who call
it), and ``block()`` fills one 3x3 block on the host.
"""
from __future__ import annotations

import numpy as np


class Kernel:
    """Base class: ``dim``, ``out_shape``, ``kind`` (``kernels/base.py:14-24``)."""

    dim: int
    kind: str
    alpha = 0.0

    @property
    def out_shape(self) -> tuple[int, int]:
        return (self.dim, self.dim)

    @property
    def is_complex(self) -> bool:
        return False

    def velocity(self, x, x0, f, eps, mu=1.0):
        raise NotImplementedError

    def block(self, x, x0, eps, out=None):
        """The (3, 3) matrix G(x, x0) for mu = 1 (host-side, one pair)."""
        G = np.empty((3, 3), dtype=np.complex128 if self.is_complex else np.float64)
        for b in range(3):
            G[:, b] = self.velocity(x, x0, np.eye(3)[b], eps)
        if out is not None:
            out[...] = G
            return out
        return G


class VectorKernel(Kernel):
    """A force (dim) at a source gives a velocity (dim) at a target (``kernels/base.py:27-32``)."""


class Stokeslet3D(VectorKernel):
    """Regularized Stokeslet in free space (``kernels/stokeslet3d.py:53-64``)."""

    dim = 3
    kind = "stokeslet"

    def velocity(self, x, x0, f, eps, mu=1.0):
        d = np.asarray(x, float) - np.asarray(x0, float)
        f = np.asarray(f)
        r2 = d @ d
        q = (r2 + eps**2) ** 1.5
        return ((r2 + 2 * eps**2) * f + (f @ d) * d) / (8 * np.pi * mu * q)

    def __repr__(self) -> str:
        return "Stokeslet3D()"


class WallStokeslet3D(VectorKernel):
    """Regularized Stokeslet above a no-slip wall at z = 0 (``kernels/images.py:92-104``).

    Free-space Stokeslet plus the Ainley et al. (2008) image system.  Sources
    need z > 0.
    """

    dim = 3
    kind = "wall"

    def velocity(self, x, x0, f, eps, mu=1.0):
        free = Stokeslet3D().velocity(x, x0, f, eps, mu)
        return free + _image_velocity(x, x0, f, eps, mu)

    def __repr__(self) -> str:
        return "WallStokeslet3D()"


def _image_velocity(x, x0, f, eps, mu=1.0):
    """Image part at one target from one source, as matrix algebra.

    Same physics as ``kernels/images.py:107-139`` (Stokeslet, dipole, doublet,
    rotlet at the mirror point), written independently of the CUDA form.
    """
    x = np.asarray(x, float)
    x0 = np.asarray(x0, float)
    f = np.asarray(f)
    h0 = x0[2]
    d = x - np.array([x0[0], x0[1], -h0])
    e2 = eps**2
    Q = d @ d + e2
    I3 = np.eye(3)
    D = np.outer(d, d)
    Z = np.diag([-1.0, -1.0, 1.0])
    stokeslet = -((0.5 / Q**0.5 + 0.5 * e2 / Q**1.5) * I3 + 0.5 / Q**1.5 * D)
    dipole = (-h0**2 * (1 / Q**1.5 - 3 * e2 / Q**2.5) * I3 + 3 * h0**2 / Q**2.5 * D) @ Z
    Hdb1 = -h0 * (3 * e2 / Q**2.5 + 1 / Q**1.5)
    Hdb2 = h0 / Q**1.5
    Hdb3 = -3 * h0 / Q**2.5
    doublet = np.zeros((3, 3))
    doublet[:2, :2] = -d[2] * (Hdb2 * I3[:2, :2] + D[:2, :2] * Hdb3)
    doublet[:2, 2] = d[:2] * (Hdb2 + d[2] ** 2 * Hdb3)
    doublet[2, :2] = -d[:2] * (Hdb1 + d[2] ** 2 * Hdb3)
    doublet[2, 2] = d[2] * (Hdb1 + 2 * Hdb2 + d[2] ** 2 * Hdb3)
    Hr1 = 3 * h0 * e2 / Q**2.5
    rotlet = Hr1 * (d[2] * np.diag([1.0, 1.0, 0.0]) - np.outer([0, 0, 1.0], [d[0], d[1], 0.0]))
    return (stokeslet + dipole + doublet + rotlet) @ f / (4 * np.pi * mu)


class Brinkmanlet3D(VectorKernel):
    """Regularized Brinkmanlet with inverse screening length alpha (``kernels/brinkmanlet3d.py:107-141``).

    ``Brinkmanlet3D(0.0)`` is the regularized Stokeslet.  A complex alpha with
    non-negative real part (oscillatory flow, alpha = (1 + i) sqrt(omega / 2))
    is accepted here; the reference raises for it.
    """

    dim = 3
    kind = "brinkman"

    def __init__(self, alpha):
        a = complex(alpha)
        if not np.isfinite(a.real) or not np.isfinite(a.imag):
            raise ValueError("alpha must be finite")
        if a.imag == 0.0:
            if a.real < 0:
                raise ValueError("alpha must be real and non-negative")
            self.alpha = float(a.real)
        else:
            if a.real < 0:
                raise ValueError("complex alpha must have a non-negative real part")
            self.alpha = a

    @property
    def is_complex(self) -> bool:
        return isinstance(self.alpha, complex)

    def __repr__(self) -> str:
        return f"Brinkmanlet3D(alpha={self.alpha})"

    def velocity(self, x, x0, f, eps, mu=1.0):
        d = np.asarray(x, float) - np.asarray(x0, float)
        f = np.asarray(f)
        R = np.sqrt(d @ d + eps**2)
        a = self.alpha
        if a == 0:
            h1, h2 = 1 / (8 * np.pi * R), 1 / (8 * np.pi * R**3)
        else:
            z = a * R
            E = np.exp(-z)
            h1 = (E * (1 + 1 / z + 1 / z**2) - 1 / z**2) / (4 * np.pi * R)
            h2 = (3 / z**2 - E * (1 + 3 / z + 3 / z**2)) / (4 * np.pi * R**3)
        H1 = h1 + eps**2 * h2
        return (H1 * f + h2 * (f @ d) * d) / mu


def kernel_params(kernel) -> tuple[int, float, float]:
    """(kind code, alpha_re, alpha_im) for the C ABI."""
    from ._lib import KIND

    kind = getattr(kernel, "kind", None)
    if kind not in KIND:
        raise TypeError(f"unsupported kernel {kernel!r}")
    a = complex(getattr(kernel, "alpha", 0.0))
    return KIND[kind], a.real, a.imag
