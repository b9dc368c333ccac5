"""``stokeslet3d_velocity`` (the reference's ``stokeslet3d.py:15-32``)."""
from __future__ import annotations

from .core import evaluate
from .kernels import Stokeslet3D


def stokeslet3d_velocity(targets, sources, forces, eps, mu=1.0):
    """Velocity at targets induced by 3D regularized Stokeslets: ``evaluate(Stokeslet3D(), ...)``."""
    return evaluate(Stokeslet3D(), targets, sources, forces, eps, mu)
