"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run once, in a container where the reference source tree is available:

    python tests/golden/make_golden.py <path of the reference source tree>

Two kinds of fixture are written:

* ``legacy_*.npz`` -- the reference's own golden data, converted from MATLAB
  ``.mat`` files: ``tests/legacy/data/kernels.mat`` (40 sources with per-source
  blob width, 60 targets, V_stokeslet, V_image; 441 wall points with
  V_wall_total) and ``tests/legacy/data/towers.mat`` (441-point glycocalyx
  towers: positions, prescribed velocities, legacy GMRES forces, residual).
  These pin ``tests/legacy/test_phase1_port.py:33-74``.  ``legacy_grid.npz`` is
  ``legacy/sdc_cuda3/velocity_t_xyz_final.raw``, the 32^3 velocity grid the 2010
  CUDA code wrote for the towers (float32, x fastest; background shear 0.1 z
  included), pinning ``tests/legacy/test_phase1_port.py:77-87``.
* ``reference_cases.npz`` -- outputs of the reference package ``fluidlets``
  (``src/fluidlets``) computed here.  Numba is not installed, so the reference
  is imported through a stand-in ``numba`` module whose ``njit`` returns the
  function unchanged and whose ``prange`` is ``range``: the reference's code
  then runs as plain Python with its own arithmetic.

Nothing at test time reads the reference tree; only the .npz files travel.
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent


def install_numba_standin():
    m = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    m.njit = njit
    m.jit = njit
    m.prange = range
    sys.modules["numba"] = m


def convert_legacy(ref: Path):
    import scipy.io as sio

    d = sio.loadmat(ref / "tests/legacy/data/kernels.mat", squeeze_me=True)
    np.savez_compressed(OUT / "legacy_kernels.npz",
                        **{k: np.asarray(d[k], dtype=np.float64) for k in
                           ["targets", "sources", "strengths", "deltas", "V_stokeslet", "V_image", "wall",
                            "V_wall_total", "V_wall_free"]})
    t = sio.loadmat(ref / "tests/legacy/data/towers.mat", squeeze_me=True)
    n = t["x0"].size // 3
    np.savez_compressed(OUT / "legacy_towers.npz",
                        x0=t["x0"].reshape(3, n).T.copy(), Vel=t["Vel"].reshape(3, n).T.copy(),
                        Forces=t["Forces"].reshape(3, n).T.copy(), resid=np.float64(t["resid"]))
    s = sio.loadmat(ref / "tests/legacy/data/sphere_drag.mat", squeeze_me=True)
    np.savez_compressed(OUT / "legacy_sphere_drag.npz",
                        **{k: np.asarray(s[k], dtype=np.float64) for k in
                           ["F_free", "F_free_N", "F_par", "F_perp", "F_stokes", "H_list", "N_list", "h_list"]})


def convert_legacy_grid(ref: Path):
    raw = np.fromfile(ref / "legacy/sdc_cuda3/velocity_t_xyz_final.raw", "<f4").reshape(-1, 3)
    # grid axes, blob width and shear rate of tests/legacy/test_phase1_port.py:16-18, 77-87
    np.savez_compressed(OUT / "legacy_grid.npz", velocity=raw, x_axis=np.array([-1.0, 8.0, 32]),
                        y_axis=np.array([-5.0, 25.0, 32]), z_axis=np.array([0.0, 20.0, 32]),
                        delta=np.float64(0.5), shear=np.float64(0.1))


def reference_cases(ref: Path):
    install_numba_standin()
    sys.path.insert(0, str(ref / "src"))
    import fluidlets as fl
    from fluidlets.core import assemble_nearest, nearest_neighbors
    from fluidlets.geometry import cube_sphere, fibonacci_sphere
    from fluidlets.kernels.brinkmanlet3d import f1, f2
    from fluidlets.swimming import SwimmerShape, swimming_problem

    rng = np.random.default_rng(20261203)
    out = {}

    def above_wall(n):
        return np.c_[rng.uniform(-1, 1, (n, 2)), rng.uniform(0.05, 1.5, n)]

    # evaluate: each kernel, per-source eps, M=33 targets, N=47 sources (ragged sizes)
    X, X0, F = above_wall(33), above_wall(47), rng.normal(size=(47, 3))
    eps = rng.uniform(0.05, 0.3, 47)
    out["ev_targets"], out["ev_sources"], out["ev_forces"], out["ev_eps"] = X, X0, F, eps
    out["ev_stokeslet"] = fl.evaluate(fl.Stokeslet3D(), X, X0, F, eps)
    out["ev_wall"] = fl.evaluate(fl.WallStokeslet3D(), X, X0, F, eps)
    for a in (0.0, 0.5, 3.0, 20.0):
        out[f"ev_brinkman_{a:g}"] = fl.evaluate(fl.Brinkmanlet3D(a), X, X0, F, eps)
    # complex viscosity and complex strengths (core/_common.py:21-23)
    mu = 2.0 - 0.5j
    Fc = F + 1j * rng.normal(size=F.shape)
    out["ev_forces_c"] = Fc
    out["ev_stokeslet_mu"] = fl.evaluate(fl.Stokeslet3D(), X, X0, F, eps, mu=mu)
    out["ev_wall_fc"] = fl.evaluate(fl.WallStokeslet3D(), X, X0, Fc, eps, mu=0.7)
    out["ev_brinkman_fc"] = fl.evaluate(fl.Brinkmanlet3D(3.0), X, X0, Fc, eps, mu=mu)
    # wall targets on z = 0
    W = np.c_[rng.uniform(-2, 2, (29, 2)), np.zeros(29)]
    out["ev_wall_targets"] = W
    out["ev_wall_on_wall"] = fl.evaluate(fl.WallStokeslet3D(), W, X0, F, eps)

    # assemble (scalar eps and per-source eps), incl. complex mu
    Y = above_wall(19)
    out["as_points"] = Y
    out["as_stokeslet"] = fl.assemble(fl.Stokeslet3D(), Y, Y, 0.2)
    out["as_wall"] = fl.assemble(fl.WallStokeslet3D(), Y, Y, eps[:19])
    out["as_brinkman"] = fl.assemble(fl.Brinkmanlet3D(3.0), Y, Y, 0.2)
    out["as_wall_mu"] = fl.assemble(fl.WallStokeslet3D(), Y, Y, 0.2, mu=mu)
    out["as_rect_targets"] = X
    out["as_rect"] = fl.assemble(fl.WallStokeslet3D(), X, Y, 0.15)

    # assemble_nearest (core/assemble.py:68-101)
    xc, Xq = cube_sphere(3), cube_sphere(7)
    nn = nearest_neighbors(Xq, xc)
    out["an_coarse"], out["an_quad"], out["an_nearest"] = xc, Xq, np.asarray(nn, np.int64)
    out["an_stokeslet"] = assemble_nearest(fl.Stokeslet3D(), xc, Xq, nn, len(xc), 0.05)
    out["an_wall"] = assemble_nearest(fl.WallStokeslet3D(), xc + [0, 0, 1.5], Xq + [0, 0, 1.5], nn, len(xc), 0.05)

    # resistance: LU and GMRES on a Fibonacci sphere (tests/test_kernels.py:61-73 setting)
    n = 200
    S = fibonacci_sphere(n)
    e = 0.5 * np.sqrt(4 * np.pi / n)
    U = np.tile([1.0, 0, 0], (n, 1))
    out["rs_points"], out["rs_eps"], out["rs_U"] = S, np.float64(e), U
    f, info = fl.resistance(fl.Stokeslet3D(), S, U, e, method="lu")
    out["rs_lu_forces"], out["rs_lu_resid"] = f, np.float64(info.residual)
    f, info = fl.resistance(fl.Stokeslet3D(), S, U, e, method="gmres")
    out["rs_gmres_forces"], out["rs_gmres_iters"] = f, np.int64(info.iterations)
    out["rs_gmres_resid"] = np.float64(info.residual)
    Sw = S + [0, 0, 1.5]
    Uw = np.tile([0, 0, 1.0], (n, 1))
    out["rs_wall_points"] = Sw
    f, info = fl.resistance(fl.WallStokeslet3D(), Sw, Uw, e, method="lu")
    out["rs_wall_lu_forces"] = f
    f, info = fl.resistance(fl.Brinkmanlet3D(1.0), S, U, e, method="gmres", restart=20)
    out["rs_brink_gmres_forces"], out["rs_brink_gmres_iters"] = f, np.int64(info.iterations)

    # swimming_problem (swimming.py:66-102)
    xs = cube_sphere(3)
    Xs = cube_sphere(6)
    V = np.array([0.2, -0.1, 0.7])
    vs = -np.tile(V, (len(xs), 1)) + 0.1 * rng.normal(size=xs.shape)
    B = np.linalg.qr(rng.normal(size=(3, 3)))[0]
    B *= np.sign(np.linalg.det(B))
    x0 = np.array([0.3, -0.2, 1.1])
    st = swimming_problem(SwimmerShape(x=xs, v=vs, X=Xs), x0, B, 0.05)
    out["sw_x"], out["sw_v"], out["sw_X"], out["sw_x0"], out["sw_B"] = xs, vs, Xs, x0, B
    out["sw_U"], out["sw_Omega"], out["sw_forces"], out["sw_nearest"] = st.U, st.Omega, st.forces, st.nearest

    # Brinkmanlet auxiliary functions f1, f2 (series and closed form)
    zs = np.array([1e-8, 0.01, 0.3, 0.499, 0.5, 0.501, 2.0, 30.0])
    out["bf_z"] = zs
    out["bf_f1"] = np.array([f1(z) for z in zs])
    out["bf_f2"] = np.array([f2(z) for z in zs])

    np.savez_compressed(OUT / "reference_cases.npz", **out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference source tree>")
    ref = Path(sys.argv[1])
    convert_legacy(ref)
    convert_legacy_grid(ref)
    reference_cases(ref)
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)
