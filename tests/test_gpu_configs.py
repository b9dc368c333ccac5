"""Parity at the benchmark configurations' own sizes.

* Sphere resistance, N = 1,536 Fibonacci points, eps = 0.25 x mean nearest-neighbour spacing,
  free Stokeslet, U = (1, 0, 0) (4,608 unknowns): the FP64 GPU LU against the oracle
  (``scipy.linalg.solve`` on the oracle's matrix, the reference's own call, ``core/solve.py:64-67``),
  and the TF32 / BF16 tensor-core LU + FP64 refinement against both, to 1e-10.
* Wall resistance, N = 8,192 (24,576 unknowns, the 4.8 GB FP64 matrix) at h/a = 1.05 and 3.0,
  motion parallel and normal to the wall: mixed against the FP64 GPU LU to 1e-10, and the FP64
  forces checked against the oracle's own kernel sum (they reproduce U to 1e-12).
* Brinkmanlet resistance by GMRES, N = 16,384 (49,152 unknowns), alpha = 10 and the complex
  alpha = (1 + i) sqrt(omega / 2), omega in {1, 10}: mixed (FP32 far field inside FP64 iterative
  refinement, rtol 1e-10) against the FP64-matvec GMRES converged to 1e-13, to 1e-10.
* A wall resistance problem with a point on the wall z = 0 is singular: LinAlgError from the FP64
  LU and the mixed LU (the reference's LAPACK call only warns there, see the test).

The relative force error is ||F - F_ref||_2 / ||F_ref||_2, the metric of the mixed-precision
target (relative error <= 1e-10 against the FP64 result).
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
scipy_linalg = pytest.importorskip("scipy.linalg")
fl = pytest.importorskip("fluidlets_gb300")
from fluidlets_gb300.core import _assemble_dev, _lu_solve_dev  # noqa: E402

W = fl.WallStokeslet3D()
S3 = fl.Stokeslet3D()
TOL = 1e-10


def rel_l2(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_sphere_resistance_1536_fp64_and_mixed_vs_oracle(record_property):
    N = 1536
    X = O.fibonacci_sphere(N)
    eps = 0.25 * O.mean_nn_spacing(X)
    assert abs(eps - 0.021832) < 5e-7
    U = np.tile([1.0, 0.0, 0.0], (N, 1))
    ref = scipy_linalg.solve(O.assemble("stokeslet", X, X, eps), U.ravel()).reshape(N, 3)
    drag_ref = ref[:, 0].sum() / (6 * np.pi)
    F64, info = fl.resistance(S3, X, U, eps, method="lu")
    assert info.method == "lu" and info.residual < 1e-13
    assert rel_l2(F64, ref) < TOL
    drag = F64[:, 0].sum() / (6 * np.pi)
    assert abs(drag - drag_ref) < 1e-10 * abs(drag_ref)
    assert abs(drag - 0.98392) < 1e-5
    record_property("drag_over_6pi_a", float(drag))
    for lu in ("tf32", "bf16"):
        Fm, im = fl.resistance(S3, X, U, eps, method="lu", precision="mixed", lu=lu)
        assert im.precision == "mixed" and im.residual < TOL
        assert rel_l2(Fm, F64) < TOL, lu
        assert rel_l2(Fm, ref) < TOL, lu
        record_property(f"{lu}_err_vs_oracle", rel_l2(Fm, ref))
        record_property(f"{lu}_ir_steps", im.ir_steps)


@pytest.fixture(scope="module")
def wall_sphere_8192():
    S = O.fibonacci_sphere(8192)
    eps = 0.25 * O.mean_nn_spacing(S)
    assert abs(eps - 0.0094103) < 5e-7
    return S, eps


@pytest.mark.parametrize("h", [1.05, 3.0])
def test_wall_resistance_8192_mixed_vs_fp64(wall_sphere_8192, h, record_property):
    S, eps = wall_sphere_8192
    n = len(S)
    dev = torch.device("cuda")
    X = torch.tensor(S + [0.0, 0.0, h], device=dev)
    e = torch.full((n,), eps, dtype=torch.float64, device=dev)
    motions = {"parallel": [1.0, 0.0, 0.0], "normal": [0.0, 0.0, 1.0]}
    Us = {m: torch.tensor(v, dtype=torch.float64, device=dev).expand(n, 3).contiguous() for m, v in motions.items()}
    # FP64 GPU LU (partial pivoting), one factorization for both right-hand sides
    K = _assemble_dev(W, X, X, e, 1.0)
    B = torch.stack([Us["parallel"].reshape(-1), Us["normal"].reshape(-1)], 1).contiguous()
    F64 = _lu_solve_dev(K, B)
    del K
    torch.cuda.empty_cache()
    F64 = {"parallel": F64[:, 0].reshape(n, 3), "normal": F64[:, 1].reshape(n, 3)}
    # the FP64 GPU forces solve the oracle's system: the oracle's O(N^2) sum (the reference's
    # _apply loop) of the forces gives back the prescribed velocities
    Xh = X.cpu().numpy()
    for m, U in Us.items():
        back = O.evaluate("wall", Xh, Xh, F64[m].cpu().numpy(), eps)
        assert rel_l2(back, U) < 1e-12, m
    for m, U in Us.items():
        for lu in ("tf32", "bf16"):
            Fm, im = fl.resistance(W, X, U, e, method="lu", precision="mixed", lu=lu)
            err = rel_l2(Fm, F64[m])
            assert im.residual < TOL and err < TOL, (m, lu, err, im)
            record_property(f"h{h}_{m}_{lu}", {"err": err, "ir_steps": im.ir_steps, "gmres_iterations": im.iterations})


@pytest.mark.parametrize("alpha,motion", [(10.0, "translate"), ((1 + 1j) * np.sqrt(0.5), "translate"),
                                          ((1 + 1j) * np.sqrt(5.0), "rotate")])
def test_brinkman_gmres_16384_mixed_vs_converged_fp64(alpha, motion, record_property):
    N = 16384
    P = O.fibonacci_sphere(N)
    eps = 0.2 * O.mean_nn_spacing(P)
    dev = torch.device("cuda")
    X = torch.tensor(P, device=dev)
    e = torch.full((N,), eps, dtype=torch.float64, device=dev)
    if motion == "translate":
        U = torch.zeros_like(X)
        U[:, 0] = 1.0
    else:  # rotation about z: (0, 0, 1) x x
        U = torch.stack([-X[:, 1], X[:, 0], torch.zeros_like(X[:, 0])], 1)
    k = fl.Brinkmanlet3D(alpha)
    Fc, ic = fl.resistance(k, X, U, e, method="gmres", restart=50, maxiter=400, rtol=1e-13)
    assert ic.residual < 1e-13
    Fm, im = fl.resistance(k, X, U, e, method="gmres", restart=50, maxiter=200, precision="mixed")
    assert Fm.is_complex() == (complex(alpha).imag != 0)
    assert im.residual < TOL and im.ir_steps >= 1
    err = rel_l2(Fm, Fc)
    assert err < TOL, err
    record_property("err_vs_converged_fp64", err)
    record_property("ir_steps", im.ir_steps)


def test_point_on_wall_is_singular_everywhere():
    """A WallStokeslet point on z = 0 makes the resistance matrix singular: its velocity is zero
    whatever the forces.  In the reference's formula (free Stokeslet + image system evaluated
    apart) that row and column cancel only to rounding (~1e-17), and LAPACK returns meaningless
    forces with an ill-conditioning warning (rcond ~1e-34).  Here the free + image block carries
    the factor t h, the row and column are exactly zero, and both the FP64 LU and the mixed
    (unpivoted, tensor-core) LU raise LinAlgError instead of returning forces."""
    import warnings

    N = 400
    X = O.fibonacci_sphere(N) + [0.0, 0.0, 1.2]
    X[17] = [0.3, -0.2, 0.0]
    eps = 0.25 * O.mean_nn_spacing(X)
    U = np.tile([1.0, 0.0, 0.0], (N, 1))
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        O.resistance("wall", X, U, eps, method="lu")
    assert any(issubclass(x.category, scipy_linalg.LinAlgWarning) for x in w)
    K = fl.assemble(W, X, X, eps)
    assert not K[51:54].any() and not K[:, 51:54].any()
    with pytest.raises(np.linalg.LinAlgError):
        fl.resistance(W, X, U, eps, method="lu")
    for lu in ("tf32", "bf16", "fp32"):
        with pytest.raises(np.linalg.LinAlgError):
            fl.resistance(W, X, U, eps, method="lu", precision="mixed", lu=lu)
