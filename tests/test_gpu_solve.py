"""CUDA assembly, LU, tensor-core update, GMRES, resistance and swimmer solves."""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import assert_close, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
fl = pytest.importorskip("fluidlets_gb300")
from fluidlets_gb300 import _device as dv  # noqa: E402
from fluidlets_gb300 import _lib  # noqa: E402
from fluidlets_gb300.geometry import cube_sphere, fibonacci_sphere  # noqa: E402

W = fl.WallStokeslet3D()
S3 = fl.Stokeslet3D()


# ---- assembly ---------------------------------------------------------------------
def test_assemble_matches_reference_golden(golden):
    g = golden
    Y, X, e = g["as_points"], g["ev_targets"], g["ev_eps"]
    assert_close(fl.assemble(S3, Y, Y, 0.2), g["as_stokeslet"], 1e-12, 1e-14)
    assert_close(fl.assemble(W, Y, Y, e[:19]), g["as_wall"], 1e-12, 1e-14)
    assert_close(fl.assemble(fl.Brinkmanlet3D(3.0), Y, Y, 0.2), g["as_brinkman"], 1e-12, 1e-14)
    K = fl.assemble(W, Y, Y, 0.2, mu=2 - 0.5j)
    assert K.dtype == np.complex128
    assert_close(K, g["as_wall_mu"], 1e-12, 1e-14)
    assert_close(fl.assemble(W, X, Y, 0.15), g["as_rect"], 1e-12, 1e-14)


def test_assemble_matches_evaluate():
    # tests/test_kernels.py:32-36
    rng = np.random.default_rng(3)
    X = np.c_[rng.uniform(-1, 1, (12, 2)), rng.uniform(0.2, 1.5, 12)]
    F = rng.normal(size=(12, 3))
    for k in (S3, W, fl.Brinkmanlet3D(2.0)):
        K = fl.assemble(k, X, X, 0.2)
        assert np.allclose(K @ F.ravel(), fl.evaluate(k, X, X, F, 0.2).ravel(), rtol=1e-13)


def test_assemble_complex_alpha_vs_oracle():
    rng = np.random.default_rng(4)
    X = rng.normal(size=(17, 3))
    k = fl.Brinkmanlet3D(1 + 1j)
    assert_close(fl.assemble(k, X, X, 0.3), O.assemble("brinkman", X, X, 0.3, alpha=1 + 1j), 1e-12, 1e-14)


def test_assemble_low_precision_outputs():
    from fluidlets_gb300.core import _assemble_dev
    rng = np.random.default_rng(5)
    X = torch.tensor(np.c_[rng.uniform(-1, 1, (40, 2)), rng.uniform(0.2, 1.5, 40)], device="cuda")
    e = torch.full((40,), 0.1, dtype=torch.float64, device="cuda")
    K64 = _assemble_dev(W, X, X, e, 1.0)
    K32 = _assemble_dev(W, X, X, e, 1.0, out_dtype=torch.float32)
    Kbf = _assemble_dev(W, X, X, e, 1.0, out_dtype=torch.bfloat16)
    assert rel_err(K32.double().cpu().numpy(), K64.cpu().numpy()) < 1e-6
    assert rel_err(Kbf.double().cpu().numpy(), K64.cpu().numpy()) < 1e-2


@pytest.mark.parametrize("n", [1, 7, 130, 1037])
def test_symmetric_self_assembly(n):
    """Targets = sources with one blob width: half the pair evaluations, the mirror blocks
    bit-identical to the direct ones for the free kernels (every output type, complex alpha and
    mu) and equal to rounding for the wall kernel (reciprocity)."""
    from fluidlets_gb300.core import _assemble_dev
    rng = np.random.default_rng(n)
    X = torch.tensor(np.c_[rng.uniform(-1, 1, (n, 2)), rng.uniform(0.05, 1.5, n)], device="cuda")
    e = torch.full((n,), 0.07, dtype=torch.float64, device="cuda")
    for k, mu in ((S3, 1.0), (fl.Brinkmanlet3D(2.5), 1.0), (fl.Brinkmanlet3D(1 + 2j), 1.0), (S3, 2 - 0.5j)):
        for dt in (torch.float64, torch.float32, torch.bfloat16):
            if dt != torch.float64 and (mu != 1.0 or complex(k.alpha).imag != 0.0):
                continue  # complex outputs are complex128 whatever the requested type
            a = _assemble_dev(k, X, X, e, mu, out_dtype=dt)
            b = _assemble_dev(k, X, X, e, mu, out_dtype=dt, sym_eps=0.07)
            assert torch.equal(a, b), (k, mu, dt)
    a = _assemble_dev(W, X, X, e, 1.0)
    b = _assemble_dev(W, X, X, e, 1.0, sym_eps=0.07, reciprocal=True)
    assert rel_err(b.cpu().numpy(), a.cpu().numpy()) < 1e-14
    assert torch.equal(_assemble_dev(W, X, X, e, 1.0, sym_eps=0.07), a)  # no reciprocity asked: the direct kernel


def test_assemble_nearest_matches_reference(golden):
    g = golden
    xc, Xq, nn = g["an_coarse"], g["an_quad"], g["an_nearest"]
    assert np.array_equal(fl.nearest_neighbors(Xq, xc), nn)
    assert_close(fl.assemble_nearest(S3, xc, Xq, nn, len(xc), 0.05), g["an_stokeslet"], 1e-12, 1e-14)
    sh = np.array([0, 0, 1.5])
    assert_close(fl.assemble_nearest(W, xc + sh, Xq + sh, nn, len(xc), 0.05), g["an_wall"], 1e-12, 1e-14)


def test_assemble_nearest_identity_and_grouped_sum():
    # tests/test_swimming.py:12-26
    X = cube_sphere(4)
    nn = fl.nearest_neighbors(X, X)
    assert np.array_equal(nn, np.arange(len(X)))
    assert_close(fl.assemble_nearest(S3, X, X, nn, len(X), 0.1), fl.assemble(S3, X, X, 0.1), 1e-14, 1e-15)
    x, Xq = cube_sphere(3), cube_sphere(9)
    nn = fl.nearest_neighbors(Xq, x)
    A = fl.assemble_nearest(S3, x, Xq, nn, len(x), 0.05)
    f = np.random.default_rng(0).normal(size=(len(x), 3))
    assert np.allclose(A @ f.ravel(), fl.evaluate(S3, x, Xq, f[nn], 0.05).ravel(), rtol=1e-12)
    with pytest.raises(ValueError):
        fl.assemble_nearest(S3, x, Xq, np.full(len(Xq), len(x)), len(x), 0.05)


# ---- dense LU ------------------------------------------------------------------------
def lu_solve(A, b):
    L = _lib.load()
    n = A.shape[0]
    Ad = torch.tensor(A, device="cuda")
    B = torch.tensor(b.reshape(n, -1), device="cuda").contiguous()
    piv = torch.empty(n, dtype=torch.int32, device="cuda")
    nb = L.flg_lu_factor_f64_workspace(n)
    ws = dv.workspace(nb)
    info = ctypes.c_int(0)
    _lib.check(L.flg_lu_factor_f64(n, dv.ptr(Ad), n, dv.ptr(piv), ctypes.byref(info), dv.ptr(ws), nb, dv.stream()))
    _lib.check(L.flg_lu_solve_f64(n, B.shape[1], dv.ptr(Ad), n, dv.ptr(piv), dv.ptr(B), B.shape[1], dv.stream()))
    return B.cpu().numpy().reshape(b.shape), Ad.cpu().numpy(), piv.cpu().numpy()


@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 129, 300, 1000])
def test_lu_f64_matches_numpy(n):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)) + 0.1 * np.eye(n)  # general matrix: pivoting needed
    b = rng.normal(size=(n, 2))
    x, LU, piv = lu_solve(A, b)
    ref = np.linalg.solve(A, b)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-9 * max(1.0, np.linalg.cond(A) / 1e3)
    if n <= 300:  # pivots as LAPACK's getrf (0-based); larger n may differ on near-ties
        import scipy.linalg
        _, piv_ref = scipy.linalg.lu_factor(A)
        assert np.array_equal(piv, piv_ref)


def test_lu_f64_singular_raises():
    A = np.ones((70, 70))
    with pytest.raises(np.linalg.LinAlgError):
        lu_solve(A, np.ones(70))


def test_tc_rank_update_tf32_and_bf16():
    L = _lib.load()
    rng = np.random.default_rng(7)
    for m, nc in [(128, 128), (300, 257), (1024, 640), (129, 1)]:
        A = rng.normal(size=(m, 128)).astype(np.float32)
        Bt = rng.normal(size=(nc, 128)).astype(np.float32)
        C = rng.normal(size=(m, nc)).astype(np.float32)
        ref = C.astype(np.float64) - A.astype(np.float64) @ Bt.astype(np.float64).T
        scale = np.linalg.norm(A.astype(np.float64) @ Bt.astype(np.float64).T)
        ldc = (nc + 3) // 4 * 4
        for mode, tol in ((0, 3e-3), (1, 2e-2)):
            Cd = torch.zeros((m, ldc), dtype=torch.float32, device="cuda")
            Cd[:, :nc] = torch.from_numpy(C)
            Ad = torch.from_numpy(A).cuda()
            Bd = torch.from_numpy(Bt).cuda()
            nb = L.flg_tc_rank_update_workspace(m, nc, mode)
            ws = dv.workspace(nb)
            _lib.check(L.flg_tc_rank_update(dv.ptr(Cd), ldc, dv.ptr(Ad), 128, dv.ptr(Bd), 128, m, nc, mode,
                                            dv.ptr(ws), nb, dv.stream()))
            out = Cd[:, :nc].double().cpu().numpy()
            err = np.linalg.norm(out - ref) / scale
            assert err < tol, (m, nc, mode, err)
            assert err > 1e-8  # the tensor cores really ran at reduced precision


@pytest.mark.parametrize("mode", ["fp32", "tf32", "bf16"])
@pytest.mark.parametrize("n", [100, 128, 300, 1000])
def test_lowp_lu_factors(mode, n):
    from fluidlets_gb300.core import _lowp_factor_dev
    X = fibonacci_sphere(n // 3 + 1)[: n // 3] if n >= 3 else None
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)) / np.sqrt(n) + 4.0 * np.eye(n)  # no pivoting needed
    K = torch.tensor(A, device="cuda")
    K32, ld32, dinv, A32 = _lowp_factor_dev(K, mode)
    assert torch.equal(A32[:, :n], K.float())  # unfactored copy for the inner matvecs
    LU = K32[:, :n].double().cpu().numpy()
    Lm = np.tril(LU, -1) + np.eye(n)
    Um = np.triu(LU)
    err = np.linalg.norm(Lm @ Um - A) / np.linalg.norm(A)
    tol = {"fp32": 1e-6, "tf32": 2e-3, "bf16": 2e-2}[mode]
    assert err < tol, err
    del X
    # dinv: inverses of the unit-lower and upper factors of every 128 x 128 diagonal block
    nblk = (n + 127) // 128
    Dv = dinv.double().cpu().numpy().reshape(2, nblk, 128, 128)
    for k in range(nblk):
        r0, r1 = 128 * k, min(n, 128 * k + 128)
        w = r1 - r0
        Lk = np.eye(128)
        Uk = np.eye(128)
        Lk[:w, :w] = Lm[r0:r1, r0:r1]
        Uk[:w, :w] = Um[r0:r1, r0:r1]
        assert np.abs(Dv[0, k] @ Lk - np.eye(128)).max() < 1e-5, (k, "Linv")
        assert np.abs(Dv[1, k] @ Uk - np.eye(128)).max() < 1e-5, (k, "Uinv")
        assert np.abs(np.triu(Dv[0, k], 1)).max() == 0 and np.abs(np.tril(Dv[1, k], -1)).max() == 0


@pytest.mark.parametrize("n", [100, 128, 300, 5000, 19500])
def test_lowp_apply_matches_triangular_solves(n):
    """flg_lu_solve_lowp: x = U^-1 L^-1 b with the FP32 factors; 19,500 unknowns give more
    128-row blocks than SMs (one CTA owns two) and a partial last block."""
    from fluidlets_gb300.core import _lowp_factor_dev
    L = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(n)
    K = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g) / n ** 0.5
    K.diagonal().add_(4.0)
    K32, ld32, dinv, A32 = _lowp_factor_dev(K, "fp32")
    del A32, K
    b = torch.randn(n, device="cuda", dtype=torch.float64, generator=g)
    x = torch.empty_like(b)
    nb = L.flg_lu_solve_lowp_workspace(n)
    ws = dv.workspace(nb)
    _lib.check(L.flg_lu_solve_lowp(n, dv.ptr(K32), ld32, dv.ptr(dinv), dv.ptr(b), dv.ptr(x), dv.ptr(ws), nb,
                                   dv.stream()))
    LU = K32[:, :n].double()
    y = torch.linalg.solve_triangular(LU, b[:, None], upper=False, unitriangular=True)
    ref = torch.linalg.solve_triangular(LU, y, upper=True)[:, 0]
    err = float(torch.linalg.vector_norm(x - ref) / torch.linalg.vector_norm(ref))
    assert err < 1e-5, err


@pytest.mark.parametrize("rows,cols", [(1, 1), (5, 3), (97, 250), (1536, 1536), (3000, 4099)])
def test_gemv_f64_and_f32(rows, cols):
    L = _lib.load()
    rng = np.random.default_rng(rows + cols)
    A = rng.normal(size=(rows, cols))
    x = rng.normal(size=cols)
    ld = (cols + 31) // 32 * 32
    Ad = torch.zeros((rows, ld), dtype=torch.float64, device="cuda")
    Ad[:, :cols] = torch.tensor(A)
    A32 = Ad.float()
    xd = torch.tensor(x, device="cuda")
    y = torch.empty(rows, dtype=torch.float64, device="cuda")
    _lib.check(L.flg_gemv_f64(rows, cols, dv.ptr(Ad), ld, dv.ptr(xd), dv.ptr(y), dv.stream()))
    ref = A @ x
    scale = np.abs(A) @ np.abs(x)
    assert np.all(np.abs(y.cpu().numpy() - ref) <= 1e-13 * scale + 1e-300)
    _lib.check(L.flg_gemv_f32(rows, cols, dv.ptr(A32), ld, dv.ptr(xd), dv.ptr(y), dv.stream()))
    # the FP32 entries times the FP64 x, to about FP64 accuracy (compensated FP32 arithmetic)
    ref32 = A32[:, :cols].double().cpu().numpy() @ x
    assert np.all(np.abs(y.cpu().numpy() - ref32) <= 1e-12 * scale + 1e-300)


# ---- resistance ------------------------------------------------------------------------
def test_resistance_lu_matches_reference(golden):
    g = golden
    S, e, U = g["rs_points"], float(g["rs_eps"]), g["rs_U"]
    f, info = fl.resistance(S3, S, U, e, method="lu")
    assert info.method == "lu" and info.residual < 1e-12
    assert_close(f, g["rs_lu_forces"], 1e-10, 1e-12)
    f, info = fl.resistance(W, g["rs_wall_points"], np.tile([0, 0, 1.0], (len(S), 1)), e, method="lu")
    assert_close(f, g["rs_wall_lu_forces"], 1e-10, 1e-12)


def test_resistance_gmres_matches_reference(golden):
    g = golden
    S, e, U = g["rs_points"], float(g["rs_eps"]), g["rs_U"]
    f, info = fl.resistance(S3, S, U, e, method="gmres")
    assert info.method == "gmres" and info.residual < 1e-9
    assert abs(info.iterations - int(g["rs_gmres_iters"])) <= 2
    assert rel_err(f, g["rs_gmres_forces"]) < 1e-8
    f, info = fl.resistance(fl.Brinkmanlet3D(1.0), S, U, e, method="gmres", restart=20)
    assert rel_err(f, g["rs_brink_gmres_forces"]) < 1e-8
    assert abs(info.iterations - int(g["rs_brink_gmres_iters"])) <= 3


def test_sphere_drag_lu_and_gmres():
    # tests/test_kernels.py:61-73
    n = 400
    X = fibonacci_sphere(n)
    eps = 0.5 * np.sqrt(4 * np.pi / n)
    U = np.tile([1.0, 0, 0], (n, 1))
    F_lu, info_lu = fl.resistance(S3, X, U, eps, method="lu")
    F_gm, info_gm = fl.resistance(S3, X, U, eps, method="gmres")
    assert info_lu.residual < 1e-12 and info_gm.residual < 1e-9
    assert np.allclose(F_lu, F_gm, rtol=1e-6, atol=1e-8)
    drag = F_lu[:, 0].sum() / (6 * np.pi)
    assert 1.0 < drag < 1.02


@pytest.mark.parametrize("lu", ["tf32", "bf16", "fp32"])
def test_mixed_lu_resistance_reaches_fp64(lu):
    n = 800
    X = fibonacci_sphere(n) + [0, 0, 1.5]
    eps = 0.25 * np.sqrt(4 * np.pi / n)
    U = np.tile([1.0, 0, 0.5], (n, 1))
    F64, _ = fl.resistance(W, X, U, eps, method="lu")
    Fm, info = fl.resistance(W, X, U, eps, method="lu", precision="mixed", lu=lu)
    assert info.residual < 1e-10 and info.precision == "mixed"
    assert np.linalg.norm(Fm - F64) / np.linalg.norm(F64) < 1e-9


def test_mixed_gmres_resistance_reaches_fp64():
    n = 2000
    X = fibonacci_sphere(n)
    eps = 0.2 * np.sqrt(4 * np.pi / n)
    U = np.tile([1.0, 0, 0], (n, 1))
    for k in (S3, fl.Brinkmanlet3D(10.0)):
        F64, i64 = fl.resistance(k, X, U, eps, method="gmres", restart=50)
        Fm, im = fl.resistance(k, X, U, eps, method="gmres", restart=50, precision="mixed")
        assert im.residual < 1e-10 and im.ir_steps >= 1
        assert np.linalg.norm(Fm - F64) / np.linalg.norm(F64) < 1e-8


def test_complex_viscosity_resistance_vs_oracle():
    n = 150
    X = fibonacci_sphere(n)
    eps = 0.4 * np.sqrt(4 * np.pi / n)
    U = np.tile([1.0, 0, 0], (n, 1))
    mu = 1.0 - 0.3j
    for method in ("lu", "gmres"):
        f, info = fl.resistance(S3, X, U, eps, mu=mu, method=method)
        ref, _ = O.resistance("stokeslet", X, U, eps, mu=mu, method="lu")
        assert f.dtype == np.complex128 and rel_err(f, ref) < 1e-8


def test_complex_alpha_gmres_vs_oracle():
    n = 300
    X = fibonacci_sphere(n)
    eps = 0.2 * np.sqrt(4 * np.pi / n)
    U = np.tile([1.0, 0, 0], (n, 1))
    a = (1 + 1j) * np.sqrt(10 / 2)
    K = O.assemble("brinkman", X, X, eps, alpha=a)
    ref = np.linalg.solve(K, U.ravel()).reshape(n, 3)
    for prec in ("fp64", "mixed"):
        f, info = fl.resistance(fl.Brinkmanlet3D(a), X, U, eps, method="gmres", restart=50, precision=prec)
        assert f.dtype == np.complex128 and info.residual < 1e-10
        assert rel_err(f, ref) < 1e-8
    f, info = fl.resistance(fl.Brinkmanlet3D(a), X, U, eps, method="lu")
    assert rel_err(f, ref) < 1e-10


def test_gmres_non_convergence_raises():
    n = 300
    X = fibonacci_sphere(n)
    with pytest.raises(RuntimeError):
        fl.resistance(S3, X, np.tile([1.0, 0, 0], (n, 1)), 0.05, method="gmres", restart=2, maxiter=1)


def test_legacy_towers_gmres(legacy_towers):
    # tests/legacy/test_phase1_port.py:62-74
    d = legacy_towers
    X, U, F_legacy = d["x0"], d["Vel"], d["Forces"]
    F, info = fl.resistance(W, X, U, 0.5, method="gmres")
    assert info.residual < 1e-9
    on_wall = X[:, 2] == 0
    assert np.abs(F[on_wall]).max() < 1e-12
    above = ~on_wall
    assert np.linalg.norm(F[above] - F_legacy[above]) / np.linalg.norm(F_legacy[above]) < 1e-3
    for k in range(3):
        tower = slice(147 * k, 147 * (k + 1))
        assert np.isclose(F[tower, 0].sum(), F_legacy[tower, 0].sum(), rtol=1e-5)


# ---- swimming ------------------------------------------------------------------------------
def test_swimming_problem_matches_reference(golden):
    g = golden
    shape = fl.SwimmerShape(x=g["sw_x"], v=g["sw_v"], X=g["sw_X"])
    st = fl.swimming_problem(shape, g["sw_x0"], g["sw_B"], 0.05)
    assert np.array_equal(st.nearest, g["sw_nearest"])
    assert rel_err(st.U, g["sw_U"]) < 1e-10 and rel_err(st.Omega, g["sw_Omega"]) < 1e-10
    assert rel_err(st.forces, g["sw_forces"]) < 1e-10
    sm = fl.swimming_problem(shape, g["sw_x0"], g["sw_B"], 0.05, precision="mixed")
    assert rel_err(sm.U, g["sw_U"]) < 1e-9 and rel_err(sm.forces, g["sw_forces"]) < 1e-9


def test_uniform_slip_swims_rigidly():
    # tests/test_swimming.py:34-40
    V = np.array([0.2, -0.1, 0.7])
    x = cube_sphere(4)
    st = fl.swimming_problem(fl.SwimmerShape(x=x, v=-np.tile(V, (len(x), 1)), X=cube_sphere(10)), np.zeros(3),
                             np.eye(3), 0.05)
    assert np.allclose(st.U, V, atol=1e-12) and np.allclose(st.Omega, 0, atol=1e-12)
    assert np.abs(st.forces).max() < 1e-10


def test_trajectory_of_steady_slip_swimmer():
    # tests/test_swimming.py:58-69
    V = np.array([0.0, 0.0, 0.5])
    Wb = np.array([0.0, 0.0, 0.25])

    def shape_at(t):
        x = cube_sphere(3)
        return fl.SwimmerShape(x=x, v=-(V + np.cross(Wb, x)), X=cube_sphere(6))

    tr = fl.swim(shape_at, (0.0, 2.0), 0.05, t_eval=[2.0], rtol=1e-9, atol=1e-12)
    assert np.allclose(tr.x0[-1], [0, 0, 1.0], atol=1e-7)
    angle = 0.25 * 2.0
    assert np.allclose(tr.B[-1][:, 0], [np.cos(angle), np.sin(angle), 0], atol=1e-7)


def test_swimmer_plan_replays_match_direct_solves():
    """One captured swimmer graph, replayed for several stages (new points, origin, orientation),
    equals the FP64 swimming_problem of each stage.  Flagellum amplitude 0.08: with the default
    0.2 the two flagella cross during the beat and the system is near-singular there."""
    from fluidlets_gb300.geometry import biflagellate_shape
    from fluidlets_gb300.swimming import SwimmerPlan

    rng = np.random.default_rng(3)
    s0 = biflagellate_shape(0.0, amplitude=0.08)
    plan = SwimmerPlan(fl.Stokeslet3D(), len(s0.x), len(s0.X), 0.02)
    for t in (0.0, 0.37, 0.81):
        s = biflagellate_shape(t, amplitude=0.08)
        x0 = rng.normal(size=3)
        B = np.linalg.qr(rng.normal(size=(3, 3)))[0]
        B *= np.sign(np.linalg.det(B))
        ref = fl.swimming_problem(s, x0, B, 0.02)
        xw, Xw = x0 + s.x @ B.T, x0 + s.X @ B.T
        rhs = np.zeros(3 * len(s.x) + 6)
        rhs[:3 * len(s.x)] = (s.v @ B.T).ravel()
        U, Om, F, nn = plan.solve(xw, Xw, x0, rhs)
        assert np.array_equal(nn, ref.nearest)
        # the rigid motion as one vector: the rotation rate here is ~300 x smaller than U, so its own
        # relative error would measure the refinement's residual against a tiny component
        assert rel_err(np.r_[U, Om], np.r_[ref.U, ref.Omega]) < 1e-9 and rel_err(F, ref.forces) < 1e-9
    plan.close()


def test_trajectory_mixed_precision_swim():
    # the steady slip swimmer of tests/test_swimming.py:58-69 through the captured-graph stages
    V = np.array([0.0, 0.0, 0.5])
    Wb = np.array([0.0, 0.0, 0.25])

    def shape_at(t):
        x = cube_sphere(3)
        return fl.SwimmerShape(x=x, v=-(V + np.cross(Wb, x)), X=cube_sphere(6))

    tr = fl.swim(shape_at, (0.0, 2.0), 0.05, t_eval=[2.0], rtol=1e-9, atol=1e-12, precision="mixed")
    assert np.allclose(tr.x0[-1], [0, 0, 1.0], atol=1e-7)
    angle = 0.25 * 2.0
    assert np.allclose(tr.B[-1][:, 0], [np.cos(angle), np.sin(angle), 0], atol=1e-7)


# ---- rigid bodies: mobility problem and grand resistance matrix ----------------------------
def _oracle_mobility(X, eps, F, T, c, kind="stokeslet"):
    # tutorials/03_mobility_resistance_swimming.ipynb (sedimenting sphere) with rotation and torque
    N = len(X)
    r = X - c
    A = np.zeros((3 * N + 6, 3 * N + 6))
    A[:3 * N, :3 * N] = O.assemble(kind, X, X, eps)
    for k in range(N):
        A[3 * k:3 * k + 3, 3 * N:3 * N + 3] = -np.eye(3)
        A[3 * k:3 * k + 3, 3 * N + 3:] = O.cross_matrix(r[k])
        A[3 * N:3 * N + 3, 3 * k:3 * k + 3] = np.eye(3)
        A[3 * N + 3:, 3 * k:3 * k + 3] = O.cross_matrix(X[k])
    rhs = np.r_[np.zeros(3 * N), F, T + np.cross(c, F)]
    s = np.linalg.solve(A, rhs)
    return s[3 * N:3 * N + 3], s[3 * N + 3:], s[:3 * N].reshape(N, 3)


def test_settling_sphere_mobility():
    X = cube_sphere(8)
    F = -6 * np.pi * np.array([0.0, 0.0, 1.0])
    U, Om, f = fl.rigid_body_mobility(fl.Stokeslet3D(), X, 0.05, F)
    assert np.allclose(U, [0, 0, -1], atol=0.03) and np.abs(Om).max() < 1e-10
    Ur, Omr, fr = _oracle_mobility(X, 0.05, F, np.zeros(3), X.mean(0))
    assert rel_err(U, Ur) < 1e-10 and rel_err(f, fr) < 1e-9
    Um, Omm, fm = fl.rigid_body_mobility(fl.Stokeslet3D(), X, 0.05, F, precision="mixed")
    assert rel_err(Um, Ur) < 1e-9 and rel_err(fm, fr) < 1e-8


def test_resistance_matrix_sphere_and_consistency():
    X = cube_sphere(8)
    R = fl.resistance_matrix(fl.Stokeslet3D(), X, 0.05)
    assert np.abs(R - R.T).max() < 1e-9 * np.abs(R).max()           # Lorentz reciprocity
    assert np.allclose(np.diag(R)[:3], 6 * np.pi, rtol=0.03)         # Stokes drag 6 pi mu a
    assert np.allclose(np.diag(R)[3:], 8 * np.pi, rtol=0.05)         # rotation 8 pi mu a^3
    assert np.abs(R[:3, 3:]).max() < 1e-9 * np.abs(R).max()
    K = O.assemble("stokeslet", X, X, 0.05)
    c = X.mean(0)
    cols = []
    for j in range(6):
        u = np.zeros((len(X), 3))
        if j < 3:
            u[:, j] = 1.0
        else:
            u = np.cross(np.eye(3)[j - 3], X - c)
        f = np.linalg.solve(K, u.ravel()).reshape(-1, 3)
        cols.append(np.r_[f.sum(0), np.cross(X - c, f).sum(0)])
    Ro = np.array(cols).T
    assert rel_err(R, Ro) < 1e-10
    assert rel_err(fl.resistance_matrix(fl.Stokeslet3D(), X, 0.05, precision="mixed"), Ro) < 1e-9
    # an off-centre ellipsoid near a wall: the mobility solution satisfies R [U; Omega] = [F; T]
    E = cube_sphere(6) * np.array([1.5, 1.0, 0.7]) + np.array([0.0, 0.0, 2.0])
    W = fl.WallStokeslet3D()
    F, T = np.array([0.3, -1.0, 0.5]), np.array([0.2, 0.1, -0.4])
    U, Om, _ = fl.rigid_body_mobility(W, E, 0.05, F, T)
    RE = fl.resistance_matrix(W, E, 0.05)
    assert rel_err(RE @ np.r_[U, Om], np.r_[F, T]) < 1e-9


# ---- bucket assembly (solve server) -------------------------------------------------------------
@pytest.mark.parametrize("kind", ["stokeslet", "wall", "brinkman"])
def test_bucket_assembly_uniform_matches_full_and_pads_with_identity(kind):
    """flg_assemble_bucket_uniform (one blob width, half the pairs) equals flg_assemble_bucket:
    bit for bit for the free kernels, to rounding for the wall kernel (its mirror blocks are the
    transposes, by reciprocity); padded rows and columns are the identity."""
    L = _lib.load()
    rng = np.random.default_rng(11)
    n_cap, n_real = 384, 301
    pts = np.zeros((n_cap, 3))
    pts[:n_real] = np.c_[rng.uniform(-1, 1, (n_real, 2)), rng.uniform(0.1, 1.5, n_real)]
    P = torch.tensor(pts, device="cuda")
    E = torch.full((n_cap,), 0.07, dtype=torch.float64, device="cuda")
    NR = torch.tensor([n_real], dtype=torch.int64, device="cuda")
    code = _lib.KIND[kind]
    are = 2.5 if kind == "brinkman" else 0.0
    n = 3 * n_cap
    out = {}
    for name in ("flg_assemble_bucket", "flg_assemble_bucket_uniform"):
        K = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(getattr(L, name)(code, are, 0.0, dv.ptr(P), dv.ptr(E), dv.ptr(NR), n_cap, 1.0, dv.ptr(K), _lib.F64,
                                    n, dv.stream()))
        out[name] = K.cpu().numpy()
    full, sym = out["flg_assemble_bucket"], out["flg_assemble_bucket_uniform"]
    assert np.isfinite(sym).all()
    if kind == "wall":
        assert rel_err(sym, full) < 1e-14
    else:
        assert np.array_equal(sym, full)
    r = 3 * n_real
    assert np.array_equal(sym[r:, r:], np.eye(n - r)) and not sym[:r, r:].any() and not sym[r:, :r].any()
    ref = O.assemble({"stokeslet": "stokeslet", "wall": "wall", "brinkman": "brinkman"}[kind], pts[:n_real],
                     pts[:n_real], 0.07, alpha=are)
    assert_close(sym[:r, :r], ref, 1e-12, 1e-14)
