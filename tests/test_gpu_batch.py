"""Batched bucket kernels: the systems of one bucket in one sequence of launches.

flg_assemble_bucket_batched (one launch, system index in grid z),
flg_lu_factor_lowp_batched_async (one CTA per system for the diagonal blocks, one tensor-core
launch over the tiles of all systems for the panels and updates) and
flg_bucket_batch_graph_create give every system of a batch what its own single-system call
gives, bit for bit, and report a bad pivot of one system in that system's flags only.  The
refined forces of each system of a batch then meet the 1e-10 target against the FP64 oracle
solve of that system alone.
"""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
fl = pytest.importorskip("fluidlets_gb300")
from fluidlets_gb300 import _device as dv  # noqa: E402
from fluidlets_gb300 import _lib  # noqa: E402


def _ld32(n):
    return (n + 31) // 32 * 32


def _factor_single(A32, n, ld, mode):
    L = _lib.load()
    dinv = torch.full((L.flg_lu_lowp_dinv_elems(n),), float("nan"), dtype=torch.float32, device="cuda")
    flags = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    nb = L.flg_lu_factor_lowp_workspace(n, mode)
    ws = dv.workspace(nb)
    _lib.check(L.flg_lu_factor_lowp_async(n, dv.ptr(A32), ld, mode, dv.ptr(dinv), dv.ptr(flags), dv.ptr(ws), nb,
                                          dv.stream()), "LU")
    torch.cuda.synchronize()
    return A32, dinv, flags


def _factor_batched(A32, n, ld, nbat, mode):
    L = _lib.load()
    de = L.flg_lu_lowp_dinv_elems(n)
    dinv = torch.full((nbat, de), float("nan"), dtype=torch.float32, device="cuda")
    flags = torch.full((nbat, 2), -1, dtype=torch.int32, device="cuda")
    nb = L.flg_lu_factor_lowp_batched_workspace(n, nbat, mode)
    ws = dv.workspace(nb)
    _lib.check(L.flg_lu_factor_lowp_batched_async(n, nbat, dv.ptr(A32), ld, n * ld, mode, dv.ptr(dinv),
                                                  dv.ptr(flags), dv.ptr(ws), nb, dv.stream()), "batched LU")
    torch.cuda.synchronize()
    return A32, dinv, flags


def _systems(nbat, n, ld, seed):
    """nbat diagonally dominant FP32 systems (the unpivoted LU is stable on them), padded to ld."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.zeros((nbat, n, ld), dtype=torch.float32, device="cuda")
    A[:, :, :n] = torch.randn((nbat, n, n), generator=g, device="cuda") / n ** 0.5
    A[:, :, :n] += 3.0 * torch.eye(n, device="cuda")
    return A


@pytest.mark.parametrize("n,lu", [(1152, "tf32"), (1152, "bf16:256"), (1536, "tf32:128"), (8448, "tf32"),
                                  (8448, "bf16")])
def test_batched_lu_equals_single_lu_bitwise(n, lu):
    """n = 1,152 and 1,536: 512-column outer panels (one and a half, and three, of them);
    n = 8,448: 1,024-column outer panels with a partial last one."""
    nbat = 3
    mode = _lib.lu_mode(lu)
    ld = _ld32(n)
    A = _systems(nbat, n, ld, seed=n)
    Ab, dinvb, flagsb = _factor_batched(A.clone(), n, ld, nbat, mode)
    assert not flagsb.any()
    for z in range(nbat):
        As, dinvs, flagss = _factor_single(A[z].clone(), n, ld, mode)
        assert not flagss.any()
        assert torch.equal(Ab[z], As), (lu, z)
        assert torch.equal(dinvb[z], dinvs), (lu, z)


def test_batched_lu_flags_the_singular_system_only():
    n, nbat, ld = 768, 3, 768
    A = _systems(nbat, n, ld, seed=5)
    A[1, 200, :] = 0.0  # system 1: a zero row -> a zero pivot at row 200 at the latest
    A[1, :, 200] = 0.0
    _, _, flags = _factor_batched(A, n, ld, nbat, _lib.lu_mode("tf32"))
    f = flags.cpu().numpy()
    assert f[0, 0] == 0 and f[2, 0] == 0
    assert 1 <= f[1, 0] <= 201
    assert not f[:, 1].any()


def test_batched_lu_rejects_fp32_mode_and_bad_stride():
    L = _lib.load()
    n, ld = 256, 256
    A = _systems(2, n, ld, seed=1)
    dinv = torch.empty((2, L.flg_lu_lowp_dinv_elems(n)), dtype=torch.float32, device="cuda")
    flags = torch.zeros((2, 2), dtype=torch.int32, device="cuda")
    nb = L.flg_lu_factor_lowp_batched_workspace(n, 2, _lib.lu_mode("tf32"))
    ws = dv.workspace(nb)
    for mode, stride in ((_lib.lu_mode("fp32"), n * ld), (_lib.lu_mode("tf32"), n * ld - 4)):
        st = L.flg_lu_factor_lowp_batched_async(n, 2, dv.ptr(A), ld, stride, mode, dv.ptr(dinv), dv.ptr(flags),
                                                dv.ptr(ws), nb, dv.stream())
        assert st == _lib.FLG_ERR_INVALID


def _bucket_inputs(kind, n_cap, counts, seed, eps_per_point=False):
    rng = np.random.default_rng(seed)
    nbat = len(counts)
    pts = np.zeros((nbat, n_cap, 3))
    eps = np.ones((nbat, n_cap))
    for z, c in enumerate(counts):
        P = O.fibonacci_sphere(c) * rng.uniform(0.8, 1.2)
        if kind == "wall":
            P = P + [0.0, 0.0, 1.0 + rng.uniform(0.05, 0.5)]
        pts[z, :c] = P
        e = 0.25 * O.mean_nn_spacing(P)
        eps[z, :c] = e * (rng.uniform(0.9, 1.1, c) if eps_per_point else 1.0)
        if not eps_per_point:
            eps[z, :] = e
    return pts, eps


@pytest.mark.parametrize("kind,uniform", [("stokeslet", True), ("wall", True), ("wall", False),
                                          ("brinkman", False)])
def test_batched_bucket_assembly_equals_single(kind, uniform):
    L = _lib.load()
    n_cap, counts = 384, [384, 301, 17]
    pts, eps = _bucket_inputs(kind, n_cap, counts, seed=7, eps_per_point=not uniform)
    code = _lib.KIND[kind]
    are = 2.5 if kind == "brinkman" else 0.0
    n, nbat = 3 * n_cap, len(counts)
    P = torch.tensor(pts, device="cuda")
    E = torch.tensor(eps, device="cuda")
    NR = torch.tensor(counts, dtype=torch.int64, device="cuda")
    Kb = torch.full((nbat, n, n), float("nan"), dtype=torch.float64, device="cuda")
    _lib.check(L.flg_assemble_bucket_batched(code, are, 0.0, dv.ptr(P), dv.ptr(E), int(uniform), dv.ptr(NR), n_cap,
                                             nbat, 1.0, dv.ptr(Kb), _lib.F64, n, n * n, dv.stream()))
    single = L.flg_assemble_bucket_uniform if uniform else L.flg_assemble_bucket
    for z in range(nbat):
        Ks = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(single(code, are, 0.0, dv.ptr(P[z]), dv.ptr(E[z]), dv.ptr(NR[z:z + 1]), n_cap, 1.0, dv.ptr(Ks),
                          _lib.F64, n, dv.stream()))
        assert torch.equal(Kb[z], Ks), z


def test_batched_bucket_graph_matches_single_graphs_and_oracle():
    """Three Stokeslet spheres of one bucket (768 points: 700, 768 and 512 real) through one
    batched graph; each system's factors equal its own bucket graph's, and its refined forces
    (the captured FP64 refinement on that system's buffers) meet 1e-10 against the oracle."""
    from fluidlets_gb300.core import IrGraph

    L = _lib.load()
    kind, n_cap, counts = "stokeslet", 768, [700, 768, 512]
    pts, eps = _bucket_inputs(kind, n_cap, counts, seed=3)
    n, nbat, ld32 = 3 * n_cap, len(counts), _ld32(3 * n_cap)
    mode = _lib.lu_mode("tf32")
    st = torch.cuda.Stream()
    sp = ctypes.c_void_p(st.cuda_stream)
    P = torch.tensor(pts, device="cuda")
    E = torch.tensor(eps, device="cuda")
    NR = torch.tensor(counts, dtype=torch.int64, device="cuda")
    K = torch.empty((nbat, n, n), dtype=torch.float64, device="cuda")
    K32 = torch.empty((nbat, n, ld32), dtype=torch.float32, device="cuda")
    A32 = torch.empty((nbat, n, ld32), dtype=torch.float32, device="cuda")
    de = L.flg_lu_lowp_dinv_elems(n)
    dinv = torch.empty((nbat, de), dtype=torch.float32, device="cuda")
    flags = torch.full((nbat, 2), -1, dtype=torch.int32, device="cuda")
    nb = L.flg_lu_factor_lowp_batched_workspace(n, nbat, mode)
    ws = dv.workspace(nb)
    h = ctypes.c_void_p(0)
    _lib.check(L.flg_bucket_batch_graph_create(_lib.KIND[kind], 0.0, 0.0, dv.ptr(P), dv.ptr(E), 1, dv.ptr(NR), n_cap,
                                               nbat, 1.0, dv.ptr(K), dv.ptr(A32), dv.ptr(K32), ld32, mode,
                                               dv.ptr(dinv), dv.ptr(flags), dv.ptr(ws), nb, sp, ctypes.byref(h)))
    try:
        K32.fill_(float("nan"))
        _lib.check(L.flg_graph_launch(h, sp))
        st.synchronize()
        assert not flags.any()
        # the single-system bucket graph of each system
        for z in range(nbat):
            Ks = torch.empty((n, n), dtype=torch.float64, device="cuda")
            K32s = torch.empty((n, ld32), dtype=torch.float32, device="cuda")
            A32s = torch.empty((n, ld32), dtype=torch.float32, device="cuda")
            dinvs = torch.empty(de, dtype=torch.float32, device="cuda")
            flagss = torch.zeros(2, dtype=torch.int32, device="cuda")
            nbs = L.flg_lu_factor_lowp_workspace(n, mode)
            wss = dv.workspace(nbs)
            hs = ctypes.c_void_p(0)
            _lib.check(L.flg_bucket_graph_create(_lib.KIND[kind], 0.0, 0.0, dv.ptr(P[z]), dv.ptr(E[z]), 1,
                                                 dv.ptr(NR[z:z + 1]), n_cap, 1.0, dv.ptr(Ks), dv.ptr(A32s),
                                                 dv.ptr(K32s), ld32, mode, dv.ptr(dinvs), dv.ptr(flagss), dv.ptr(wss),
                                                 nbs, sp, ctypes.byref(hs)))
            try:
                _lib.check(L.flg_graph_launch(hs, sp))
                st.synchronize()
            finally:
                L.flg_graph_destroy(hs)
            assert torch.equal(K[z], Ks) and torch.equal(A32[z], A32s), z
            assert torch.equal(K32[z], K32s) and torch.equal(dinv[z], dinvs), z
        # refinement per system on the batch's buffers
        for z, c in enumerate(counts):
            U = np.tile([1.0, 0.0, 0.0], (c, 1))
            b = torch.zeros(n, dtype=torch.float64, device="cuda")
            b[:3 * c] = torch.tensor(U.ravel(), device="cuda")
            x = torch.zeros(n, dtype=torch.float64, device="cuda")
            ir = IrGraph(K[z], A32[z], K32[z], ld32, dinv[z], b, x, 1e-12, stream=st)
            try:
                ir.launch(st)
                status, it, outer, resid = ir.result(st)
            finally:
                ir.close()
            assert status == 0 and resid < 1e-12
            F = x[:3 * c].reshape(c, 3).cpu().numpy()
            assert not x[3 * c:].any()
            ref, _ = O.resistance(kind, pts[z, :c], U, eps[z, 0], method="lu")
            assert np.linalg.norm(F - ref) / np.linalg.norm(ref) < 1e-10, z
    finally:
        L.flg_graph_destroy(h)


def test_batched_swimmer_graph_matches_single_plans():
    """Three biflagellate swimmer instants (678 unknowns each) through one SwimmerPlan of three
    systems (one batched graph, one refinement per system): each equals its own single-system
    plan's solve and the plain FP64 swimmer solve."""
    from fluidlets_gb300.geometry import biflagellate_shape
    from fluidlets_gb300.swimming import SwimmerPlan

    rng = np.random.default_rng(4)
    items = []
    for t in (0.1, 0.45, 0.8):
        sh = biflagellate_shape(t, amplitude=0.08)
        B = np.linalg.qr(rng.normal(size=(3, 3)))[0]
        B *= np.sign(np.linalg.det(B))
        x0 = rng.normal(size=3) * 0.1
        x = x0 + sh.x @ B.T
        X = x0 + sh.X @ B.T
        rhs = np.zeros(3 * len(x) + 6)
        rhs[:3 * len(x)] = (sh.v @ B.T).ravel()
        items.append((sh, B, x0, (x, X, x0, rhs)))
    N, Q = len(items[0][3][0]), len(items[0][3][1])
    group = SwimmerPlan(fl.Stokeslet3D(), N, Q, 0.02, cap=3)
    single = SwimmerPlan(fl.Stokeslet3D(), N, Q, 0.02)
    try:
        outs = group.solve_group([it[3] for it in items])
        for (sh, B, x0, item), out in zip(items, outs):
            assert not isinstance(out, Exception), out
            U, Om, F, nn, resid = out
            U1, Om1, F1, nn1 = single.solve(*item)
            assert resid < 1e-10
            assert np.array_equal(nn, nn1)
            assert np.array_equal(U, U1) and np.array_equal(Om, Om1) and np.array_equal(F, F1)
            ref = fl.swimming_problem(sh, x0, B, 0.02)
            both, both_ref = np.concatenate([U, Om]), np.concatenate([ref.U, ref.Omega])
            assert np.linalg.norm(both - both_ref) / np.linalg.norm(both_ref) < 1e-9
        # a group of two on the same plan (the graph of two systems)
        outs2 = group.solve_group([items[2][3], items[0][3]])
        assert np.array_equal(outs2[0][0], outs[2][0]) and np.array_equal(outs2[1][2], outs[0][2])
    finally:
        group.close()
        single.close()
