"""CUDA kernel sums vs the oracle and the reference's golden vectors."""
import numpy as np
import pytest

import oracle as O
from conftest import assert_close, legacy_grid_points, rel_err

pytestmark = pytest.mark.gpu

fl = pytest.importorskip("fluidlets_gb300")
KERNELS = {"stokeslet": fl.Stokeslet3D(), "wall": fl.WallStokeslet3D()}


def kern(kind, alpha=0.0):
    return fl.Brinkmanlet3D(alpha) if kind == "brinkman" else KERNELS[kind]


@pytest.mark.parametrize("name,kind,alpha", [("stokeslet", "stokeslet", 0.0), ("wall", "wall", 0.0),
                                             ("brinkman_0", "brinkman", 0.0), ("brinkman_0.5", "brinkman", 0.5),
                                             ("brinkman_3", "brinkman", 3.0), ("brinkman_20", "brinkman", 20.0)])
def test_fp64_matches_reference_golden(golden, name, kind, alpha):
    g = golden
    u = fl.evaluate(kern(kind, alpha), g["ev_targets"], g["ev_sources"], g["ev_forces"], g["ev_eps"])
    assert u.dtype == np.float64 and u.shape == (33, 3)
    assert_close(u, g[f"ev_{name}"], rtol=1e-12, atol_rel=1e-14)


def test_legacy_matlab_vectors(legacy_kernels):
    d = legacy_kernels
    u = fl.evaluate(fl.Stokeslet3D(), d["targets"], d["sources"], d["strengths"], d["deltas"])
    assert np.allclose(u, d["V_stokeslet"], rtol=1e-13, atol=1e-15)
    u = fl.evaluate(fl.WallStokeslet3D(), d["targets"], d["sources"], d["strengths"], d["deltas"])
    assert np.allclose(u, d["V_stokeslet"] + d["V_image"], rtol=1e-13, atol=1e-15)
    u = fl.evaluate(fl.WallStokeslet3D(), d["wall"], d["sources"], d["strengths"], d["deltas"])
    assert np.allclose(u, d["V_wall_total"], atol=1e-15)


def test_complex_viscosity_and_strengths(golden):
    g = golden
    X, Y, F, e = g["ev_targets"], g["ev_sources"], g["ev_forces"], g["ev_eps"]
    u = fl.evaluate(fl.Stokeslet3D(), X, Y, F, e, mu=2 - 0.5j)
    assert u.dtype == np.complex128
    assert_close(u, g["ev_stokeslet_mu"], rtol=1e-12, atol_rel=1e-14)
    assert_close(fl.evaluate(fl.WallStokeslet3D(), X, Y, g["ev_forces_c"], e, mu=0.7), g["ev_wall_fc"], 1e-12, 1e-14)
    assert_close(fl.evaluate(fl.Brinkmanlet3D(3.0), X, Y, g["ev_forces_c"], e, mu=2 - 0.5j), g["ev_brinkman_fc"],
                 1e-12, 1e-14)
    u = fl.evaluate(fl.Stokeslet3D(), X, Y, F, e, mu=2.0 + 0j)
    assert u.dtype == np.complex128


def test_wall_velocity_vanishes(golden):
    g = golden
    u = fl.evaluate(fl.WallStokeslet3D(), g["ev_wall_targets"], g["ev_sources"], g["ev_forces"], g["ev_eps"])
    assert np.abs(u).max() < 1e-14
    u = fl.evaluate(fl.WallStokeslet3D(), g["ev_wall_targets"], g["ev_sources"], g["ev_forces"], g["ev_eps"],
                    precision="mixed")
    assert np.abs(u).max() < 1e-14


@pytest.mark.parametrize("alpha", [0.7 + 0.7j, 2.236 + 2.236j, 0.05 + 0.2j])
@pytest.mark.parametrize("fc", [False, True])
def test_complex_alpha_vs_oracle(alpha, fc):
    rng = np.random.default_rng(5)
    X, Y = rng.normal(size=(37, 3)), rng.normal(size=(53, 3))
    F = rng.normal(size=(53, 3)) + (1j * rng.normal(size=(53, 3)) if fc else 0)
    e = rng.uniform(0.05, 0.3, 53)
    u = fl.evaluate(fl.Brinkmanlet3D(alpha), X, Y, F, e, mu=1.3)
    ref = O.evaluate("brinkman", X, Y, F, e, mu=1.3, alpha=alpha)
    assert u.dtype == np.complex128
    assert_close(u, ref, rtol=1e-12, atol_rel=1e-14)
    um = fl.evaluate(fl.Brinkmanlet3D(alpha), X, Y, F, e, mu=1.3, precision="mixed")
    assert rel_err(um, ref) < 1e-5


SIZES = [(1, 1), (31, 33), (33, 31), (257, 129), (1000, 3001), (4096, 255)]


@pytest.mark.parametrize("kind,alpha", [("stokeslet", 0.0), ("wall", 0.0), ("brinkman", 1.5), ("brinkman", 12.0)])
@pytest.mark.parametrize("M,N", SIZES)
def test_ragged_sizes_fp64_and_mixed(kind, alpha, M, N):
    rng = np.random.default_rng(M * 7919 + N)
    X = np.c_[rng.uniform(-1, 1, (M, 2)), rng.uniform(0.0, 1.5, M)]
    Y = np.c_[rng.uniform(-1, 1, (N, 2)), rng.uniform(0.01, 1.5, N)]
    F = rng.normal(size=(N, 3))
    e = rng.uniform(0.01, 0.08, N)
    ref = O.evaluate(kind, X, Y, F, e, alpha=alpha)
    k = kern(kind, alpha)
    assert_close(fl.evaluate(k, X, Y, F, e), ref, rtol=1e-11, atol_rel=1e-13)
    um = fl.evaluate(k, X, Y, F, e, precision="mixed")
    assert np.linalg.norm(um - ref) / np.linalg.norm(ref) < 2e-6


def test_self_interaction_and_near_pairs_mixed():
    """Targets == sources (the resistance matvec): every target has its own source at r = 0."""
    rng = np.random.default_rng(11)
    from fluidlets_gb300.geometry import fibonacci_sphere
    X = fibonacci_sphere(3000) + [0, 0, 1.2]
    F = rng.normal(size=X.shape)
    e = 0.3 * np.sqrt(4 * np.pi / 3000)
    for kind in ("stokeslet", "wall"):
        ref = O.evaluate(kind, X, X, F, e)
        assert_close(fl.evaluate(kern(kind), X, X, F, e), ref, rtol=1e-11, atol_rel=1e-13)
        um = fl.evaluate(kern(kind), X, X, F, e, precision="mixed")
        assert np.linalg.norm(um - ref) / np.linalg.norm(ref) < 1e-6


def test_empty_inputs():
    X = np.zeros((0, 3))
    Y = np.random.default_rng(0).normal(size=(5, 3))
    assert fl.evaluate(fl.Stokeslet3D(), X, Y, Y, 0.1).shape == (0, 3)
    u = fl.evaluate(fl.Stokeslet3D(), Y, np.zeros((0, 3)), np.zeros((0, 3)), 0.1)
    assert u.shape == (5, 3) and not u.any()


def test_bad_shapes_raise():
    with pytest.raises(ValueError):
        fl.evaluate(fl.Stokeslet3D(), np.zeros((4, 2)), np.zeros((3, 3)), np.zeros((3, 3)), 0.1)
    with pytest.raises(ValueError):
        fl.Brinkmanlet3D(-1.0)
    with pytest.raises(ValueError):
        fl.evaluate(fl.Stokeslet3D(), np.zeros((4, 3)), np.zeros((3, 3)), np.zeros((3, 3)), 0.1, precision="fp16")


def test_deterministic_bitwise():
    rng = np.random.default_rng(2)
    X, Y, F = rng.normal(size=(5000, 3)), rng.normal(size=(7000, 3)), rng.normal(size=(7000, 3))
    Y[:, 2] = np.abs(Y[:, 2]) + 0.01
    for prec in ("fp64", "mixed"):
        a = fl.evaluate(fl.WallStokeslet3D(), X, Y, F, 0.02, precision=prec)
        b = fl.evaluate(fl.WallStokeslet3D(), X, Y, F, 0.02, precision=prec)
        assert np.array_equal(a, b)


def test_torch_tensors_pass_through():
    import torch
    rng = np.random.default_rng(4)
    X, Y, F = rng.normal(size=(100, 3)), rng.normal(size=(80, 3)), rng.normal(size=(80, 3))
    u = fl.evaluate(fl.Stokeslet3D(), torch.tensor(X, device="cuda"), torch.tensor(Y, device="cuda"),
                    torch.tensor(F, device="cuda"), 0.1)
    assert isinstance(u, torch.Tensor) and u.is_cuda
    assert_close(u.cpu().numpy(), O.evaluate("stokeslet", X, Y, F, 0.1), 1e-12, 1e-14)


def test_config2_density_mixed_accuracy_sample():
    """Wall-Stokeslet sum at the benchmark's source density (262,144 sources, eps = 0.01): a
    sample of interior and on-wall targets, mixed precision vs the FP64 oracle."""
    from fluidlets_gb300.geometry import wall_sum_workload
    T, S, F, eps = wall_sum_workload(seed=1)
    idx = np.r_[np.arange(0, 262144, 4096), 262144 + np.arange(0, 16384, 1024)]
    ref = O.evaluate("wall", T[idx], S, F, eps)
    um = fl.evaluate(fl.WallStokeslet3D(), T[idx], S, F, eps, precision="mixed")
    interior = idx < 262144
    assert np.linalg.norm(um[interior] - ref[interior]) / np.linalg.norm(ref[interior]) < 2e-6
    assert np.abs(um[~interior]).max() < 1e-12
    u64 = fl.evaluate(fl.WallStokeslet3D(), T[idx], S, F, eps)
    assert_close(u64, ref, rtol=1e-11, atol_rel=1e-13)


@pytest.mark.parametrize("kind,alpha", [("wall", 0.0), ("stokeslet", 0.0), ("brinkman", 2.0)])
def test_mixed_large_sets_in_cell_order(kind, alpha):
    """Target sets large enough to be processed in cell order (a counting sort by source cell;
    the sources' own order when the targets are the sources), where most far-field tiles run
    without the near-pair mask: mixed vs the FP64 GPU sum, and the order of the given targets
    does not change any result bit."""
    from fluidlets_gb300.geometry import wall_sum_workload
    T, S, F, eps = wall_sum_workload(24000, 40000, 2048, 0.02, seed=5)
    k = kern(kind, alpha)
    um = fl.evaluate(k, T, S, F, eps, precision="mixed")
    u64 = fl.evaluate(k, T, S, F, eps)
    interior = T[:, 2] > 0
    assert rel_err(um[interior], u64[interior]) < 2e-6
    if kind == "wall":
        assert np.abs(um[~interior]).max() == 0.0
    perm = np.random.default_rng(6).permutation(len(T))
    assert np.array_equal(fl.evaluate(k, T[perm], S, F, eps, precision="mixed"), um[perm])
    # targets = sources (40,000): the cell order of the sources themselves
    X = np.r_[S, T[:16000]]
    FX = np.random.default_rng(7).normal(size=X.shape)
    assert rel_err(fl.evaluate(k, X, X, FX, eps, precision="mixed"), fl.evaluate(k, X, X, FX, eps)) < 2e-6


def test_mixed_clustered_sources_keep_the_near_mask():
    """Dense clusters (most tiles near most targets, every tile masked) next to a far cluster
    (tiles unmasked): mixed vs FP64 on the same 40,000 targets."""
    rng = np.random.default_rng(8)
    a = rng.normal(scale=0.02, size=(30000, 3)) + [0, 0, 0.5]
    b = rng.normal(scale=0.02, size=(10000, 3)) + [3.0, 0, 0.5]
    S = np.r_[a, b]
    F = rng.normal(size=S.shape)
    T = np.r_[rng.normal(scale=0.02, size=(20000, 3)) + [0, 0, 0.5], rng.normal(scale=0.5, size=(20000, 3)) + [0, 0, 1.5]]
    for k in (fl.WallStokeslet3D(), fl.Stokeslet3D()):
        um = fl.evaluate(k, T, S, F, 0.004, precision="mixed")
        u64 = fl.evaluate(k, T, S, F, 0.004)
        assert rel_err(um, u64) < 5e-6


# ---- structured grids: the 32^3 legacy grid (tests/legacy/test_phase1_port.py:77-87) ----
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_grid_reproduces_2010_velocity_grid(legacy_towers, legacy_grid, precision):
    t, g = legacy_towers, legacy_grid
    axes, grid = legacy_grid_points(g)
    V = fl.evaluate_grid(fl.WallStokeslet3D(), axes, t["x0"], t["Forces"], float(g["delta"]), precision=precision)
    V[:, 0] += float(g["shear"]) * grid[:, 2]
    stored = g["velocity"].astype(np.float64)
    assert np.linalg.norm(V - stored) / np.linalg.norm(stored) < 1e-6  # float32 CUDA output


def test_grid_equals_evaluate_on_meshgrid(legacy_towers, legacy_grid):
    import torch

    t, g = legacy_towers, legacy_grid
    axes, grid = legacy_grid_points(g)
    W = fl.WallStokeslet3D()
    a = fl.evaluate_grid(W, axes, t["x0"], t["Forces"], 0.5)
    b = fl.evaluate(W, grid, t["x0"], t["Forces"], 0.5)
    assert np.array_equal(a, b)
    f = fl.evaluate_grid(W, axes, t["x0"], t["Forces"], 0.5, field=True)
    assert f.shape == (32, 32, 32, 3) and np.array_equal(f.reshape(-1, 3), a)
    # ragged axes, torch in -> torch out
    ax = (np.linspace(0, 1, 5), np.linspace(-1, 1, 3), np.array([0.5]))
    src = torch.tensor(t["x0"][:50], device="cuda")
    u = fl.evaluate_grid(W, ax, src, torch.tensor(t["Forces"][:50], device="cuda"), 0.5, field=True)
    assert isinstance(u, torch.Tensor) and tuple(u.shape) == (1, 3, 5, 3)
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    ref = O.evaluate("wall", np.c_[X.ravel(), Y.ravel(), Z.ravel()], t["x0"][:50], t["Forces"][:50], 0.5)
    assert_close(u.reshape(-1, 3).cpu().numpy(), ref, 1e-12)


# ---- nearest-neighbour map (core/assemble.py:61-65) --------------------------------
def test_nearest_neighbors_match_kdtree():
    from scipy.spatial import cKDTree

    from fluidlets_gb300.geometry import biflagellate_shape

    rng = np.random.default_rng(7)
    for Q, N in [(1, 1), (5000, 700), (3001, 2500)]:
        quad, force = rng.normal(size=(Q, 3)), rng.normal(size=(N, 3))
        got = fl.nearest_neighbors(quad, force)
        assert got.dtype == np.int64 and got.shape == (Q,)
        assert np.array_equal(got, cKDTree(force).query(quad)[1])
    s = biflagellate_shape(0.3)
    assert np.array_equal(fl.nearest_neighbors(s.X, s.x), cKDTree(s.x).query(s.X)[1])
    assert fl.nearest_neighbors(np.zeros((0, 3)), force).shape == (0,)
    with pytest.raises(ValueError):
        fl.nearest_neighbors(quad, np.zeros((0, 3)))


# ---- geometry on the device (geometry/spheres.py) --------------------------------------------
def test_device_spheres_match_reference_formulas():
    from fluidlets_gb300 import geometry as G

    for n in (1, 3, 12, 40):
        d = G.cube_sphere_device(n, 0.7, (0.1, -2.0, 3.0)).cpu().numpy()
        assert np.array_equal(d, O.cube_sphere(n, 0.7, (0.1, -2.0, 3.0)))  # sqrt and division: exact
        assert np.array_equal(G.cube_sphere(n, 0.7, (0.1, -2.0, 3.0)), d)
    for n in (1, 2, 1536, 65536):
        d = G.fibonacci_sphere_device(n, 2.0, (1.0, 0.0, -1.0)).cpu().numpy()
        h = O.fibonacci_sphere(n, 2.0, (1.0, 0.0, -1.0))
        assert np.abs(d - h).max() <= 8 * np.finfo(float).eps  # CUDA's acos/sin/cos vs the C library's
    rng = np.random.default_rng(5)
    for P in (O.fibonacci_sphere(2000), rng.uniform(-1, 1, (3001, 3)), O.cube_sphere(12)):
        assert abs(G.mean_nn_spacing(P) - O.mean_nn_spacing(P)) <= 1e-13 * O.mean_nn_spacing(P)
