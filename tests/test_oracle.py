"""The CPU oracle against the reference's own golden data (no GPU).

Pins oracle/ before it is trusted as the checker of the CUDA path:
* legacy MATLAB vectors, tests/legacy/test_phase1_port.py:33-59;
* outputs of the reference package itself (tests/golden/make_golden.py);
* complex-alpha Brinkmanlet functions against mpmath (no reference exists).
"""
import numpy as np
import pytest

import oracle as O
from conftest import assert_close, legacy_grid_points, rel_err


def test_stokeslet_matches_legacy_StokesletEval(legacy_kernels):
    d = legacy_kernels
    u = O.evaluate("stokeslet", d["targets"], d["sources"], d["strengths"], d["deltas"])
    assert np.allclose(u, d["V_stokeslet"], rtol=1e-13, atol=1e-15)


def test_wall_matches_legacy_StokesletEval_plus_ImageEval(legacy_kernels):
    d = legacy_kernels
    u = O.evaluate("wall", d["targets"], d["sources"], d["strengths"], d["deltas"])
    assert np.allclose(u, d["V_stokeslet"] + d["V_image"], rtol=1e-13, atol=1e-15)
    u = O.evaluate("wall", d["wall"], d["sources"], d["strengths"], d["deltas"])
    assert np.allclose(u, d["V_wall_total"], atol=1e-15)


def test_tower_operator_residual_equals_legacy(legacy_towers):
    # tests/legacy/test_phase1_port.py:54-59: same operator as StokesSelf.m to roundoff
    d = legacy_towers
    r = np.linalg.norm(O.evaluate("wall", d["x0"], d["x0"], d["Forces"], 0.5) - d["Vel"]) / np.linalg.norm(d["Vel"])
    assert abs(r - float(d["resid"])) < 1e-12


def test_oracle_reproduces_2010_velocity_grid(legacy_towers, legacy_grid):
    # tests/legacy/test_phase1_port.py:77-87 on every 16th point of the 32^3 grid (the full grid
    # runs on the GPU): tower forces from the legacy GMRES, plus the background shear 0.1 z
    t, g = legacy_towers, legacy_grid
    _, grid = legacy_grid_points(g)
    sel = np.arange(0, len(grid), 16)
    V = O.evaluate("wall", grid[sel], t["x0"], t["Forces"], float(g["delta"]))
    V[:, 0] += float(g["shear"]) * grid[sel, 2]
    stored = g["velocity"][sel].astype(np.float64)
    assert np.linalg.norm(V - stored) / np.linalg.norm(stored) < 1e-6  # float32 CUDA output


@pytest.mark.parametrize("name,kind,alpha", [("stokeslet", "stokeslet", 0.0), ("wall", "wall", 0.0),
                                             ("brinkman_0", "brinkman", 0.0), ("brinkman_0.5", "brinkman", 0.5),
                                             ("brinkman_3", "brinkman", 3.0), ("brinkman_20", "brinkman", 20.0)])
def test_evaluate_matches_reference(golden, name, kind, alpha):
    g = golden
    u = O.evaluate(kind, g["ev_targets"], g["ev_sources"], g["ev_forces"], g["ev_eps"], alpha=alpha)
    assert rel_err(u, g[f"ev_{name}"]) < 1e-15


def test_complex_cases_match_reference(golden):
    g = golden
    X, Y, F, e = g["ev_targets"], g["ev_sources"], g["ev_forces"], g["ev_eps"]
    assert rel_err(O.evaluate("stokeslet", X, Y, F, e, mu=2 - 0.5j), g["ev_stokeslet_mu"]) < 1e-15
    assert rel_err(O.evaluate("wall", X, Y, g["ev_forces_c"], e, mu=0.7), g["ev_wall_fc"]) < 1e-15
    assert rel_err(O.evaluate("brinkman", X, Y, g["ev_forces_c"], e, mu=2 - 0.5j, alpha=3.0),
                   g["ev_brinkman_fc"]) < 1e-15
    assert np.abs(O.evaluate("wall", g["ev_wall_targets"], Y, F, e)).max() < 1e-15


def test_assemble_matches_reference(golden):
    g = golden
    Y, X = g["as_points"], g["ev_targets"]
    assert rel_err(O.assemble("stokeslet", Y, Y, 0.2), g["as_stokeslet"]) == 0.0
    assert rel_err(O.assemble("wall", Y, Y, g["ev_eps"][:19]), g["as_wall"]) == 0.0
    assert rel_err(O.assemble("brinkman", Y, Y, 0.2, alpha=3.0), g["as_brinkman"]) < 1e-15
    assert rel_err(O.assemble("wall", Y, Y, 0.2, mu=2 - 0.5j), g["as_wall_mu"]) == 0.0
    assert rel_err(O.assemble("wall", X, Y, 0.15), g["as_rect"]) == 0.0


def test_assemble_nearest_matches_reference(golden):
    g = golden
    xc, Xq, nn = g["an_coarse"], g["an_quad"], g["an_nearest"]
    assert np.array_equal(O.nearest_neighbors(Xq, xc), nn)
    assert rel_err(O.assemble_nearest("stokeslet", xc, Xq, nn, len(xc), 0.05), g["an_stokeslet"]) == 0.0
    sh = np.array([0, 0, 1.5])
    assert rel_err(O.assemble_nearest("wall", xc + sh, Xq + sh, nn, len(xc), 0.05), g["an_wall"]) == 0.0


def test_resistance_matches_reference(golden):
    g = golden
    S, e, U = g["rs_points"], float(g["rs_eps"]), g["rs_U"]
    f, info = O.resistance("stokeslet", S, U, e, method="lu")
    assert rel_err(f, g["rs_lu_forces"]) < 1e-14 and info.residual < 1e-12
    f, info = O.resistance("stokeslet", S, U, e, method="gmres")
    assert rel_err(f, g["rs_gmres_forces"]) < 1e-12 and info.iterations == int(g["rs_gmres_iters"])


def test_swimming_problem_matches_reference(golden):
    g = golden
    U, Om, F, *_ = O.swimming_problem(g["sw_x"], g["sw_v"], g["sw_X"], g["sw_x0"], g["sw_B"], 0.05)
    assert rel_err(U, g["sw_U"]) < 1e-13 and rel_err(Om, g["sw_Omega"]) < 1e-13
    assert rel_err(F, g["sw_forces"]) < 1e-13


def test_brinkman_series_matches_reference(golden):
    g = golden
    for z, a, b in zip(g["bf_z"], g["bf_f1"], g["bf_f2"]):
        f1, f2 = O.brink_f(z)
        assert f1.imag == 0 and abs(f1.real - a) <= 2e-16 * abs(a) and abs(f2.real - b) <= 2e-16 * abs(b)


@pytest.mark.parametrize("z", [0.01 + 0.01j, 0.3 - 0.2j, 0.35 + 0.35j, 0.36 + 0.36j, 1 + 1j, 2.2 + 2.2j, 3.16 + 3.16j,
                               0.1 + 4j])
def test_complex_alpha_functions_match_mpmath(z):
    """Complex-alpha extension: f1, f2 at complex z vs 50-digit mpmath closed forms."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50
    Z = mp.mpc(z.real, z.imag)
    E = mp.exp(-Z)
    e1 = E * (1 + 1 / Z + 1 / Z**2) - 1 / Z**2
    e2 = 3 / Z**2 - E * (1 + 3 / Z + 3 / Z**2)
    f1, f2 = O.brink_f(z)
    assert abs(f1 - complex(e1)) <= 1e-13 * abs(complex(e1))
    assert abs(f2 - complex(e2)) <= 1e-13 * abs(complex(e2))


def test_complex_alpha_tends_to_real_alpha_and_stokeslet():
    rng = np.random.default_rng(3)
    X, Y, F = rng.normal(size=(7, 3)), rng.normal(size=(9, 3)), rng.normal(size=(9, 3))
    u_r = O.evaluate("brinkman", X, Y, F, 0.1, alpha=2.0)
    u_c = O.evaluate("brinkman", X, Y, F, 0.1, alpha=2.0 + 1e-12j)
    assert rel_err(u_c, u_r) < 1e-10
    u_s = O.evaluate("stokeslet", X, Y, F, 0.1)
    u_0 = O.evaluate("brinkman", X, Y, F, 0.1, alpha=1e-14 + 1e-14j)
    assert rel_err(u_0, u_s) < 1e-12


def test_oracle_detects_a_planted_error(golden):
    """A wrong kernel (image sign flipped) must fail the same comparison."""
    g = golden
    good = O.evaluate("wall", g["ev_targets"], g["ev_sources"], g["ev_forces"], g["ev_eps"])
    free = O.evaluate("stokeslet", g["ev_targets"], g["ev_sources"], g["ev_forces"], g["ev_eps"])
    planted = 2 * free - good  # free - image instead of free + image
    assert rel_err(planted, g["ev_wall"]) > 1e-2 and rel_err(good, g["ev_wall"]) < 1e-15
