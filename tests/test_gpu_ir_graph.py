"""GMRES-IR as one CUDA graph (flg_gmres_ir_graph_*): the refinement and inner loops run as
conditional graph nodes steered on the device.  Its solutions equal the host-driven refinement's
(flg_gmres_ir_dense) and the FP64 LU's; a replay with a new right-hand side in the same buffer
solves the new system; a tolerance it cannot reach ends with FLG_ERR_NOT_CONVERGED, as the
reference's solver reports non-convergence (core/solve.py:77-78)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
fl = pytest.importorskip("fluidlets_gb300")
from fluidlets_gb300 import _lib  # noqa: E402
from fluidlets_gb300.core import IrGraph, _assemble_dev, _gmres_ir_dense_dev, _lowp_factor_dev, _lu_solve_dev  # noqa: E402


def system(N, kernel, h=0.0, seed=0):
    X = torch.tensor(O.fibonacci_sphere(N) + [0.0, 0.0, h], device="cuda")
    e = torch.full((N,), 0.25 * O.mean_nn_spacing(X.cpu().numpy()), dtype=torch.float64, device="cuda")
    K = _assemble_dev(kernel, X, X, e, 1.0)
    g = torch.Generator(device="cuda").manual_seed(seed)
    return K, g


@pytest.mark.parametrize("N,kind,lu", [(400, "stokeslet", "tf32"), (1536, "wall", "bf16"), (700, "wall", "fp32")])
def test_graph_refinement_matches_host_refinement_and_lu(N, kind, lu):
    kernel = fl.Stokeslet3D() if kind == "stokeslet" else fl.WallStokeslet3D()
    K, gen = system(N, kernel, h=0.0 if kind == "stokeslet" else 1.3)
    n = K.shape[0]
    K32, ld32, dinv, A32 = _lowp_factor_dev(K, lu)
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        ir = IrGraph(K, A32, K32, ld32, dinv, b, x, 1e-12)
        for call in range(2):  # two right-hand sides through the same buffers
            rhs = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
            b.copy_(rhs)
            ir.launch(st)
            status, iters, outer, resid = ir.result(st)
            assert status == _lib.FLG_OK and resid < 1e-12 and outer >= 1, (status, resid, outer)
            xh, ih, oh, rh = _gmres_ir_dense_dev(K, K32, ld32, dinv, rhs, 1e-12, 30, 200, A32=A32)
            ref = _lu_solve_dev(K.clone(), rhs)
            assert float(torch.linalg.vector_norm(x - ref) / torch.linalg.vector_norm(ref)) < 1e-10
            assert float(torch.linalg.vector_norm(x - xh) / torch.linalg.vector_norm(xh)) < 1e-10
            assert abs(outer - oh) <= 1
        ir.close()


def test_graph_refinement_reports_non_convergence():
    K, gen = system(300, fl.Stokeslet3D())
    n = K.shape[0]
    K32, ld32, dinv, A32 = _lowp_factor_dev(K, "bf16")
    b = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
    x = torch.empty_like(b)
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        ir = IrGraph(K, A32, K32, ld32, dinv, b, x, 1e-30, max_outer=3)
        ir.launch(st)
        status, iters, outer, resid = ir.result(st)
    assert status == _lib.FLG_ERR_NOT_CONVERGED and outer <= 3 and resid < 1e-10
