"""Failure detection without a GPU fault: every spin-wait of the library's kernels is bounded.

flg_wait_selftest makes one kind of wait impossible to satisfy -- the FP64 LU panel's grid
barrier with an arrival that never comes, the low-precision solve's poll of a value nothing
publishes, the tensor-core update's mbarrier wait on a phase no arrival completes -- with a
200 ms limit.  Each must end by itself, report FLG_ERR_TIMEOUT (RuntimeError in Python, the
exception type the reference raises for a failed solve, core/solve.py:77-78) and leave the
context usable: a solve right after it still matches the oracle.
"""
import time

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
fl = pytest.importorskip("fluidlets_gb300")
from fluidlets_gb300 import _device as dv  # noqa: E402
from fluidlets_gb300 import _lib  # noqa: E402


@pytest.mark.parametrize("which", [0, 1, 2], ids=["grid_barrier", "published_value", "mbarrier"])
def test_bounded_wait_runs_out_and_reports(which):
    L = _lib.load()
    nb = L.flg_wait_selftest_workspace()
    ws = dv.workspace(nb)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = L.flg_wait_selftest(which, 200.0, dv.ptr(ws), nb, dv.stream())
    dt = time.perf_counter() - t0
    assert st == _lib.FLG_ERR_TIMEOUT, (st, L.flg_last_error())
    assert b"timed out" in L.flg_last_error()
    assert 0.19 <= dt < 5.0, dt
    with pytest.raises(RuntimeError, match="timed out"):
        _lib.check(st, "self-test")
    # the context is still usable
    X = O.fibonacci_sphere(150)
    U = np.tile([1.0, 0.0, 0.0], (150, 1))
    f, _ = fl.resistance(fl.Stokeslet3D(), X, U, 0.1, method="lu", precision="mixed")
    fo, _ = O.resistance("stokeslet", X, U, 0.1, method="lu")
    assert np.abs(f - fo).max() <= 1e-9 * np.abs(fo).max()


def test_wait_selftest_rejects_bad_arguments():
    L = _lib.load()
    ws = dv.workspace(L.flg_wait_selftest_workspace())
    assert L.flg_wait_selftest(3, 100.0, dv.ptr(ws), ws.numel(), dv.stream()) == _lib.FLG_ERR_INVALID
    assert L.flg_wait_selftest(0, 0.0, dv.ptr(ws), ws.numel(), dv.stream()) == _lib.FLG_ERR_INVALID
    assert L.flg_wait_selftest(0, 100.0, dv.ptr(ws), 8, dv.stream()) == _lib.FLG_ERR_INVALID
