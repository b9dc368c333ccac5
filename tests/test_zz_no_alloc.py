"""flg_evaluate_noalloc: the FP64 kernel sum for callers that cannot allocate.

Callers such as a host application that has reserved all device memory for its
own pool, or a plug-in whose framework forbids cudaMalloc after start-up, can
neither allocate nor hand over a workspace; this entry point keeps its scratch
in a fixed 16 MiB device array inside the library.  The test calls it through
the C ABI, twice in a row on different inputs (the array keeps the previous
call's contents), and compares each result with flg_evaluate's FP64 result.
This file sorts last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
from fluidlets_gb300 import _device as dv  # noqa: E402
from fluidlets_gb300 import _lib  # noqa: E402


def _evaluate(L, kind, alpha, X, Y, F, e, mu, noalloc):
    M, N = X.shape[0], Y.shape[0]
    fc = F.is_complex()
    out_c = fc or alpha.imag != 0 or mu.imag != 0
    out = torch.full((M, 3), float("nan"), dtype=torch.complex128 if out_c else torch.float64, device="cuda")
    if noalloc:
        st = L.flg_evaluate_noalloc(kind, alpha.real, alpha.imag, dv.ptr(X), M, dv.ptr(Y), dv.ptr(e), N, dv.ptr(F),
                                    int(fc), mu.real, mu.imag, dv.ptr(out), dv.stream())
    else:
        nb = L.flg_evaluate_workspace(kind, M, N, int(fc), alpha.imag, 0)
        ws = dv.workspace(nb)
        st = L.flg_evaluate(kind, alpha.real, alpha.imag, dv.ptr(X), M, dv.ptr(Y), dv.ptr(e), N, dv.ptr(F), int(fc),
                            mu.real, mu.imag, dv.ptr(out), 0, dv.ptr(ws), nb, dv.stream())
    _lib.check(st)
    torch.cuda.synchronize()
    return out.cpu().numpy()


# (kind, alpha, complex strengths, mu, M, N).  The last two cases hold enough targets that the
# default number of source splits would overflow the fixed array (6 splits x 2.88 MB > 16 MiB), so
# the call runs fewer, longer splits: real output (24 B per target) and complex (48 B).
CASES = [(1, 0j, False, 1 + 0j, 2000, 3001), (2, 1.5 + 1.5j, True, 0.8 - 0.2j, 777, 1234),
         (1, 0j, False, 1 + 0j, 120000, 4000), (0, 0j, True, 1 + 0j, 60000, 3000)]


@pytest.mark.parametrize("case", CASES)
def test_noalloc_matches_evaluate_on_two_calls_in_a_row(case):
    kind, alpha, fcomplex, mu, M, N = case
    L = _lib.load()
    assert L.flg_evaluate_noalloc_max_bytes() == 16 << 20
    for call in range(2):
        rng = np.random.default_rng(100 * kind + call)
        X = torch.tensor(np.c_[rng.uniform(-1, 1, (M, 2)), rng.uniform(0, 1.5, M)], device="cuda")
        Y = torch.tensor(np.c_[rng.uniform(-1, 1, (N, 2)), rng.uniform(0.01, 1.5, N)], device="cuda")
        F = rng.normal(size=(N, 3)) + (1j * rng.normal(size=(N, 3)) if fcomplex else 0)
        F = torch.tensor(F, device="cuda")
        e = torch.tensor(rng.uniform(0.02, 0.1, N), device="cuda")
        ref = _evaluate(L, kind, alpha, X, Y, F, e, mu, noalloc=False)
        got = _evaluate(L, kind, alpha, X, Y, F, e, mu, noalloc=True)
        assert np.isfinite(got).all()
        scale = np.abs(ref).max()
        assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(ref) + 1e-14 * scale)


def test_noalloc_rejects_too_many_targets():
    L = _lib.load()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    M = (16 << 20) // 24 + 1  # one target more than the fixed array holds (real output)
    st = L.flg_evaluate_noalloc(0, 0.0, 0.0, dv.ptr(buf), M, dv.ptr(buf), dv.ptr(buf), 1, dv.ptr(buf), 0, 1.0, 0.0,
                                dv.ptr(buf), dv.stream())
    assert st == _lib.FLG_ERR_INVALID
    assert b"scratch" in L.flg_last_error()
