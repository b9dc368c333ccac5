"""The C-ABI library builds, loads without a GPU and exports every declared entry point."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "fluidlets_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(flg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from fluidlets_gb300 import build
    build.build()
    from fluidlets_gb300 import _lib
    return _lib


def test_header_and_binding_agree(lib):
    assert declared_functions() == sorted(lib.exported_symbols())


def test_library_exports_every_declared_symbol(lib):
    assert lib.missing_symbols() == []
    assert lib.load().flg_version() == 10000


def test_invalid_arguments_rejected_on_host(lib):
    L = lib.load()
    # unknown kernel kind -> FLG_ERR_INVALID before any CUDA call
    st = L.flg_evaluate(7, 0.0, 0.0, None, 1, None, None, 1, None, 0, 1.0, 0.0, None, 0, None, 0, None)
    assert st == lib.FLG_ERR_INVALID
    assert b"kind" in L.flg_last_error()
    st = L.flg_evaluate(2, -1.0, 0.0, None, 1, None, None, 1, None, 0, 1.0, 0.0, None, 0, None, 0, None)
    assert st == lib.FLG_ERR_INVALID


def header_constants():
    text = (ROOT / "include" / "fluidlets_gb300.h").read_text()
    return {k: int(v, 0) for k, v in re.findall(r"#define\s+(FLG_[A-Z0-9_]+)\s+(0x[0-9A-Fa-f]+|\d+)\b", text)}


def test_lu_mode_names_match_the_header(lib):
    """The Python LU mode names (precision, and the tile width of the tensor-core updates) encode
    the header's mode constants; every name the serving autotuner tries is a valid mode."""
    c = header_constants()
    assert lib.LU_MODE["tf32"] == c["FLG_LU_TF32"] and lib.LU_MODE["bf16"] == c["FLG_LU_BF16"]
    assert lib.LU_MODE["fp32"] == c["FLG_LU_FP32"]
    for prec in ("tf32", "bf16"):
        assert lib.LU_MODE[f"{prec}:128"] == c[f"FLG_LU_{prec.upper()}"] | c["FLG_LU_TILE_N128"]
        assert lib.LU_MODE[f"{prec}:256"] == c[f"FLG_LU_{prec.upper()}"] | c["FLG_LU_TILE_N256"]
    from fluidlets_gb300.serve import TUNE_CANDIDATES
    assert set(TUNE_CANDIDATES) <= set(lib.LU_MODE) and len(set(TUNE_CANDIDATES)) == 7


def test_lu_workspace_does_not_depend_on_the_tile_width(lib):
    L = lib.load()
    for n in (128, 1000, 4608):
        for prec in ("tf32", "bf16"):
            base = L.flg_lu_factor_lowp_workspace(n, lib.LU_MODE[prec])
            assert base > 0
            assert L.flg_lu_factor_lowp_workspace(n, lib.LU_MODE[prec + ":128"]) == base
            assert L.flg_lu_factor_lowp_workspace(n, lib.LU_MODE[prec + ":256"]) == base


def test_batched_lu_workspace_scales_with_the_batch(lib):
    """The batched LU's scratch is the single system's per system (the BF16 copies of the
    panels included), across both outer-panel widths (512 columns below n = 8,192, 1,024 from
    there); the batched swimmer graph's workspace covers its LU's."""
    L = lib.load()
    for n in (768, 4608, 8192, 12288):
        for prec in ("tf32", "bf16"):
            one = L.flg_lu_factor_lowp_batched_workspace(n, 1, lib.LU_MODE[prec])
            assert one + 256 == L.flg_lu_factor_lowp_workspace(n, lib.LU_MODE[prec])
            for k in (2, 4):
                wk = L.flg_lu_factor_lowp_batched_workspace(n, k, lib.LU_MODE[prec])
                assert k * one - 4096 <= wk <= k * one + 4096, (n, prec, k)
    # 1,024-column outer panels double the K-major copy of U from n = 8,192 on
    assert L.flg_lu_factor_lowp_batched_workspace(8192, 1, 0) > 1.4 * L.flg_lu_factor_lowp_batched_workspace(8064, 1, 0)
    for k in (1, 3):
        assert L.flg_swimmer_batch_graph_workspace(224, 896, k, 0) >= L.flg_lu_factor_lowp_batched_workspace(678, k, 0)


def test_unknown_lu_name_is_a_value_error(lib):
    assert lib.lu_mode("bf16:128") == lib.LU_MODE["bf16:128"]
    for bad in ("tf16", "fp32:128", "tf32:64", None):
        with pytest.raises(ValueError):
            lib.lu_mode(bad)


def test_uniform_blob_width_detection():
    """The symmetric self-assembly is chosen only for one blob width: a scalar, a one-element
    tensor, or a host array of equal entries (device arrays are not inspected)."""
    import numpy as np
    import torch

    from fluidlets_gb300.core import _uniform_eps
    assert _uniform_eps(0.25) == 0.25 and _uniform_eps(np.float64(0.5)) == 0.5
    assert _uniform_eps(np.full(7, 0.1)) == 0.1 and _uniform_eps([0.2, 0.2]) == 0.2
    assert _uniform_eps(np.array([0.1, 0.2])) is None
    assert _uniform_eps(torch.tensor(0.3, dtype=torch.float64)) == 0.3
    assert _uniform_eps(torch.full((5,), 0.3, dtype=torch.float64)) is None
