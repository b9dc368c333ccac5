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
