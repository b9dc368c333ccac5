"""ctypes binding of libfluidlets_gb300.so (declared in include/fluidlets_gb300.h).

There is no CPU fallback: if the library has not been built, or no CUDA
device is present, every compute call raises.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_size_t, c_void_p

import numpy as np

from .build import lib_path

FLG_OK, FLG_ERR_INVALID, FLG_ERR_CUDA, FLG_ERR_NOT_CONVERGED, FLG_ERR_SINGULAR, FLG_ERR_NOMEM, FLG_ERR_TIMEOUT = range(7)
KIND = {"stokeslet": 0, "wall": 1, "brinkman": 2}
PREC = {"fp64": 0, "mixed": 1}
F64, C128, F32, BF16 = 0, 1, 2, 3
LU_MODE = {"tf32": 0, "bf16": 1, "fp32": 2}
# tensor-core modes with a forced tile width of the trailing updates ("tf32:128": 128 x 128 tiles)
LU_TILE = {128: 0x100, 256: 0x200}
LU_MODE.update({f"{p}:{t}": LU_MODE[p] | b for p in ("tf32", "bf16") for t, b in LU_TILE.items()})


def lu_mode(name: str) -> int:
    """Mode constant of a low-precision LU name ("tf32", "bf16", "fp32", "tf32:128", ...)."""
    try:
        return LU_MODE[name]
    except (KeyError, TypeError):
        raise ValueError(f"unknown lu {name!r}: expected one of {', '.join(LU_MODE)}") from None

# name -> (restype, argtypes); mirrors include/fluidlets_gb300.h
_P = c_void_p
SIGNATURES = {
    "flg_version": (c_int, []),
    "flg_last_error": (ctypes.c_char_p, []),
    "flg_evaluate_workspace": (c_size_t, [c_int, c_int64, c_int64, c_int, c_double, c_int]),
    "flg_evaluate": (c_int, [c_int, c_double, c_double, _P, c_int64, _P, _P, c_int64, _P, c_int, c_double,
                             c_double, _P, c_int, _P, c_size_t, _P]),
    "flg_evaluate_noalloc_max_bytes": (c_size_t, []),
    "flg_evaluate_noalloc": (c_int, [c_int, c_double, c_double, _P, c_int64, _P, _P, c_int64, _P, c_int, c_double,
                                     c_double, _P, _P]),
    "flg_assemble": (c_int, [c_int, c_double, c_double, _P, c_int64, _P, _P, c_int64, c_double, c_double, _P,
                             c_int, c_int64, _P]),
    "flg_assemble_self_uniform": (c_int, [c_int, c_double, c_double, _P, c_int64, c_double, c_double, c_double, _P,
                                          c_int, c_int64, _P]),
    "flg_assemble_bucket": (c_int, [c_int, c_double, c_double, _P, _P, _P, c_int64, c_double, _P, c_int, c_int64,
                                    _P]),
    "flg_assemble_bucket_uniform": (c_int, [c_int, c_double, c_double, _P, _P, _P, c_int64, c_double, _P, c_int,
                                            c_int64, _P]),
    "flg_assemble_bucket_batched": (c_int, [c_int, c_double, c_double, _P, _P, c_int, _P, c_int64, c_int, c_double,
                                            _P, c_int, c_int64, c_int64, _P]),
    "flg_assemble_nearest_workspace": (c_size_t, [c_int64, c_int64]),
    "flg_assemble_nearest": (c_int, [c_int, c_double, c_double, _P, c_int64, _P, _P, _P, c_int64, c_int64,
                                     c_double, c_double, _P, c_int, c_int64, _P, c_size_t, _P]),
    "flg_swimmer_constraints": (c_int, [_P, c_int64, POINTER(c_double), _P, _P, c_int64, _P, c_int, c_int64,
                                        _P]),
    "flg_lu_factor_f64_workspace": (c_size_t, [c_int64]),
    "flg_lu_factor_f64": (c_int, [c_int64, _P, c_int64, _P, POINTER(c_int), _P, c_size_t, _P]),
    "flg_lu_solve_f64": (c_int, [c_int64, c_int64, _P, c_int64, _P, _P, c_int64, _P]),
    "flg_lu_lowp_dinv_elems": (c_int64, [c_int64]),
    "flg_lu_factor_lowp_workspace": (c_size_t, [c_int64, c_int]),
    "flg_lu_factor_lowp": (c_int, [c_int64, _P, c_int64, c_int, _P, POINTER(c_int), _P, c_size_t, _P]),
    "flg_lu_factor_lowp_async": (c_int, [c_int64, _P, c_int64, c_int, _P, _P, _P, c_size_t, _P]),
    "flg_lu_factor_lowp_batched_workspace": (c_size_t, [c_int64, c_int, c_int]),
    "flg_lu_factor_lowp_batched_async": (c_int, [c_int64, c_int, _P, c_int64, c_int64, c_int, _P, _P, _P, c_size_t,
                                                 _P]),
    "flg_lu_solve_lowp_workspace": (c_size_t, [c_int64]),
    "flg_lu_solve_lowp": (c_int, [c_int64, _P, c_int64, _P, _P, _P, _P, c_size_t, _P]),
    "flg_tc_rank_update_workspace": (c_size_t, [c_int64, c_int64, c_int]),
    "flg_tc_rank_update": (c_int, [_P, c_int64, _P, c_int64, _P, c_int64, c_int64, c_int64, c_int, _P, c_size_t,
                                   _P]),
    "flg_gmres_workspace": (c_size_t, [c_int64, c_int, c_int, c_int]),
    "flg_gmres": (c_int, [c_int, c_double, c_double, _P, _P, c_int64, c_double, c_double, _P, _P, c_int,
                          c_double, c_int, c_int, c_int, c_double, POINTER(c_int), POINTER(c_int),
                          POINTER(c_double), _P, c_size_t, _P]),
    "flg_gmres_ir_dense_workspace": (c_size_t, [c_int64, c_int]),
    "flg_gmres_ir_dense": (c_int, [c_int64, _P, c_int64, _P, c_int64, _P, c_int64, _P, _P, _P, c_double, c_int, c_int,
                                   POINTER(c_int), POINTER(c_int), POINTER(c_double), _P, c_size_t, _P]),
    "flg_bucket_graph_create": (c_int, [c_int, c_double, c_double, _P, _P, c_int, _P, c_int64, c_double, _P, _P, _P,
                                        c_int64, c_int, _P, _P, _P, c_size_t, _P, POINTER(c_void_p)]),
    "flg_bucket_batch_graph_create": (c_int, [c_int, c_double, c_double, _P, _P, c_int, _P, c_int64, c_int, c_double,
                                              _P, _P, _P, c_int64, c_int, _P, _P, _P, c_size_t, _P,
                                              POINTER(c_void_p)]),
    "flg_gmres_ir_graph_workspace": (c_size_t, [c_int64, c_int]),
    "flg_gmres_ir_graph_create": (c_int, [c_int64, _P, c_int64, _P, c_int64, _P, c_int64, _P, _P, _P, c_double, c_int,
                                          c_int, _P, c_size_t, _P, POINTER(c_void_p)]),
    "flg_gmres_ir_graph_result": (c_int, [_P, POINTER(c_int), POINTER(c_int), POINTER(c_double), _P]),
    "flg_lowp_factor_graph_create": (c_int, [c_int64, _P, c_int64, _P, _P, c_int64, c_int, _P, _P, _P, c_size_t, _P,
                                             POINTER(c_void_p)]),
    "flg_graph_launch": (c_int, [_P, _P]),
    "flg_graph_destroy": (c_int, [_P]),
    "flg_assemble_nearest_async": (c_int, [c_int, c_double, c_double, _P, c_int64, _P, _P, _P, c_int64, c_int64,
                                           c_double, c_double, _P, c_int, c_int64, _P, _P, c_size_t, _P]),
    "flg_swimmer_constraints_dev": (c_int, [_P, c_int64, _P, _P, _P, c_int64, _P, c_int, c_int64, _P]),
    "flg_swimmer_graph_workspace": (c_size_t, [c_int64, c_int64, c_int]),
    "flg_swimmer_batch_graph_workspace": (c_size_t, [c_int64, c_int64, c_int, c_int]),
    "flg_swimmer_batch_graph_create": (c_int, [c_int, c_double, c_double, _P, c_int64, _P, _P, _P, c_int64, _P, c_int,
                                               c_int, c_double, _P, _P, _P, c_int64, c_int, _P, _P, _P, c_size_t, _P,
                                               POINTER(c_void_p)]),
    "flg_swimmer_graph_create": (c_int, [c_int, c_double, c_double, _P, c_int64, _P, _P, _P, c_int64, _P, c_int,
                                         c_double, _P, _P, _P, c_int64, c_int, _P, _P, _P, c_size_t, _P,
                                         POINTER(c_void_p)]),
    "flg_grid_points": (c_int, [_P, c_int64, _P, c_int64, _P, c_int64, _P, _P]),
    "flg_fibonacci_sphere": (c_int, [c_int64, c_double, POINTER(c_double), _P, _P]),
    "flg_cube_sphere": (c_int, [c_int64, c_double, POINTER(c_double), _P, _P]),
    "flg_mean_nn_spacing_workspace": (c_size_t, [c_int64]),
    "flg_mean_nn_spacing": (c_int, [_P, c_int64, _P, _P, c_size_t, _P]),
    "flg_nearest_neighbors": (c_int, [_P, c_int64, _P, c_int64, _P, _P]),
    "flg_gemv_f64": (c_int, [c_int64, c_int64, _P, c_int64, _P, _P, _P]),
    "flg_gemv_f32": (c_int, [c_int64, c_int64, _P, c_int64, _P, _P, _P]),
    "flg_convert_f64_f32": (c_int, [c_int64, c_int64, _P, c_int64, _P, c_int64, _P]),
    "flg_convert_f64_f32x2": (c_int, [c_int64, c_int64, _P, c_int64, _P, _P, c_int64, _P]),
    "flg_measure_peaks": (c_int, [POINTER(c_double), POINTER(c_double), _P]),
    "flg_profile_enable": (c_int, [c_int]),
    "flg_profile_read": (c_int, [c_int, POINTER(c_double), POINTER(c_int64)]),
    "flg_launch_count": (c_int64, []),
    "flg_wait_selftest_workspace": (c_size_t, []),
    "flg_wait_selftest": (c_int, [c_int, c_double, _P, c_size_t, _P]),
}
SLOT = {"far_f32": 0, "near_f64": 1, "sum_f64": 2, "assemble": 3, "lu_update": 4, "lu_panel": 5, "gemv": 6, "lu_solve": 7, "lu_diag": 8}

_lib = None


class LinAlgError(np.linalg.LinAlgError):
    pass


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not path.exists():
            raise RuntimeError(f"{path} is missing: build it with `python -m fluidlets_gb300.build` "
                               "(fluidlets_gb300 has no CPU fallback)")
        L = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue  # reported by missing_symbols(); calling it raises AttributeError
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(SIGNATURES)


def missing_symbols():
    L = load()
    return [n for n in SIGNATURES if getattr(L, n, None) is None]


def check(status: int, what: str = "") -> None:
    if status == FLG_OK:
        return
    msg = load().flg_last_error().decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if status == FLG_ERR_INVALID:
        raise ValueError(text)
    if status == FLG_ERR_NOT_CONVERGED:
        raise RuntimeError(text)
    if status == FLG_ERR_SINGULAR:
        raise LinAlgError(text)
    if status == FLG_ERR_NOMEM:
        raise MemoryError(text)
    if status == FLG_ERR_TIMEOUT:
        raise RuntimeError(text)
    raise RuntimeError(f"CUDA error in {text}")
