"""ctypes binding of libspreg.so (the C ABI declared in include/spreg.h).

The library is built in-tree by ``sparse-register-tiling_gb300/build.py``.  There is no CPU
fallback: if the library is missing every entry point raises ``SpregLibraryMissing``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libspreg.so")

SPREG_OK = 0
SPREG_ERR_INVALID_ARG = 1
SPREG_ERR_CUDA = 2
SPREG_ERR_UNSUPPORTED = 3
SPREG_ERR_STATE = 4
SPREG_ERR_CHECK = 5
SPREG_ERR_NOMEM = 6

F32, BF16, F16 = 0, 1, 2
ZERO_PATTERN_ID = 0xFFFF
EPILOGUE_NONE, EPILOGUE_RELU = 0, 1


class SpregLibraryMissing(RuntimeError):
    """libspreg.so has not been built; run sparse-register-tiling_gb300/build.py."""


class SpregError(RuntimeError):
    """A libspreg call returned a non-zero status (the reference raises RuntimeError via TORCH_CHECK)."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"spreg error {status}: {msg}")
        self.status = status


class PanelDesc(C.Structure):
    _fields_ = [("values_off", C.c_int64), ("cols_off", C.c_int64), ("counts_off", C.c_int64),
                ("num_values", C.c_int32), ("num_cols", C.c_int32)]


class PackedInfo(C.Structure):
    _fields_ = [("rows", C.c_int64), ("cols", C.c_int64), ("num_panels", C.c_int64), ("num_units", C.c_int64),
                ("mr", C.c_int32), ("num_nkern", C.c_int32), ("m_tile", C.c_int32), ("k_tile", C.c_int32),
                ("num_k_tiles", C.c_int32), ("value_dtype", C.c_int32), ("col_offset", C.c_int64),
                ("nnz", C.c_int64), ("num_values", C.c_int64), ("num_col_indices", C.c_int64),
                ("padding", C.c_int64), ("arena_bytes", C.c_int64), ("required_storage", C.c_int64),
                ("algorithmic_bytes", C.c_int64), ("empty_units", C.c_int64)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class Csr(C.Structure):
    _fields_ = [("rows", C.c_int64), ("cols", C.c_int64), ("nnz", C.c_int64), ("row_ptrs", C.c_void_p),
                ("col_inds", C.c_void_p), ("values", C.c_void_p)]


class PackOpts(C.Structure):
    _fields_ = [("m_tile", C.c_int32), ("k_tile", C.c_int32), ("col_offset", C.c_int64), ("value_dtype", C.c_int32)]


class ArenaGeom(C.Structure):
    _fields_ = [("rows", C.c_int64), ("cols", C.c_int64), ("m_tile", C.c_int32), ("k_tile", C.c_int32),
                ("col_offset", C.c_int64), ("value_dtype", C.c_int32), ("reserved", C.c_int32)]


class ExecArgs(C.Structure):
    _fields_ = [("b", C.c_void_p), ("ldb", C.c_int64), ("c", C.c_void_p), ("ldc", C.c_int64), ("n", C.c_int64),
                ("b_dtype", C.c_int32), ("c_dtype", C.c_int32), ("load_c", C.c_int32), ("epilogue", C.c_int32),
                ("nr", C.c_int32), ("warps_per_cta", C.c_int32), ("b_staging", C.c_int32),
                ("meta_staging", C.c_int32), ("job_order", C.c_int32), ("panel_rounds", C.c_int32),
                ("load_balance", C.c_int32), ("reserved", C.c_int32)]


class WorkItem(C.Structure):
    _fields_ = [("a", C.c_void_p), ("args", ExecArgs)]


class DenseRowsF32Item(C.Structure):
    _fields_ = [("a_split", C.c_void_p), ("rows", C.c_int64), ("k", C.c_int64), ("ld_split", C.c_int64),
                ("row_scale", C.c_void_p), ("row_index", C.c_void_p), ("b", C.c_void_p), ("ldb", C.c_int64),
                ("c", C.c_void_p), ("ldc", C.c_int64), ("n", C.c_int64), ("load_c", C.c_int32),
                ("epilogue", C.c_int32), ("tile_n", C.c_int32), ("reserved", C.c_int32)]


class TileConfig(C.Structure):
    _fields_ = [("m_tile", C.c_int32), ("k_tile", C.c_int32), ("n_tile", C.c_int32), ("nr", C.c_int32),
                ("outer_schedule", C.c_int32), ("value_dtype", C.c_int32), ("sparse_a", C.c_int32),
                ("tiling_strategy", C.c_int32), ("beta_10x", C.c_int32), ("load_balance", C.c_int32)]


P = C.c_void_p
I32P = C.POINTER(C.c_int32)
# name -> (restype, argtypes); every function of include/spreg.h
PROTOTYPES = {
    "spreg_last_error": (C.c_char_p, []),
    "spreg_version": (C.c_int, []),
    "spreg_mapping_create": (C.c_int, [C.c_int32, P, P, P, C.c_int32, C.POINTER(P)]),
    "spreg_mapping_destroy": (None, [P]),
    "spreg_mapping_mr": (C.c_int32, [P]),
    "spreg_mapping_num_nkern": (C.c_int32, [P]),
    "spreg_mapping_nkern_patterns": (C.c_int, [P, P]),
    "spreg_mapping_encode": (C.c_int32, [P, C.c_int32]),
    "spreg_sort_and_encode_patterns": (C.c_int, [P, P, C.c_int64, P, P, P]),
    "spreg_pack_csr": (C.c_int, [P, C.POINTER(Csr), C.POINTER(PackOpts), C.POINTER(P), P]),
    "spreg_pack_dense": (C.c_int, [P, P, C.c_int64, C.c_int64, C.c_int64, C.POINTER(PackOpts), C.POINTER(P), P]),
    "spreg_packed_destroy": (None, [P]),
    "spreg_packed_get_info": (C.c_int, [P, C.POINTER(PackedInfo)]),
    "spreg_packed_device_ptrs": (C.c_int, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
    "spreg_packed_to_host": (C.c_int, [P, P, C.c_int64, P, C.c_int64, P, C.c_int64, P]),
    "spreg_dense_rows_bf16": (C.c_int, [P, C.c_int64, C.c_int64, C.c_int64, P, P, C.c_int64, P, C.c_int64,
                                        C.c_int64, C.c_int32, C.c_int32, C.c_int32, P]),
    "spreg_dense_rows_bf16_batched": (C.c_int, [P, C.c_int32, P]),
    "spreg_dense_rows_f32_split": (C.c_int, [P, C.c_int64, C.c_int64, C.c_int64, P, C.c_int64, P, P]),
    "spreg_dense_rows_f32": (C.c_int, [C.POINTER(DenseRowsF32Item), P]),
    "spreg_dense_rows_f32_batched": (C.c_int, [P, C.c_int32, P]),
    "spreg_dense_rows_f32_plan_create": (C.c_int, [P, C.c_int32, C.POINTER(P), P]),
    "spreg_dense_rows_bf16_plan_create": (C.c_int, [P, C.c_int32, C.POINTER(P), P]),
    "spreg_dense_rows_plan_run": (C.c_int, [P, P]),
    "spreg_dense_rows_plan_destroy": (None, [P]),
    "spreg_pack_from_arena": (C.c_int, [P, C.POINTER(ArenaGeom), P, C.c_int64, P, C.c_int64, P, C.c_int64,
                                        C.POINTER(P), P]),
    "spreg_tile_create": (C.c_int, [P, C.c_int64, C.c_int64, C.c_int64, C.POINTER(P)]),
    "spreg_tile_pack_panel": (C.c_int, [P, C.c_int64, C.c_int64, P, P, C.c_int64, P, C.c_int64]),
    "spreg_tile_pack": (C.c_int, [P, C.c_int32, P]),
    "spreg_tile_padding": (C.c_int64, [P]),
    "spreg_tile_packed": (P, [P]),
    "spreg_tile_destroy": (None, [P]),
    "spreg_execute": (C.c_int, [P, C.POINTER(ExecArgs), P]),
    "spreg_execute_batched": (C.c_int, [P, C.c_int32, P]),
    "spreg_device_status": (C.c_int, [C.POINTER(C.c_int32), C.c_int32]),
    "spreg_execute_batched_noalloc": (C.c_int, [P, C.c_int32, P]),
    "spreg_execute_timed": (C.c_int, [P, C.POINTER(ExecArgs), C.c_int64, C.POINTER(C.c_double), P]),
    "spreg_execute_explain": (C.c_int, [P, C.POINTER(ExecArgs), C.c_char_p, C.c_int64]),
    "spreg_load_balance_plan": (C.c_int, [P, C.POINTER(ExecArgs), C.POINTER(C.c_int64), C.POINTER(C.c_int32), P,
                                          C.c_int64]),
    "spreg_selftest_wait_timeout": (C.c_int, [C.c_uint32, C.POINTER(C.c_int32), C.POINTER(C.c_uint32), P]),
    "spreg_csr_spmm": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_int64, P, P, P, P, C.c_int64, P, C.c_int64,
                                 C.c_int32, P]),
    "spreg_csr_spmm_timed": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_int64, P, P, P, P, C.c_int64, P,
                                       C.c_int64, C.c_int32, C.c_int64, C.POINTER(C.c_double), P]),
    "spreg_matmul_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, P, P, P, C.POINTER(TileConfig), P,
                                      C.POINTER(P)]),
    "spreg_matmul_allocate_executor": (C.c_int, [P, C.c_int32]),
    "spreg_matmul_run": (C.c_int, [P, P, P]),
    "spreg_matmul_run_async": (C.c_int, [P, P, P]),
    "spreg_matmul_sync": (C.c_int, [P]),
    "spreg_matmul_set_direct_output": (C.c_int, [P, C.c_int32]),
    "spreg_matmul_run_device": (C.c_int, [P, P, P, P]),
    "spreg_matmul_get_config": (C.c_int, [P, C.POINTER(TileConfig)]),
    "spreg_matmul_required_storage": (C.c_int64, [P]),
    "spreg_matmul_packed": (P, [P]),
    "spreg_matmul_destroy": (None, [P]),
}

_lib = None
_lock = threading.Lock()


def lib():
    """The loaded libspreg.so (raises SpregLibraryMissing if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise SpregLibraryMissing(
                    f"{LIB_PATH} not found: build it with `python sparse-register-tiling_gb300/build.py` "
                    "(there is no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in PROTOTYPES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def last_error() -> str:
    return lib().spreg_last_error().decode(errors="replace")


def check(status: int) -> None:
    if status != SPREG_OK:
        raise SpregError(status, last_error())


def stream_handle(stream=None) -> int:
    """cudaStream_t of a torch stream (current stream by default) as an integer."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)
