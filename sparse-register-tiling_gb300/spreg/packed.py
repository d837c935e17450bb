"""PackedMatrix: a sparse A packed on the GPU, and the executor call C (+)= A . B."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .mapping import Mapping

DESC_DTYPE = np.dtype([("values_off", "<i8"), ("cols_off", "<i8"), ("counts_off", "<i8"),
                       ("num_values", "<i4"), ("num_cols", "<i4")])


def torch_dtype_code(dt) -> int:
    import torch
    if dt == torch.float32:
        return _lib.F32
    if dt == torch.bfloat16:
        return _lib.BF16
    if dt == torch.float16:
        return _lib.F16
    raise TypeError(f"unsupported dtype {dt} (float32, bfloat16 or float16)")


def torch_dtype_of(code: int):
    import torch
    return {_lib.F32: torch.float32, _lib.BF16: torch.bfloat16, _lib.F16: torch.float16}[code]


def _require_cuda(t, name):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")


class PackedMatrix:
    """Owner (or borrower) of a ``spreg_packed*``."""

    def __init__(self, handle, mapping: Mapping, owner: bool = True, keepalive=None):
        self._h = handle
        self.mapping = mapping
        self._owner = owner
        self._keepalive = keepalive
        self.info = self._get_info()

    # ---------------------------------------------------------------- construction
    @classmethod
    def from_dense(cls, A, mapping: Mapping, m_tile: int = 0, k_tile: int = 0, col_offset: int = 0,
                   value_dtype: int = _lib.F32, stream=None) -> "PackedMatrix":
        """Pack a dense float32 CUDA matrix; its nonzeros define the column patterns."""
        import torch
        _require_cuda(A, "A")
        if A.dtype != torch.float32 or A.dim() != 2:
            raise ValueError("A must be a 2-D float32 tensor")
        if A.stride(1) != 1:
            A = A.contiguous()
        opts = _lib.PackOpts(m_tile, k_tile, col_offset, value_dtype)
        h = C.c_void_p()
        _lib.check(_lib.lib().spreg_pack_dense(mapping.handle, A.data_ptr(), A.shape[0], A.shape[1], A.stride(0),
                                               C.byref(opts), C.byref(h), _lib.stream_handle(stream)))
        return cls(h, mapping)

    @classmethod
    def from_csr(cls, row_ptrs, col_inds, values, shape, mapping: Mapping, m_tile: int = 0, k_tile: int = 0,
                 col_offset: int = 0, value_dtype: int = _lib.F32, stream=None) -> "PackedMatrix":
        """Pack a CSR matrix given as CUDA tensors (int32 row_ptrs / col_inds, float32 values)."""
        import torch
        for t, n in ((row_ptrs, "row_ptrs"), (col_inds, "col_inds"), (values, "values")):
            _require_cuda(t, n)
        row_ptrs = row_ptrs.to(torch.int32).contiguous()
        col_inds = col_inds.to(torch.int32).contiguous()
        values = values.to(torch.float32).contiguous()
        csr = _lib.Csr(int(shape[0]), int(shape[1]), int(col_inds.numel()), row_ptrs.data_ptr(),
                       col_inds.data_ptr() if col_inds.numel() else None, values.data_ptr() if values.numel() else None)
        opts = _lib.PackOpts(m_tile, k_tile, col_offset, value_dtype)
        h = C.c_void_p()
        _lib.check(_lib.lib().spreg_pack_csr(mapping.handle, C.byref(csr), C.byref(opts), C.byref(h),
                                             _lib.stream_handle(stream)))
        return cls(h, mapping)

    @classmethod
    def from_torch_sparse(cls, A, mapping: Mapping, **kw) -> "PackedMatrix":
        A = A.to_sparse_csr()
        return cls.from_csr(A.crow_indices(), A.col_indices(), A.values(), A.shape, mapping, **kw)

    # ---------------------------------------------------------------- queries
    @property
    def handle(self):
        return self._h

    def _get_info(self) -> dict:
        info = _lib.PackedInfo()
        _lib.check(_lib.lib().spreg_packed_get_info(self._h, C.byref(info)))
        return info.as_dict()

    @property
    def shape(self):
        return (self.info["rows"], self.info["cols"])

    @property
    def value_dtype(self) -> int:
        return self.info["value_dtype"]

    def to_host(self):
        """(arena uint8[arena_bytes], descs structured[num_units], scales float32[num_panels] or None)."""
        import torch
        n_arena = self.info["arena_bytes"]
        arena = np.zeros(max(n_arena, 1), dtype=np.uint8)
        descs = np.zeros(max(self.info["num_units"], 1), dtype=DESC_DTYPE)
        scales = np.zeros(max(self.info["num_panels"], 1), dtype=np.float32)
        _lib.check(_lib.lib().spreg_packed_to_host(self._h, arena.ctypes.data, arena.size, descs.ctypes.data,
                                                   descs.size, scales.ctypes.data, scales.size,
                                                   _lib.stream_handle(torch.cuda.current_stream())))
        sc = scales[: self.info["num_panels"]] if self.value_dtype == _lib.F16 else None
        return arena[:n_arena], descs[: self.info["num_units"]], sc

    # ---------------------------------------------------------------- executor
    def exec_args(self, B, C_out, n=None, load_c=False, epilogue=_lib.EPILOGUE_NONE, nr=0, warps=0,
                  staging=0, meta=0, order=0, rounds=0, balance=0) -> _lib.ExecArgs:
        n = B.shape[1] if n is None else int(n)
        return _lib.ExecArgs(B.data_ptr(), B.stride(0), C_out.data_ptr(), C_out.stride(0), n,
                             torch_dtype_code(B.dtype), torch_dtype_code(C_out.dtype), int(bool(load_c)),
                             int(epilogue), int(nr), int(warps), int(staging), int(meta), int(order), int(rounds),
                             int(balance), 0)

    def _check_operands(self, B, C_out):
        _require_cuda(B, "B")
        _require_cuda(C_out, "C")
        if B.dim() != 2 or C_out.dim() != 2 or B.stride(1) != 1 or C_out.stride(1) != 1:
            raise ValueError("B and C must be 2-D with unit column stride")
        need = self.info["cols"] + self.info["col_offset"]
        if B.shape[0] < need:
            raise ValueError(f"B has {B.shape[0]} rows; the packed column indices reach {need}")
        if C_out.shape[0] != self.info["rows"]:
            raise ValueError(f"C has {C_out.shape[0]} rows, A has {self.info['rows']}")

    def execute(self, B, C_out=None, n=None, load_c=False, epilogue=_lib.EPILOGUE_NONE, nr=0, warps=0,
                out_dtype=None, stream=None, staging=0, meta=0, order=0, rounds=0, balance=0):
        """C (+)= A . B over the first n columns of B; returns C.  ``rounds`` > 1: panel rounds of the
        B-tile kernel (the strip of B for every K tile stays in shared memory for that many rounds of
        panels).  ``balance`` = 1: the load-balanced split of the heaviest panels' K tiles
        (`load_balance_plan`)."""
        import torch
        if C_out is None:
            if load_c:
                raise ValueError("load_c needs an output tensor")
            C_out = torch.empty((self.info["rows"], B.shape[1]), device=B.device,
                                dtype=out_dtype if out_dtype is not None else torch.float32)
        self._check_operands(B, C_out)
        args = self.exec_args(B, C_out, n, load_c, epilogue, nr, warps, staging, meta, order, rounds, balance)
        _lib.check(_lib.lib().spreg_execute(self._h, C.byref(args), _lib.stream_handle(stream)))
        return C_out

    def execute_timed(self, B, C_out, num_runs: int = 1, n=None, nr=0, warps=0, stream=None, staging=0,
                      meta=0, rounds=0, balance=0) -> float:
        """Median per-run time (ns) over 150 x num_runs runs of C = A . B (template:308-349)."""
        self._check_operands(B, C_out)
        args = self.exec_args(B, C_out, n, False, 0, nr, warps, staging, meta, rounds=rounds, balance=balance)
        t = C.c_double()
        _lib.check(_lib.lib().spreg_execute_timed(self._h, C.byref(args), int(num_runs), C.byref(t),
                                                  _lib.stream_handle(stream)))
        return float(t.value)

    def explain(self, B, C_out, n=None, load_c=False, epilogue=_lib.EPILOGUE_NONE, nr=0, warps=0, staging=0, meta=0,
                order=0, rounds=0, balance=0) -> dict:
        """The plan execute() would make with these arguments (spreg_execute_explain), as a dict."""
        self._check_operands(B, C_out)
        args = self.exec_args(B, C_out, n, load_c, epilogue, nr, warps, staging, meta, order, rounds, balance)
        buf = C.create_string_buffer(512)
        _lib.check(_lib.lib().spreg_execute_explain(self._h, C.byref(args), buf, len(buf)))
        out = {}
        for kv in buf.value.decode().split():
            k, _, v = kv.partition("=")
            out[k] = int(v) if v.lstrip("-").isdigit() else v
        return out

    def load_balance_plan(self, B, C_out, n=None, nr=0, warps=0, staging=0, rounds=0):
        """(heavy panels, split K tile, their row-panel indices) of the load-balanced split that
        execute(B, C_out, ..., balance=1) makes when it runs alone (spreg_load_balance_plan);
        (0, 0, []) when nothing is split."""
        self._check_operands(B, C_out)
        args = self.exec_args(B, C_out, n, nr=nr, warps=warps, staging=staging, rounds=rounds, balance=1)
        h, t = C.c_int64(), C.c_int32()
        ids = np.zeros(max(1, int(self.info["num_panels"])), dtype=np.int32)
        _lib.check(_lib.lib().spreg_load_balance_plan(self._h, C.byref(args), C.byref(h), C.byref(t),
                                                      ids.ctypes.data, ids.size))
        return int(h.value), int(t.value), ids[: int(h.value)].copy()

    # ---------------------------------------------------------------- bytes / flops
    def algorithmic_bytes(self, n: int, b_bytes: int = 4, c_bytes: int = 4, load_c: bool = False) -> int:
        """Packed values + indices + counts + descriptors (+scales) + B (K x n) + C (M x n, x2 if load_c)."""
        i = self.info
        return int(i["algorithmic_bytes"] + i["cols"] * n * b_bytes + i["rows"] * n * c_bytes * (2 if load_c else 1))

    def flops(self, n: int) -> int:
        """2 * nnz * n (tools/paperv2/dlmc/utils.py:47-48); padding FMAs are not counted."""
        return 2 * int(self.info["nnz"]) * int(n)

    def __del__(self):
        try:
            if self._owner and self._h is not None:
                _lib.lib().spreg_packed_destroy(self._h)
                self._h = None
        except Exception:
            pass


def device_status(reset: bool = False) -> int:
    """Status word of the current device (nonzero: a kernel gave up a bounded wait)."""
    v = C.c_int32()
    _lib.check(_lib.lib().spreg_device_status(C.byref(v), int(bool(reset))))
    return int(v.value)


def selftest_wait_timeout(limit: int = 1000) -> tuple:
    """(status word, polls) after a kernel waited `limit` polls on an mbarrier nothing arrives on:
    the bounded wait every executor uses gives up and records 30 instead of hanging."""
    st, polls = C.c_int32(), C.c_uint32()
    _lib.check(_lib.lib().spreg_selftest_wait_timeout(int(limit), C.byref(st), C.byref(polls),
                                                      _lib.stream_handle(None)))
    return int(st.value), int(polls.value)


def execute_batched(items, stream=None) -> None:
    """Run [(PackedMatrix, B, C, kwargs), ...] as one work list."""
    arr = (_lib.WorkItem * max(len(items), 1))()
    for i, (pm, B, Cm, kw) in enumerate(items):
        pm._check_operands(B, Cm)
        arr[i].a = pm.handle
        arr[i].args = pm.exec_args(B, Cm, **kw)
    _lib.check(_lib.lib().spreg_execute_batched(arr, len(items), _lib.stream_handle(stream)))


def work_items(triples):
    """spreg_work_item array of [(PackedMatrix, B, C), ...] (C = A . B over all of B's columns)."""
    arr = (_lib.WorkItem * max(len(triples), 1))()
    for i, (pm, B, Cm) in enumerate(triples):
        pm._check_operands(B, Cm)
        arr[i].a = pm.handle
        arr[i].args = pm.exec_args(B, Cm)
    return arr
