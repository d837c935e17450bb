"""Dense panels on the tensor cores, the rest register-tiled.

A row panel (M_r rows) whose fill -- nonzeros / (M_r x K) -- reaches `tc_fill` runs as part of a
dense BF16 product on the tensor cores (``spreg_dense_rows_bf16``: tcgen05 MMA, FP32 accumulation
in tensor memory); the other panels are packed and executed as usual.  The threshold is a tuning
parameter (`tune_tc_fill` measures it); 1.0 disables the tensor-core part, 0.0 runs every panel on
it.

Order of the two parts, so that load_c and the ReLU epilogue apply once to every row: without
load_c the register-tiled part runs first (its empty dense panels store zeros), then the tensor-core
part writes those rows; with load_c the tensor-core part runs first (C_in + A.B, epilogue), then
the register-tiled part adds nothing to those rows (ReLU of a ReLU result is the same value).
Results of the tensor-core rows are not bit-identical to the register-tiled order; the error bound
is that of an FP32-accumulated BF16 product.
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from . import _lib
from .mapping import Mapping
from .packed import PackedMatrix


def set_tc_cluster(mode: int) -> None:
    """Clusters of the tensor-core launches that follow (process-wide): 0 automatic, 1 single CTAs,
    2 CTA pairs sharing each B tile through TMA multicast (spreg_tc_set_cluster)."""
    _lib.check(_lib.lib().spreg_tc_set_cluster(int(mode)))


def dense_rows_bf16(a_rows, row_index, B, C, n: Optional[int] = None, load_c: bool = False,
                    epilogue: int = _lib.EPILOGUE_NONE, stream=None, check_rows: bool = True):
    """C[row_index[i], :n] (+)= a_rows[i, :K] . B[:, :n] with K = B's rows, on the tensor cores (CUDA
    tensors; a_rows (at least K columns) and B BF16, row_index int32 rows of C, C float32 or BF16).

    check_rows reads the row indices back to check them against C (a device synchronisation);
    callers whose indices are known to be in range pass False."""
    import torch
    n = B.shape[1] if n is None else int(n)
    k = B.shape[0]
    if a_rows.shape[1] < k:
        raise ValueError(f"a_rows has {a_rows.shape[1]} columns, B has {k} rows")
    if n > B.shape[1] or n > C.shape[1]:
        raise ValueError("n exceeds the columns of B or C")
    for t, nm in ((a_rows, "a_rows"), (row_index, "row_index"), (B, "B"), (C, "C")):
        if not t.is_cuda:
            raise ValueError(f"{nm} must be a CUDA tensor")
    if a_rows.dtype != torch.bfloat16 or B.dtype != torch.bfloat16 or row_index.dtype != torch.int32:
        raise ValueError("a_rows and B must be bfloat16, row_index int32")
    if C.dtype not in (torch.float32, torch.bfloat16):
        raise ValueError("C must be float32 or bfloat16")
    if a_rows.stride(1) != 1 or B.stride(1) != 1 or C.stride(1) != 1:
        raise ValueError("operands need unit column stride")
    if row_index.numel() != a_rows.shape[0]:
        raise ValueError("one row index per A row")
    if check_rows and row_index.numel() and (int(row_index.min()) < 0 or int(row_index.max()) >= C.shape[0]):
        raise ValueError("a row index lies outside C")
    cd = _lib.F32 if C.dtype == torch.float32 else _lib.BF16
    _lib.check(_lib.lib().spreg_dense_rows_bf16(
        a_rows.data_ptr(), a_rows.shape[0], k, a_rows.stride(0), row_index.data_ptr(), B.data_ptr(),
        B.stride(0), C.data_ptr(), C.stride(0), n, cd, int(bool(load_c)), int(epilogue), _lib.stream_handle(stream)))
    return C


def panel_fill(A, mr: int):
    """Fill of every row panel (nonzeros / (mr x K)) of a CUDA float32 matrix."""
    import torch
    m, k = A.shape
    P = (m + mr - 1) // mr
    nz = torch.zeros(P * mr, device=A.device, dtype=torch.float32)
    nz[:m] = (A != 0).sum(dim=1).to(torch.float32)
    return nz.view(P, mr).sum(dim=1) / float(mr * max(k, 1))


class HybridMatrix:
    """A pruned matrix split into tensor-core panels (fill >= tc_fill) and register-tiled panels.

    BF16 storage (values and B), FP32 or BF16 output -- the tensor cores take BF16 operands."""

    def __init__(self, packed: PackedMatrix, a_rows, row_index, rows: int, cols: int, tc_fill: float):
        self.packed = packed
        self.a_rows = a_rows
        self.row_index = row_index
        self.rows, self.cols = rows, cols
        self.tc_fill = tc_fill

    @classmethod
    def from_dense(cls, A, mapping: Mapping, tc_fill: float, k_tile: int = 0, m_tile: int = 0) -> "HybridMatrix":
        import torch
        if not A.is_cuda or A.dtype != torch.float32 or A.dim() != 2:
            raise ValueError("A must be a 2-D float32 CUDA tensor")
        mr = mapping.mr
        m, k = A.shape
        fill = panel_fill(A, mr)
        dense_p = torch.nonzero(fill >= tc_fill).flatten() if tc_fill <= 1.0 else torch.zeros(0, dtype=torch.long,
                                                                                              device=A.device)
        rows = (dense_p[:, None] * mr + torch.arange(mr, device=A.device)[None, :]).flatten()
        rows = rows[rows < m]
        A_sp = A.clone()
        k8 = max(8, (k + 7) // 8 * 8)
        a_rows = torch.zeros((rows.numel(), k8), dtype=torch.bfloat16, device=A.device)
        if rows.numel():
            a_rows[:, :k] = A[rows].to(torch.bfloat16)
            A_sp[rows] = 0.0
        packed = PackedMatrix.from_dense(A_sp, mapping, m_tile=m_tile, k_tile=k_tile, value_dtype=_lib.BF16)
        return cls(packed, a_rows, rows.to(torch.int32).contiguous(), m, k, tc_fill)

    @property
    def tc_rows(self) -> int:
        return int(self.row_index.numel())

    def execute(self, B, C=None, n: Optional[int] = None, load_c: bool = False, epilogue: int = _lib.EPILOGUE_NONE,
                nr: int = 0, stream=None):
        import torch
        if C is None:
            if load_c:
                raise ValueError("load_c needs an output tensor")
            C = torch.empty((self.rows, B.shape[1]), device=B.device, dtype=torch.float32)
        if B.shape[0] < self.cols or C.shape[0] != self.rows or (n or B.shape[1]) > min(B.shape[1], C.shape[1]):
            raise ValueError(f"B needs {self.cols} rows, C {self.rows} rows, both at least n columns")
        kw = dict(n=n, load_c=load_c, epilogue=epilogue, nr=nr, stream=stream)
        if self.tc_rows == self.rows and self.cols > 0:
            self._tc(B, C, n, load_c, epilogue, stream)  # every row is a tensor-core row
        elif self.tc_rows and self.cols > 0:
            if load_c:
                self._tc(B, C, n, True, epilogue, stream)
                self.packed.execute(B, C, **kw)
            else:
                self.packed.execute(B, C, **kw)
                self._tc(B, C, n, False, epilogue, stream)
        else:
            self.packed.execute(B, C, **kw)
        return C

    def _tc(self, B, C, n, load_c, epilogue, stream):
        n = B.shape[1] if n is None else int(n)
        import torch
        cd = _lib.F32 if C.dtype == torch.float32 else _lib.BF16
        _lib.check(_lib.lib().spreg_dense_rows_bf16(
            self.a_rows.data_ptr(), self.a_rows.shape[0], self.cols, self.a_rows.stride(0), self.row_index.data_ptr(),
            B.data_ptr(), B.stride(0), C.data_ptr(), C.stride(0), n, cd, int(bool(load_c)), int(epilogue),
            _lib.stream_handle(stream)))


def tune_tc_fill(A, mapping: Mapping, n: int, fills=(1.01, 0.5, 0.3, 0.2, 0.1, 0.05, 0.0), k_tile: int = 0,
                 reps: int = 20) -> dict:
    """Time the hybrid at each threshold on the device (BF16, n columns); returns {fill: us} and the
    fastest threshold."""
    import torch
    B = torch.randn((A.shape[1], n), device=A.device).to(torch.bfloat16)
    C = torch.empty((A.shape[0], n), device=A.device)
    out = {}
    for f in fills:
        h = HybridMatrix.from_dense(A, mapping, f, k_tile=k_tile)
        for _ in range(3):  # warm-up: lazy set-up and clock ramp stay out of the timed calls
            h.execute(B, C)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            h.execute(B, C)
        e1.record()
        torch.cuda.synchronize()
        out[float(f)] = e0.elapsed_time(e1) / reps * 1e3
    best = min(out, key=out.get)
    return {"us": out, "best_fill": best}
