"""Dense panels on the tensor cores, the rest register-tiled.

A row panel (M_r rows) whose fill -- nonzeros / (M_r x K) -- reaches `tc_fill` runs as part of a
dense product on the tensor cores; the other panels are packed and executed as usual.  The threshold
is a tuning parameter (`tune_tc_fill` measures it); above 1.0 disables the tensor-core part, 0.0 runs
every panel on it.  Two storage forms:
  * BF16 (``spreg_dense_rows_bf16``): BF16 values and B, FP32 accumulation in tensor memory; the error
    bound is that of an FP32-accumulated BF16 product;
  * FP32 (``spreg_dense_rows_f32``): the FP32 executor's accuracy at tensor-core rate.  The dense rows
    and B are split into scaled FP16 pairs and multiplied as hi.hi + hi.lo + lo.hi; the result carries
    the error of an FP32 dot product in the tensor core's summation order (the register-tiled rows stay
    bit-identical to the oracle).

Order of the two parts, so that load_c and the ReLU epilogue apply once to every row: without
load_c the register-tiled part runs first (its empty dense panels store zeros), then the tensor-core
part writes those rows; with load_c the tensor-core part runs first (C_in + A.B, epilogue), then
the register-tiled part adds nothing to those rows (ReLU of a ReLU result is the same value).
The reference runs every panel register-tiled (cpp_testbed/src/spmm/nano/SpMM_SOP.h:174-178).
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from . import _lib
from .mapping import Mapping
from .packed import PackedMatrix


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


def split_rows_f32(a_rows, stream=None):
    """The FP16 split pair of FP32 rows (spreg_dense_rows_f32_split): returns (a_split, row_scale) with
    a_split 2R x K8 float16 (rows [0, R) high halves, [R, 2R) low halves) and row_scale float32 R."""
    import torch
    if not a_rows.is_cuda or a_rows.dtype != torch.float32 or a_rows.dim() != 2 or a_rows.stride(1) != 1:
        raise ValueError("a_rows must be a 2-D float32 CUDA tensor with unit column stride")
    R, k = a_rows.shape
    k8 = max(8, (k + 7) // 8 * 8)
    a_split = torch.empty((2 * R, k8), dtype=torch.float16, device=a_rows.device)
    scale = torch.empty(R, dtype=torch.float32, device=a_rows.device)
    _lib.check(_lib.lib().spreg_dense_rows_f32_split(a_rows.data_ptr(), R, k, a_rows.stride(0), a_split.data_ptr(),
                                                     k8, scale.data_ptr(), _lib.stream_handle(stream)))
    return a_split, scale


def f32_item(a_split, row_scale, row_index, B, C, n: Optional[int] = None, k: Optional[int] = None,
             load_c: bool = False, epilogue: int = _lib.EPILOGUE_NONE, tile_n: int = 0) -> "_lib.DenseRowsF32Item":
    """spreg_dense_rows_f32_item of one FP32-accurate product (CUDA tensors: the split pair, FP32 B and C)."""
    import torch
    n = B.shape[1] if n is None else int(n)
    k = B.shape[0] if k is None else int(k)
    R = a_split.shape[0] // 2
    if B.dtype != torch.float32 or C.dtype != torch.float32 or a_split.dtype != torch.float16:
        raise ValueError("B and C must be float32, the split pair float16")
    if B.stride(1) != 1 or C.stride(1) != 1 or a_split.shape[1] < k or B.shape[0] < k:
        raise ValueError("operands need unit column stride and K columns / rows")
    if n > B.shape[1] or n > C.shape[1] or row_index.numel() != R or row_scale.numel() != R:
        raise ValueError("n exceeds B or C, or the row index / scales do not match the split pair")
    return _lib.DenseRowsF32Item(a_split.data_ptr(), R, k, a_split.stride(0), row_scale.data_ptr(),
                                 row_index.data_ptr(), B.data_ptr(), B.stride(0), C.data_ptr(), C.stride(0), n,
                                 int(bool(load_c)), int(epilogue), int(tile_n), 0)


def dense_rows_f32(a_split, row_scale, row_index, B, C, n: Optional[int] = None, load_c: bool = False,
                   epilogue: int = _lib.EPILOGUE_NONE, stream=None):
    """C[row_index[i], :n] (+)= A_rows[i, :K] . B[:, :n] with FP32 accuracy on the tensor cores (A_rows
    given as its split pair from `split_rows_f32`; B, C float32 CUDA tensors)."""
    import ctypes
    it = f32_item(a_split, row_scale, row_index, B, C, n=n, load_c=load_c, epilogue=epilogue)
    _lib.check(_lib.lib().spreg_dense_rows_f32(ctypes.byref(it), _lib.stream_handle(stream)))
    return C


def bf16_items(rows) -> np.ndarray:
    """spreg_dense_rows_item records (numpy) of BF16 products [(a_rows, row_index, B, C, n, k, load_c,
    epilogue), ...] (CUDA tensors; C float32 or BF16)."""
    import torch
    from .serving import TC_ITEM_DTYPE
    it = np.zeros(len(rows), dtype=TC_ITEM_DTYPE)
    for i, (a, idx, B, C, n, k, load_c, epi) in enumerate(rows):
        it[i] = (a.data_ptr(), a.shape[0], k, a.stride(0), idx.data_ptr(), B.data_ptr(), B.stride(0), C.data_ptr(),
                 C.stride(0), n, _lib.F32 if C.dtype == torch.float32 else _lib.BF16, int(bool(load_c)), int(epi), 0)
    return it


class DenseRowsPlan:
    """A reusable plan of tensor-core products over fixed tensors (spreg_dense_rows_f32_plan_create for
    FP32-accurate items, spreg_dense_rows_bf16_plan_create for a numpy array of BF16 items): a run is
    the B preparation and the tensor-core launches, with no host-side work (capturable)."""

    def __init__(self, items, stream=None):
        import ctypes
        h = ctypes.c_void_p()
        if isinstance(items, np.ndarray):
            _lib.check(_lib.lib().spreg_dense_rows_bf16_plan_create(items.ctypes.data, len(items), ctypes.byref(h),
                                                                    _lib.stream_handle(stream)))
        else:
            arr = (_lib.DenseRowsF32Item * max(1, len(items)))(*items)
            _lib.check(_lib.lib().spreg_dense_rows_f32_plan_create(arr, len(items), ctypes.byref(h),
                                                                   _lib.stream_handle(stream)))
        self._h = h

    def run(self, stream=None) -> None:
        _lib.check(_lib.lib().spreg_dense_rows_plan_run(self._h, _lib.stream_handle(stream)))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().spreg_dense_rows_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HybridMatrix:
    """A pruned matrix split into tensor-core panels (fill >= tc_fill) and register-tiled panels.

    value_dtype BF16: BF16 values and B, FP32 or BF16 output.  value_dtype F32: FP32 values, B and C;
    the tensor-core rows run as FP32-accurate split products."""

    def __init__(self, packed: PackedMatrix, a_rows, row_index, rows: int, cols: int, tc_fill: float,
                 value_dtype: int = _lib.BF16, row_scale=None):
        self.packed = packed
        self.a_rows = a_rows          # BF16 rows, or (F32) the FP16 split pair (2 x tc_rows rows)
        self.row_scale = row_scale    # F32 only
        self.row_index = row_index
        self.rows, self.cols = rows, cols
        self.tc_fill = tc_fill
        self.value_dtype = value_dtype

    @classmethod
    def from_dense(cls, A, mapping: Mapping, tc_fill: float, k_tile: int = 0, m_tile: int = 0,
                   value_dtype: int = _lib.BF16) -> "HybridMatrix":
        import torch
        if not A.is_cuda or A.dtype != torch.float32 or A.dim() != 2:
            raise ValueError("A must be a 2-D float32 CUDA tensor")
        if value_dtype not in (_lib.BF16, _lib.F32):
            raise ValueError("the hybrid stores BF16 or FP32 values")
        mr = mapping.mr
        m, k = A.shape
        fill = panel_fill(A, mr)
        dense_p = torch.nonzero(fill >= tc_fill).flatten() if tc_fill <= 1.0 else torch.zeros(0, dtype=torch.long,
                                                                                              device=A.device)
        rows = (dense_p[:, None] * mr + torch.arange(mr, device=A.device)[None, :]).flatten()
        rows = rows[rows < m]
        A_sp = A.clone()
        k8 = max(8, (k + 7) // 8 * 8)
        scale = None
        if value_dtype == _lib.F32:
            a_rows, scale = split_rows_f32(A[rows].contiguous()) if rows.numel() else (
                torch.zeros((0, k8), dtype=torch.float16, device=A.device),
                torch.zeros(0, dtype=torch.float32, device=A.device))
        else:
            a_rows = torch.zeros((rows.numel(), k8), dtype=torch.bfloat16, device=A.device)
            if rows.numel():
                a_rows[:, :k] = A[rows].to(torch.bfloat16)
        if rows.numel():
            A_sp[rows] = 0.0
        packed = PackedMatrix.from_dense(A_sp, mapping, m_tile=m_tile, k_tile=k_tile, value_dtype=value_dtype)
        return cls(packed, a_rows, rows.to(torch.int32).contiguous(), m, k, tc_fill, value_dtype, scale)

    @property
    def tc_rows(self) -> int:
        return int(self.row_index.numel())

    @property
    def all_tc(self) -> bool:
        return self.tc_rows == self.rows and self.cols > 0

    def tc_item(self, B, C, n: Optional[int] = None, load_c: bool = False, epilogue: int = _lib.EPILOGUE_NONE):
        """spreg_dense_rows_f32_item of the tensor-core part (F32 storage)."""
        return f32_item(self.a_rows, self.row_scale, self.row_index, B, C, n=n, k=self.cols, load_c=load_c,
                        epilogue=epilogue)

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
        if self.all_tc:
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
        if self.value_dtype == _lib.F32:
            import ctypes
            it = self.tc_item(B, C, n=n, load_c=load_c, epilogue=epilogue)
            _lib.check(_lib.lib().spreg_dense_rows_f32(ctypes.byref(it), _lib.stream_handle(stream)))
            return
        cd = _lib.F32 if C.dtype == torch.float32 else _lib.BF16
        _lib.check(_lib.lib().spreg_dense_rows_bf16(
            self.a_rows.data_ptr(), self.a_rows.shape[0], self.cols, self.a_rows.stride(0), self.row_index.data_ptr(),
            B.data_ptr(), B.stride(0), C.data_ptr(), C.stride(0), n, cd, int(bool(load_c)), int(epilogue),
            _lib.stream_handle(stream)))


class HybridBatch:
    """Many hybrid SpMMs C_i = A_i . B_i over fixed tensors in as few launches as possible: the
    register-tiled parts in one batched executor call, the tensor-core parts as one reusable plan
    (B preparation + tensor-core launches; BF16 products of one weight coalesce).  Without load_c
    the register-tiled part runs first, as in HybridMatrix.execute.  All hybrids of one batch share
    a storage type."""

    def __init__(self, triples, stream=None):
        from .packed import work_items
        self.triples = list(triples)
        kinds = {h.value_dtype for h, _, _ in self.triples}
        if len(kinds) > 1:
            raise ValueError("one storage type per HybridBatch")
        tc_t = [(h, B, C) for h, B, C in self.triples if h.tc_rows and h.cols > 0]
        if not tc_t:
            self.plan = None
        elif kinds == {_lib.F32}:
            self.plan = DenseRowsPlan([h.tc_item(B, C) for h, B, C in tc_t], stream=stream)
        else:
            self.plan = DenseRowsPlan(bf16_items([(h.a_rows, h.row_index, B, C, B.shape[1], h.cols, False, 0)
                                                  for h, B, C in tc_t]), stream=stream)
        sp = [(h.packed, B, C) for h, B, C in self.triples if not h.all_tc]
        self.items = work_items(sp) if sp else None
        self.n_sparse = len(sp)

    def run(self, stream=None) -> None:
        if self.items is not None:
            _lib.check(_lib.lib().spreg_execute_batched(self.items, self.n_sparse, _lib.stream_handle(stream)))
        if self.plan is not None:
            self.plan.run(stream)


def tune_tc_fill(A, mapping: Mapping, n: int, fills=(1.01, 0.5, 0.3, 0.2, 0.1, 0.05, 0.0), k_tile: int = 0,
                 reps: int = 20, value_dtype: int = _lib.BF16, batch: int = 8) -> dict:
    """Time the hybrid at each threshold on the device (BF16 or FP32 storage, n columns): `batch`
    SpMMs of A with distinct B as one HybridBatch (one batched register-tiled launch, one tensor-core
    plan), so neither part pays per-call set-up; returns {fill: us per SpMM} and the fastest
    threshold."""
    import torch
    Bs = [torch.randn((A.shape[1], n), device=A.device) for _ in range(max(1, batch))]
    if value_dtype == _lib.BF16:
        Bs = [b.to(torch.bfloat16) for b in Bs]
    Cs = [torch.empty((A.shape[0], n), device=A.device) for _ in Bs]
    out = {}
    for f in fills:
        h = HybridMatrix.from_dense(A, mapping, f, k_tile=k_tile, value_dtype=value_dtype)
        hb = HybridBatch([(h, b, c) for b, c in zip(Bs, Cs)])
        cur = torch.cuda.current_stream()
        side = torch.cuda.Stream()
        side.wait_stream(cur)
        with torch.cuda.stream(side):
            hb.run()  # lazy set-up outside the capture
        cur.wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()  # device time: the batched launch's host planning stays out
        with torch.cuda.graph(g):
            hb.run()
        for _ in range(3):  # warm-up: clock ramp stays out of the timed replays
            g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
        out[float(f)] = e0.elapsed_time(e1) / reps * 1e3 / len(Bs)
        del g, hb, h
    best = min(out, key=out.get)
    return {"us": out, "best_fill": best, "batch": len(Bs)}
