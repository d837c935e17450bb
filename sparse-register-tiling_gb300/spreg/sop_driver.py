"""Drop-in for the reference's Python SOP binding surface.

Mirrors sbench/SOP/sop_driver.py:38-129 (``Acc``, ``SOPModule``, ``make_sop_module``) and the
torch module built from sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:396-409
(``sort_and_encode_patterns``, ``SOPTile.pack_panel`` / ``pack_tile`` / ``padding``,
``execute_tile``), with the packer and executor running as sm_103a kernels of libspreg.so.

Differences from the reference, all documented extensions:
  * a last panel with fewer than M_r rows is zero-padded (the reference rejects it, template:139);
  * execute_tile accepts N_c not a multiple of N_r (the reference exits, template:300-303);
  * B may be a CPU or CUDA tensor; C comes back on B's device.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Callable, Iterable

import numpy as np

from . import _lib
from .mapping import Mapping
from .packed import PackedMatrix, torch_dtype_code


@dataclass
class Acc:
    """Accumulator shape: M = panel height M_r, N = accumulator width in 512-bit vectors (16 floats)."""
    M: int = 4
    N: int = 4

    @property
    def nr_floats(self) -> int:
        return 16 * self.N


def pattern_code(vec) -> int:
    """Bit i set iff vec[i] != 0 (sbench/SOP/distribution.py:10-15)."""
    v = np.asarray(vec.cpu() if hasattr(vec, "cpu") else vec)
    return int(sum(1 << i for i, x in enumerate(v.reshape(-1)) if x != 0))


def panel_pattern_codes(panel_t: np.ndarray) -> np.ndarray:
    """Pattern code of every row of a transposed panel (K x M_r)."""
    bits = (panel_t != 0).astype(np.int64)
    return (bits << np.arange(panel_t.shape[1], dtype=np.int64)).sum(axis=1).astype(np.int32)


def _nr_of(acc: Acc) -> int:
    nr = acc.nr_floats
    return nr if nr in (32, 64, 128, 256, 512) else 0


class SOPTile:
    """SOPTile(rows, cols, num_panels) of template:101-262, packed on the GPU by pack_tile()."""

    def __init__(self, module: "SOPModule", rows: int, cols: int, num_panels: int):
        self.module = module
        self.rows, self.cols, self.num_panels = int(rows), int(cols), int(num_panels)
        h = C.c_void_p()
        _lib.check(_lib.lib().spreg_tile_create(module.mapping.handle, self.rows, self.cols, self.num_panels,
                                                C.byref(h)))
        self._h = h
        self._packed = None

    def pack_panel(self, panel_id: int, col_offset: int, pat_codes, col_indices, dense_panel) -> None:
        """Stage one panel: entries (nanokernel pattern code, column) and its dense (K x M_r) values."""
        codes = np.ascontiguousarray(np.asarray(pat_codes.cpu() if hasattr(pat_codes, "cpu") else pat_codes),
                                     dtype=np.int32)
        cols = np.ascontiguousarray(np.asarray(col_indices.cpu() if hasattr(col_indices, "cpu") else col_indices),
                                    dtype=np.int32)
        dense = np.asarray(dense_panel.detach().cpu() if hasattr(dense_panel, "detach") else dense_panel,
                           dtype=np.float32)
        if dense.ndim != 2 or dense.shape[1] != self.module.acc.M:
            raise RuntimeError(f"dense_panel must be (K, {self.module.acc.M}), got {tuple(dense.shape)}")
        if codes.shape != cols.shape:
            raise RuntimeError("pat_codes and col_indices differ in length")
        dense = np.ascontiguousarray(dense)
        _lib.check(_lib.lib().spreg_tile_pack_panel(self._h, int(panel_id), int(col_offset), codes.ctypes.data,
                                                    cols.ctypes.data, codes.size, dense.ctypes.data, dense.shape[0]))

    def pack_tile(self, value_dtype: int | None = None, stream=None) -> None:
        vd = self.module.value_dtype if value_dtype is None else value_dtype
        _lib.check(_lib.lib().spreg_tile_pack(self._h, vd, _lib.stream_handle(stream)))
        self._packed = PackedMatrix(_lib.lib().spreg_tile_packed(self._h), self.module.mapping, owner=False,
                                    keepalive=self)

    def padding(self) -> int:
        if self._packed is None:
            raise RuntimeError("padding() is available after pack_tile()")
        return int(_lib.lib().spreg_tile_padding(self._h))

    @property
    def tile_packed(self) -> bool:
        return self._packed is not None

    @property
    def packed(self) -> PackedMatrix:
        if self._packed is None:
            raise RuntimeError("tile is not packed (call pack_tile)")
        return self._packed

    def __del__(self):
        try:
            if self._h is not None:
                self._packed = None
                _lib.lib().spreg_tile_destroy(self._h)
                self._h = None
        except Exception:
            pass


class SOPModule:
    """Module for one (Acc, nanokernel set, pattern mapping) -- sop_driver.py:38-85."""

    def __init__(self, acc: Acc, patterns, pattern_mapping, mapping: Mapping, kernel_id: str,
                 value_dtype: int = _lib.F32):
        self.acc = acc
        self.patterns = patterns
        self.pattern_mapping = pattern_mapping
        self.mapping = mapping
        self.kernel_id = kernel_id
        self.value_dtype = value_dtype

    def make_sop_tile(self, tile, col_offset: int = 0) -> SOPTile:
        """Split a dense tile into M_r-row panels, map every column's pattern and pack (sop_driver.py:47-74)."""
        t = np.asarray(tile.detach().cpu() if hasattr(tile, "detach") else tile, dtype=np.float32)
        mr = self.acc.M
        num_panels = math.ceil(t.shape[0] / mr)
        sop_tile = self.SOPTile(t.shape[0], t.shape[1], num_panels)
        for panel_id in range(num_panels):
            rows = t[panel_id * mr:(panel_id + 1) * mr, :]
            if rows.shape[0] < mr:
                rows = np.vstack([rows, np.zeros((mr - rows.shape[0], t.shape[1]), np.float32)])
            panel = np.ascontiguousarray(rows.T)
            codes = panel_pattern_codes(panel)
            pc, ci = [], []
            for i, code in enumerate(codes):
                mapped = self.pattern_mapping(int(code))
                if isinstance(mapped, (int, np.integer)):
                    pc.append(int(mapped))
                    ci.append(i)
                else:
                    for m in mapped:
                        pc.append(int(m))
                        ci.append(i)
            sop_tile.pack_panel(panel_id, col_offset, np.asarray(pc, np.int32), np.asarray(ci, np.int32), panel)
        sop_tile.pack_tile()
        return sop_tile

    def SOPTile(self, rows: int, cols: int, num_panels: int) -> SOPTile:
        return SOPTile(self, rows, cols, num_panels)

    def sort_and_encode_patterns(self, pat_codes):
        return sort_and_encode_patterns(self.mapping, pat_codes)

    def execute_tile(self, tile: SOPTile, B, num_runs: int = 1024, N_c: int | None = None):
        """(median time per run in ns, C = A . B over the first N_c columns) -- template:351-392."""
        import torch
        N_c = B.shape[-1] if N_c is None else int(N_c)
        if not tile.tile_packed:
            raise RuntimeError("tile.tile_packed failed: call pack_tile() first")
        if B.shape[0] != tile.cols:
            raise RuntimeError(f"cols size mismatch with B.size(0) ({tile.cols} vs {B.shape[0]})")
        if not B.is_contiguous():
            raise RuntimeError("B must be contiguous")
        dev_B = B if B.is_cuda else B.cuda()
        want = torch.float32 if tile.packed.value_dtype == _lib.F32 else \
            (torch.bfloat16 if tile.packed.value_dtype == _lib.BF16 else torch.float16)
        if dev_B.dtype != want:
            dev_B = dev_B.to(want)
        Cd = torch.zeros((tile.rows, B.shape[1]), dtype=torch.float32, device=dev_B.device)
        t_ns = tile.packed.execute_timed(dev_B, Cd, num_runs=num_runs, n=N_c, nr=_nr_of(self.acc))
        Cd.zero_()
        tile.packed.execute(dev_B, Cd, n=N_c, load_c=True, nr=_nr_of(self.acc))
        torch.cuda.synchronize()
        return t_ns, (Cd if B.is_cuda else Cd.cpu())

    def executor(self, csr, B, num_runs: int = 1024, N_c: int | None = None):
        """Pack a torch sparse CSR matrix and execute it (sop_driver.py:83-85)."""
        import torch
        A = csr.to_sparse_csr()
        dev = B.device if B.is_cuda else torch.device("cuda")
        pm = PackedMatrix.from_csr(A.crow_indices().to(dev), A.col_indices().to(dev), A.values().to(dev),
                                   A.shape, self.mapping, value_dtype=self.value_dtype)
        N_c = B.shape[-1] if N_c is None else int(N_c)
        dB = B.to(dev)
        Cd = torch.zeros((A.shape[0], B.shape[1]), dtype=torch.float32, device=dev)
        t_ns = pm.execute_timed(dB, Cd, num_runs=num_runs, n=N_c, nr=_nr_of(self.acc))
        Cd.zero_()
        pm.execute(dB, Cd, n=N_c, nr=_nr_of(self.acc))
        torch.cuda.synchronize()
        return t_ns, (Cd if B.is_cuda else Cd.cpu())


class CsrModule:
    """The reference's `csr` torch module (sbench/SOP/sop_driver.py:33-34, built from
    _C/pytorch_csr_wrapper.cpp): the CSR baseline that the register-tiled executor is timed against
    (sop_bench.py:197).  Here it runs as a CUDA kernel (`spreg_csr_spmm`): row x N-tile FMAs in CSR
    order, bit-identical to the restated baseline."""

    def executor(self, mat, B, num_runs: int = 1024, n_tile: int = 64):
        """(time, C) = executor(mat, B, num_runs, n_tile) (pytorch_csr_wrapper.cpp:314-353): C = mat . B
        for a 2-D sparse CSR tensor and a contiguous B; time = median ns per run of 150 x num_runs
        runs after num_runs warm-up runs.  C is on B's device."""
        import torch
        if not getattr(mat, "is_sparse_csr", False) and getattr(mat, "layout", None) != torch.sparse_csr:
            raise RuntimeError("mat must be a sparse CSR tensor (TORCH_INTERNAL_ASSERT mat.is_sparse_csr())")
        if mat.dim() != 2:
            raise RuntimeError("mat must be 2-D")
        rows, cols = int(mat.shape[0]), int(mat.shape[1])
        if cols != B.shape[0]:
            raise RuntimeError(f"mat.size(1) size mismatch with B.size(0) ({cols} vs {B.shape[0]})")
        if not B.is_contiguous():
            raise RuntimeError("B must be contiguous")
        nnz = int(mat._nnz())
        if nnz > 2 ** 31 - 1:
            raise RuntimeError("nnz out of range for int32 indices")
        dev = B.device if B.is_cuda else torch.device("cuda", torch.cuda.current_device())
        rp = mat.crow_indices().to(dev, torch.int32).contiguous()
        ci = mat.col_indices().to(dev, torch.int32).contiguous()
        v = mat.values().to(dev, torch.float32).contiguous()
        dB = B.to(dev, torch.float32).contiguous()
        n = int(dB.shape[1])
        Cd = torch.zeros((rows, n), dtype=torch.float32, device=dev)
        stream = _lib.stream_handle(None)
        args = (rows, cols, n, nnz, rp.data_ptr(), ci.data_ptr() if nnz else None, v.data_ptr() if nnz else None,
                dB.data_ptr(), n, Cd.data_ptr(), n, int(n_tile))
        t = C.c_double()
        _lib.check(_lib.lib().spreg_csr_spmm_timed(*args, int(num_runs), C.byref(t), stream))
        Cd.zero_()
        _lib.check(_lib.lib().spreg_csr_spmm(*args, stream))
        torch.cuda.synchronize(dev)
        return float(t.value), (Cd if B.is_cuda else Cd.cpu())


csr = CsrModule()


def sort_and_encode_patterns(mapping: Mapping, pat_codes):
    """(encoded, order) of template:84-98, computed by a GPU kernel; returns int32 tensors on pat_codes' device."""
    import torch
    src = torch.as_tensor(pat_codes, dtype=torch.int32)
    d = src.cuda() if not src.is_cuda else src
    d = d.contiguous()
    enc = torch.empty_like(d)
    order = torch.empty_like(d)
    _lib.check(_lib.lib().spreg_sort_and_encode_patterns(mapping.handle, d.data_ptr(), d.numel(), enc.data_ptr(),
                                                         order.data_ptr(), _lib.stream_handle(None)))
    if not src.is_cuda:
        return enc.cpu(), order.cpu()
    return enc, order


kernel_cache: dict = {}


def kernel_typename(acc: Acc, nanokernels: Iterable[int], arch: str = "GB300") -> str:
    ks = sorted(set(int(k) for k in nanokernels if int(k)))
    tag = hex(abs(hash(tuple(ks))) & 0xFFFFF)[2:]
    return f"spreg_{arch}_M{acc.M}_N{acc.N}_{len(ks)}k_{tag}"


def make_sop_module(acc: Acc, patterns, pattern_mapping: Callable[[int], int | list[int]] | Mapping,
                    regen: bool = False, value_dtype: int = _lib.F32) -> SOPModule:
    """make_sop_module(acc, patterns, pattern_mapping) of sop_driver.py:88-129.

    ``patterns`` is the nanokernel set (0 is not a valid pattern, sop_driver.py:90); the
    executor is already compiled, so nothing is generated or JIT-built."""
    patterns = list(patterns)
    assert 0 not in patterns, "Zero is not a valid pattern"
    if isinstance(pattern_mapping, Mapping):
        mapping = Mapping(pattern_mapping.mr, pattern_mapping.table, patterns)
        fn = pattern_mapping
    else:
        mapping = Mapping.from_callable(acc.M, pattern_mapping, patterns)
        fn = pattern_mapping
    kid = kernel_typename(acc, patterns)
    return SOPModule(acc, patterns, fn, mapping, kid, value_dtype)
