"""MatMulSpecialized: the C++ inspector/executor pair of the reference, on the GPU.

Mirrors the use in cpp_testbed/src/spmm/nano/SpMM_SOP.h:107-178:
``MatMulSpecialized(m, k, n, values, row_ptrs, col_inds, tile_config, nThreads, executor_id,
mapping_id, packed)`` packs A in the constructor; ``get_config()``, ``allocate_executor(n)``,
``require_storage`` and ``__call__(C, B)`` (operator()(C, B): C = A . B) follow.
Host arrays (numpy / CPU tensors) run through the host-buffer C entry point, CUDA tensors
through the device entry point.
"""
from __future__ import annotations

import ctypes as C
import re
from dataclasses import asdict, dataclass

import numpy as np

from . import _lib
from .mapping import Mapping
from .packed import PackedMatrix

# Outer schedules of tools/paper/configs.py:9-25.  K runs inside every GPU job, so a schedule with N
# outside M hands out column strips outer (spreg_exec_args.job_order = 1), the others row panels outer.
SCHEDULES = {"KNM": 0, "NKM": 1, "MNK": 2, "NMK": 3, "KMN": 4, "MKN": 5, "KM": 6, "MK": 7, "KN": 8, "NK": 9,
             "MN": 10, "NM": 11, "K": 12, "N": 13, "M": 14}


@dataclass
class TileConfig:
    """sop::TileConfig / SOPConfig (SpMM_SOP.h:33-54).  M_c/K_c = 0 means one tile (the GPU default)."""
    M_c: int = 0
    K_c: int = 0
    N_c: int = 0
    nr: int = 0
    runtimeSchedule: int = 0
    value_dtype: int = _lib.F32
    sparse_a: int = 1
    tiling_strategy: int = 0
    beta: float = 1.0
    load_balance: int = 0  # the load-balanced kernel (KD_IntelLoadBalanced; spreg_exec_args.load_balance)

    def to_c(self) -> _lib.TileConfig:
        return _lib.TileConfig(self.M_c, self.K_c, self.N_c, self.nr, self.runtimeSchedule, self.value_dtype,
                               self.sparse_a, self.tiling_strategy, int(round(self.beta * 10)), int(self.load_balance))

    @classmethod
    def from_c(cls, t: _lib.TileConfig) -> "TileConfig":
        return cls(t.m_tile, t.k_tile, t.n_tile, t.nr, t.outer_schedule, t.value_dtype, t.sparse_a,
                   t.tiling_strategy, t.beta_10x / 10.0, t.load_balance)

    @classmethod
    def from_sop_config(cls, cfg: dict) -> "TileConfig":
        """From the reference's int config map (m_tile, k_tile, n_tile, tiling_strategy, beta_10x, sparse_a)."""
        return cls(M_c=cfg.get("m_tile", 0), K_c=cfg.get("k_tile", 0), N_c=cfg.get("n_tile", 0),
                   tiling_strategy=cfg.get("tiling_strategy", 0), beta=cfg.get("beta_10x", 10) / 10.0,
                   sparse_a=cfg.get("sparse_a", 1))


def _host_i32(x):
    a = np.asarray(x.cpu() if hasattr(x, "cpu") else x)
    return np.ascontiguousarray(a, dtype=np.int32)


def _host_f32(x):
    a = np.asarray(x.detach().cpu() if hasattr(x, "detach") else x)
    return np.ascontiguousarray(a, dtype=np.float32)


def nr_from_executor_id(executor_id: str) -> int:
    """Columns per strip from an executor id such as 'AVX512_512_4' (nr vectors of vec_width_bits)."""
    m = re.search(r"_(\d+)_(\d+)$", executor_id or "")
    if not m:
        return 0
    nr = int(m.group(1)) // 32 * int(m.group(2))
    return nr if nr in (32, 64, 128, 256, 512) else 0


class MatMulSpecialized:
    def __init__(self, m: int, k: int, n: int, values, row_ptrs, col_inds, tile_config: TileConfig | None = None,
                 nThreads: int = 1, executor_id: str = "", mapping_id: str | Mapping = "61fee", packed: bool = True):
        self.m, self.k, self.n = int(m), int(k), int(n)
        self.mapping = mapping_id if isinstance(mapping_id, Mapping) else Mapping.load(mapping_id)
        cfg = tile_config or TileConfig()
        if cfg.nr == 0:
            cfg.nr = nr_from_executor_id(executor_id)
        self.nThreads = nThreads  # the GPU needs no thread count; kept for the reference signature
        self.executor_id = executor_id
        v, rp, ci = _host_f32(values), _host_i32(row_ptrs), _host_i32(col_inds)
        self._keep = (v, rp, ci)
        h = C.c_void_p()
        ccfg = cfg.to_c()
        _lib.check(_lib.lib().spreg_matmul_create(self.m, self.k, self.n, v.ctypes.data, rp.ctypes.data,
                                                  ci.ctypes.data, C.byref(ccfg), self.mapping.handle, C.byref(h)))
        self._h = h
        self._keep = None
        self.packed = PackedMatrix(_lib.lib().spreg_matmul_packed(h), self.mapping, owner=False, keepalive=self)

    def get_config(self) -> TileConfig:
        t = _lib.TileConfig()
        _lib.check(_lib.lib().spreg_matmul_get_config(self._h, C.byref(t)))
        return TileConfig.from_c(t)

    def allocate_executor(self, n: int) -> None:
        _lib.check(_lib.lib().spreg_matmul_allocate_executor(self._h, int(n)))
        self.n = int(n)

    @property
    def require_storage(self) -> int:
        return int(_lib.lib().spreg_matmul_required_storage(self._h))

    def __call__(self, C_out, B, stream=None):
        """operator()(C, B): C = A . B.  C is (m x n) and B is (k x n), both row-major."""
        if hasattr(B, "is_cuda") and B.is_cuda:
            if not (C_out.is_cuda and B.is_contiguous() and C_out.is_contiguous()):
                raise ValueError("device call needs contiguous CUDA B and C")
            if tuple(B.shape) != (self.k, self.n) or tuple(C_out.shape) != (self.m, self.n):
                raise ValueError(f"expected B {self.k}x{self.n} and C {self.m}x{self.n}")
            _lib.check(_lib.lib().spreg_matmul_run_device(self._h, C_out.data_ptr(), B.data_ptr(),
                                                          _lib.stream_handle(stream)))
            return C_out
        fast = self._torch_host_ptrs(C_out, B)
        if fast is not None:
            _lib.check(_lib.lib().spreg_matmul_run(self._h, fast[0], fast[1]))
            return C_out
        b, ptr = self._host_args(C_out, B)
        _lib.check(_lib.lib().spreg_matmul_run(self._h, ptr, b.ctypes.data))
        return C_out

    def run_async(self, C_out, B):
        """operator()(C, B) on host buffers, enqueued without waiting (copy in, product, copy out on
        this matmul's stream).  C_out and B must stay alive and unchanged until sync(); pin them
        (torch pin_memory) for copies that overlap other matmuls' work."""
        fast = self._torch_host_ptrs(C_out, B)  # contiguous float32 CPU tensors: no numpy round trip
        if fast is not None:
            _lib.check(_lib.lib().spreg_matmul_run_async(self._h, fast[0], fast[1]))
            return C_out
        b, ptr = self._host_args(C_out, B)
        src = B.data_ptr() if hasattr(B, "data_ptr") else (B.ctypes.data if isinstance(B, np.ndarray) else None)
        if b.ctypes.data != src:  # a converted copy would be freed before the enqueued copy reads it
            raise ValueError("run_async needs B as a contiguous float32 host buffer (no conversion copy)")
        _lib.check(_lib.lib().spreg_matmul_run_async(self._h, ptr, b.ctypes.data))
        return C_out

    def _torch_host_ptrs(self, C_out, B):
        """(C, B) data pointers when both are contiguous float32 CPU torch tensors of the right
        shapes, else None (the general path converts and checks)."""
        import torch
        if not (isinstance(B, torch.Tensor) and isinstance(C_out, torch.Tensor)):
            return None
        if B.is_cuda or C_out.is_cuda or B.dtype != torch.float32 or C_out.dtype != torch.float32:
            return None
        if not (B.is_contiguous() and C_out.is_contiguous()):
            return None
        if tuple(B.shape) != (self.k, self.n) or tuple(C_out.shape) != (self.m, self.n):
            return None
        return C_out.data_ptr(), B.data_ptr()

    def set_direct_output(self, direct: bool = True) -> None:
        """Host-buffer calls with a pinned C store C straight into it from the kernel (no copy out);
        other C buffers keep the copy path.  Results are identical."""
        _lib.check(_lib.lib().spreg_matmul_set_direct_output(self._h, int(bool(direct))))

    def sync(self) -> None:
        """Wait for this matmul's enqueued calls; their C buffers then hold the results."""
        _lib.check(_lib.lib().spreg_matmul_sync(self._h))

    def _host_args(self, C_out, B):
        b = _host_f32(B)
        if b.shape != (self.k, self.n):
            raise ValueError(f"expected B {self.k}x{self.n}, got {b.shape}")
        if hasattr(C_out, "numpy"):  # CPU tensor
            if not C_out.is_contiguous() or C_out.dtype.__str__() != "torch.float32":
                raise ValueError("C must be a contiguous float32 CPU tensor")
            if tuple(C_out.shape) != (self.m, self.n):
                raise ValueError(f"expected C {self.m}x{self.n}")
            ptr = C_out.data_ptr()
        else:
            if C_out.dtype != np.float32 or not C_out.flags["C_CONTIGUOUS"]:
                raise ValueError("C must be a contiguous float32 array")
            if C_out.shape != (self.m, self.n):
                raise ValueError(f"expected C {self.m}x{self.n}")
            ptr = C_out.ctypes.data
        return b, ptr

    def __del__(self):
        try:
            if getattr(self, "_h", None) is not None:
                self.packed = None
                _lib.lib().spreg_matmul_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def config_dict(self) -> dict:
        return asdict(self.get_config())
