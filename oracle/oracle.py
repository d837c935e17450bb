"""Python front end of the CPU oracle (oracle/spreg_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
reference arm import this module, as the checker or the timed CPU baseline.  The product
package never imports it.

Every function restates a step of the reference's sparse-register-tiling path; the C source
cites the reference file:line of each.  Pinning: tests/test_oracle.py checks it against the
reference's mapping-file ids (md5 of content), its known-answer tests (0/1 A times B = ones),
the packer invariant, and outputs of the reference's own spmm_naive.cpp compiled by
``make ref`` (tests/golden/ holds fixtures generated from it for machines without the reference).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_naive.so")
# Checkout of the reference project, for building its spmm_naive (absent on machines without it).
REFERENCE_ROOT = os.environ.get("SPREG_REFERENCE", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

F32, BF16, F16 = 0, 1, 2
ZERO = 0xFFFF
DESC_DTYPE = np.dtype([("values_off", "<i8"), ("cols_off", "<i8"), ("counts_off", "<i8"),
                       ("num_values", "<i4"), ("num_cols", "<i4")])

_lib = None
_ref = None


def build(with_reference: bool | None = None) -> None:
    """Compile liboracle.so, and _ref/libref_naive.so when the reference checkout is present."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if with_reference is None:
        with_reference = os.path.exists(os.path.join(REFERENCE_ROOT, "cpp_testbed/src/spmm/baselines/spmm_naive.cpp"))
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REFERENCE_ROOT}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_reference=False)
        _lib = C.CDLL(LIB_PATH)
        _lib.orc_f16_panel_scale.restype = C.c_float
        _lib.orc_f16_panel_scale.argtypes = [C.c_float]
        _lib.orc_max_threads.restype = C.c_int
    return _lib


def has_ref() -> bool:
    return os.path.exists(REF_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_PATH)
    return _ref


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def max_threads() -> int:
    return int(lib().orc_max_threads())


# ---------------------------------------------------------------- conversions
def f32_to_bf16(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    out = np.empty(a.shape, dtype=np.uint16)
    lib().orc_f32_to_bf16_array(_p(a), _p(out), C.c_int64(a.size))
    return out


def f32_to_f16(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    out = np.empty(a.shape, dtype=np.uint16)
    lib().orc_f32_to_f16_array(_p(a), _p(out), C.c_int64(a.size))
    return out


def bf16_to_f32(u: np.ndarray) -> np.ndarray:
    return (np.asarray(u, dtype=np.uint32) << 16).view(np.float32)


def f16_to_f32(u: np.ndarray) -> np.ndarray:
    return np.asarray(u, dtype=np.uint16).view(np.float16).astype(np.float32)


def f16_panel_scale(maxabs: float) -> float:
    return float(lib().orc_f16_panel_scale(C.c_float(maxabs)))


# ---------------------------------------------------------------- mapping tables
class Tables:
    """id <-> pattern tables of a nanokernel set plus the mapping lists (offsets / codes)."""

    def __init__(self, mr: int, table: dict, nanokernels=None):
        self.mr = int(mr)
        offs = [0]
        codes: list[int] = []
        for p in range(2 ** self.mr):
            codes += [int(c) for c in table.get(p, [])]
            offs.append(len(codes))
        self.offsets = np.asarray(offs, dtype=np.int32)
        self.codes = np.asarray(codes if codes else [0], dtype=np.int32)
        self.id_to_pattern = np.zeros(256, dtype=np.int32)
        self.code_to_id = np.zeros(256, dtype=np.int32)
        nks = None if nanokernels is None else np.asarray(list(nanokernels), dtype=np.int32)
        n = lib().orc_mapping_build(self.mr, _p(self.offsets), _p(self.codes),
                                    _p(nks) if nks is not None else None,
                                    0 if nks is None else len(nks), _p(self.id_to_pattern), _p(self.code_to_id))
        if n < 0:
            raise ValueError("bad mapping")
        self.num_nkern = int(n)

    @classmethod
    def of(cls, mapping) -> "Tables":
        """From any object with .mr, .table and optionally .nanokernels (e.g. spreg.Mapping)."""
        return cls(mapping.mr, mapping.table, getattr(mapping, "nanokernels", None))


def sort_and_encode(t: Tables, pat_codes) -> tuple[np.ndarray, np.ndarray]:
    codes = np.ascontiguousarray(pat_codes, dtype=np.int32)
    enc = np.zeros(max(codes.size, 1), dtype=np.int32)
    order = np.zeros(max(codes.size, 1), dtype=np.int32)
    rc = lib().orc_sort_and_encode(_p(t.code_to_id), _p(codes), C.c_int64(codes.size), _p(enc), _p(order))
    if rc:
        raise ValueError("pattern code is not a nanokernel")
    return enc[: codes.size], order[: codes.size]


def permute_inplace(order, v) -> np.ndarray:
    o = np.ascontiguousarray(order, dtype=np.int32)
    out = np.ascontiguousarray(np.array(v, dtype=np.int32, copy=True))
    lib().orc_permute_inplace(_p(o), _p(out), C.c_int64(o.size))
    return out


def pack_panel(t: Tables, col_offset: int, pat_codes, col_indices, dense_panel: np.ndarray):
    """SOPTile::pack_panel restated: returns dict(counts, cols, values, padding)."""
    codes = np.ascontiguousarray(pat_codes, dtype=np.int32)
    cols = np.ascontiguousarray(col_indices, dtype=np.int32)
    dense = np.ascontiguousarray(dense_panel, dtype=np.float32)
    n = codes.size
    counts = np.zeros(max(t.num_nkern, 1), dtype=np.int32)
    cols_out = np.zeros(max(n, 1), dtype=np.int32)
    vals_out = np.zeros(max(n * t.mr, 1), dtype=np.float32)
    nv, nu, pad = C.c_int64(), C.c_int64(), C.c_int64()
    rc = lib().orc_pack_panel(t.mr, t.num_nkern, _p(t.code_to_id), _p(t.id_to_pattern), C.c_int64(col_offset),
                              _p(codes), _p(cols), C.c_int64(n), _p(dense), C.c_int64(dense.shape[0]), _p(counts),
                              _p(cols_out), _p(vals_out), C.byref(nv), C.byref(nu), C.byref(pad))
    if rc:
        raise ValueError({-1: "bad code", -2: "column out of range", -3: "invariant failed"}.get(rc, rc))
    return {"counts": counts[: t.num_nkern], "cols": cols_out[: nu.value], "values": vals_out[: nv.value],
            "padding": pad.value}


class Packed:
    """Oracle packing of a whole dense matrix (arena bytes + descriptors + scales + sizes)."""

    def __init__(self, t: Tables, A: np.ndarray, m_tile=0, k_tile=0, col_offset=0, value_dtype=F32):
        A = np.ascontiguousarray(A, dtype=np.float32)
        self.t = t
        self.M, self.K = A.shape
        self.value_dtype = value_dtype
        sizes = np.zeros(10, dtype=np.int64)
        P = (self.M + t.mr - 1) // t.mr
        args = (t.mr, t.num_nkern, _p(t.code_to_id), _p(t.id_to_pattern), _p(t.offsets), _p(t.codes), _p(A),
                C.c_int64(self.M), C.c_int64(self.K), C.c_int64(self.K), C.c_int32(m_tile), C.c_int32(k_tile),
                C.c_int64(col_offset), C.c_int(value_dtype))
        scales = np.ones(max(P, 1), dtype=np.float32)
        lib().orc_pack_dense(*args, None, None, _p(scales), _p(sizes))
        self.num_units = int(sizes[0])
        self.arena = np.zeros(max(int(sizes[1]), 1), dtype=np.uint8)
        self.descs = np.zeros(max(self.num_units, 1), dtype=DESC_DTYPE)
        rc = lib().orc_pack_dense(*args, _p(self.arena), _p(self.descs), _p(scales), _p(sizes))
        if rc:
            raise ValueError(f"oracle pack failed ({rc})")
        self.arena = self.arena[: int(sizes[1])]
        self.descs = self.descs[: self.num_units]
        self.scales = scales[:P] if value_dtype == F16 else None
        self._scales_buf = scales
        keys = ["num_units", "arena_bytes", "num_values", "num_col_indices", "padding", "nnz", "required_storage",
                "empty_units", "num_k_tiles", "panels_per_tile"]
        self.sizes = {k: int(v) for k, v in zip(keys, sizes)}
        self.num_panels = P

    def execute(self, B: np.ndarray, out: np.ndarray | None = None, n=None, load_c=False, epilogue=0, b_dtype=None,
                c_dtype=F32, threads=0) -> np.ndarray:
        """out (+)= A . B with the reference executor's FMA order.  16-bit B / out are uint16 bit arrays."""
        b_dtype = self.value_dtype if b_dtype is None else b_dtype
        B = np.ascontiguousarray(B)
        n = B.shape[1] if n is None else int(n)
        if out is None:
            out = np.zeros((self.M, B.shape[1]), dtype=np.float32 if c_dtype == F32 else np.uint16)
        arena = self.arena if self.arena.size else np.zeros(1, np.uint8)
        descs = self.descs if self.descs.size else np.zeros(1, DESC_DTYPE)
        lib().orc_execute(self.t.mr, self.t.num_nkern, _p(self.t.id_to_pattern), _p(arena), _p(descs),
                          _p(self._scales_buf), self.value_dtype, C_int64(self.M), C_int64(self.num_panels),
                          C_int64(self.sizes["panels_per_tile"]), C_int64(self.sizes["num_k_tiles"]), _p(B), b_dtype,
                          C_int64(B.shape[1]), _p(out), c_dtype, C_int64(out.shape[1]), C_int64(n),
                          int(bool(load_c)), int(epilogue), int(threads))
        return out

    def execute_fast(self, B: np.ndarray, out: np.ndarray | None = None, load_c=False, epilogue=0,
                     threads=0) -> np.ndarray:
        """The SIMD CPU executor (spreg_cpu_fast.c: per-pattern FMA blocks on vector registers; the timed
        CPU baseline), bit-identical to `execute` for FP32; N a multiple of 16."""
        if self.value_dtype != F32:
            raise ValueError("the SIMD CPU executor runs FP32 values")
        B = np.ascontiguousarray(B, dtype=np.float32)
        if out is None:
            out = np.zeros((self.M, B.shape[1]), dtype=np.float32)
        arena = self.arena if self.arena.size else np.zeros(1, np.uint8)
        descs = self.descs if self.descs.size else np.zeros(1, DESC_DTYPE)
        rc = lib().orc_execute_fast(self.t.mr, self.t.num_nkern, _p(self.t.id_to_pattern), _p(arena), _p(descs),
                                    C_int64(self.M), C_int64(self.num_panels), C_int64(self.sizes["panels_per_tile"]),
                                    C_int64(self.sizes["num_k_tiles"]), _p(B), C_int64(B.shape[1]), _p(out),
                                    C_int64(out.shape[1]), C_int64(B.shape[1]), int(bool(load_c)), int(epilogue),
                                    int(threads))
        if rc:
            raise ValueError("the SIMD CPU executor needs N a multiple of 16 and M_r <= 8")
        return out


def load_balanced_execute(t: Tables, A: np.ndarray, B: np.ndarray, heavy_panels, split_tile: int, k_tile: int,
                          m_tile=0, col_offset=0, value_dtype=F32, out: np.ndarray | None = None, load_c=False,
                          epilogue=0) -> np.ndarray:
    """The stated order of a load-balanced SpMM (the GPU executor's spreg_exec_args.load_balance):
    row panels in `heavy_panels` are C = lo + hi, one FP32 add, then the epilogue, where lo is the
    reference executor's chain over K tiles [0, split_tile) (from C with load_c, else from zero) and hi
    the chain over tiles [split_tile, T) from zero; every other panel is the reference executor's
    chain over all K tiles (template:265-305).

    Each half is executed from A with the other half's columns zeroed: units (panel, K tile) are
    packed independently, so the kept tiles pack and run exactly as in A, and the zeroed tiles have
    no entries (no FMAs).  FP32 or BF16 values (F16 packing scales each panel over all of K)."""
    if value_dtype == F16:
        raise ValueError("the load-balanced order is stated for FP32 and BF16 values")
    A = np.ascontiguousarray(A, dtype=np.float32)
    C0 = np.zeros((A.shape[0], B.shape[1]), dtype=np.float32) if out is None else out.astype(np.float32)
    kw = dict(m_tile=m_tile, k_tile=k_tile, col_offset=col_offset, value_dtype=value_dtype)
    full = Packed(t, A, **kw).execute(B, C0.copy(), load_c=load_c, epilogue=epilogue)
    kc = split_tile * k_tile
    a_lo, a_hi = A.copy(), A.copy()
    a_lo[:, kc:] = 0.0
    a_hi[:, :kc] = 0.0
    lo = Packed(t, a_lo, **kw).execute(B, C0.copy(), load_c=load_c)
    hi = Packed(t, a_hi, **kw).execute(B, np.zeros_like(C0))
    mr = t.mr
    for p in heavy_panels:
        r0, r1 = int(p) * mr, min(int(p) * mr + mr, A.shape[0])
        v = (lo[r0:r1] + hi[r0:r1]).astype(np.float32)
        full[r0:r1] = np.where(v > 0, v, np.float32(0.0)).astype(np.float32) if epilogue == 1 else v
    if out is not None:
        out[...] = full
    return full


def C_int64(v):
    return C.c_int64(int(v))


def csr_spmm(row_ptrs, col_inds, values, B: np.ndarray, threads=0) -> np.ndarray:
    """Restated CSR baseline (row x N-tile FMAs), OpenMP over rows."""
    rp = np.ascontiguousarray(row_ptrs, dtype=np.int32)
    ci = np.ascontiguousarray(col_inds, dtype=np.int32)
    v = np.ascontiguousarray(values, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    M = rp.size - 1
    out = np.zeros((M, B.shape[1]), dtype=np.float32)
    lib().orc_csr_spmm(C_int64(M), C_int64(B.shape[1]), _p(rp), _p(ci if ci.size else np.zeros(1, np.int32)),
                       _p(v if v.size else np.zeros(1, np.float32)), _p(B), C_int64(B.shape[1]), _p(out),
                       C_int64(B.shape[1]), int(threads))
    return out


def csr_spmm_fast(row_ptrs, col_inds, values, B: np.ndarray, threads=0) -> np.ndarray:
    """The CSR baseline as SIMD code (spreg_cpu_fast.c), bit-identical to `csr_spmm`; N a multiple of 64."""
    rp = np.ascontiguousarray(row_ptrs, dtype=np.int32)
    ci = np.ascontiguousarray(col_inds, dtype=np.int32)
    v = np.ascontiguousarray(values, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    M = rp.size - 1
    out = np.zeros((M, B.shape[1]), dtype=np.float32)
    rc = lib().orc_csr_spmm_fast(C_int64(M), C_int64(B.shape[1]), _p(rp), _p(ci if ci.size else np.zeros(1, np.int32)),
                                 _p(v if v.size else np.zeros(1, np.float32)), _p(B), C_int64(B.shape[1]), _p(out),
                                 C_int64(B.shape[1]), int(threads))
    if rc:
        raise ValueError("the SIMD CSR baseline needs N a multiple of 64")
    return out


def ref_naive(row_ptrs, col_inds, values, B: np.ndarray) -> np.ndarray:
    """The reference's own spmm_naive (compiled from its source by `make ref`)."""
    rp = np.ascontiguousarray(row_ptrs, dtype=np.int32)
    ci = np.ascontiguousarray(col_inds, dtype=np.int32)
    v = np.ascontiguousarray(values, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    M = rp.size - 1
    out = np.zeros((M, B.shape[1]), dtype=np.float32)
    ref_lib().ref_spmm_naive(M, B.shape[0], B.shape[1], int(v.size), _p(v if v.size else np.zeros(1, np.float32)),
                             _p(rp), _p(ci if ci.size else np.zeros(1, np.int32)), _p(B), _p(out))
    return out


def dense_fp64(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """FP64 dense oracle C = A @ B."""
    return np.asarray(A, dtype=np.float64) @ np.asarray(B, dtype=np.float64)


def rel_err(x: np.ndarray, ref: np.ndarray) -> float:
    """||x - ref||_F / ||ref||_F (0 if both are zero)."""
    d = np.linalg.norm(np.asarray(x, np.float64) - np.asarray(ref, np.float64))
    r = np.linalg.norm(np.asarray(ref, np.float64))
    return float(d / r) if r > 0 else float(d)


def within_64eps(x: np.ndarray, y: np.ndarray) -> bool:
    """Elementwise |x - y| < 64 eps max(|x|, |y|) or < 64 eps (cpp_testbed/demo/SPMM_demo.cpp:106-112)."""
    x = np.asarray(x, np.float32)
    y = np.asarray(y, np.float32)
    eps = np.finfo(np.float32).eps
    d = np.abs(x - y)
    return bool(np.all((d < 64 * eps * np.maximum(np.abs(x), np.abs(y))) | (d < 64 * eps)))
