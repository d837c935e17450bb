"""Sparse-matrix files and the on-disk packed-weight format.

Readers (the reference's inputs):
* ``load_smtx`` -- the DLMC ``.smtx`` pattern format as sbench's torch op reads it
  (sbench/cpp/smtx_loader.cpp:5-45): line 1 ``rows, cols, nnz``; then rows + 1 row pointers;
  then, from the next line, nnz column indices.  Returns the pattern only.
* ``read_smtx`` -- the same file as the C++ testbed reads it (cpp_testbed/include/ParseSMTX.h:15-55):
  a CSR whose values are all 1.0.
* ``read_mtx`` -- Matrix Market ``coordinate`` files (cpp_testbed/include/ParseMatrixMarket.h:48-128):
  ``%`` comment lines skipped, 1-based (row, col, value) triplets, ``symmetric`` files mirrored
  off the diagonal; ``pattern`` files (no value column) read as 1.0.  Entries are ordered by
  (row, column) into CSR; a repeated coordinate is an error (the packer's column patterns need one
  value per position).  Missing files raise instead of exiting.

Packed format (``save_packed`` / ``load_packed``): a versioned file holding the reference's packed
arena bytes (SOPTile::pack_tile layout), the panel descriptors, the F16 scales, the mapping (id and
text) and the packing geometry (M_r, M_c, K_c, column offset, value type, suggested N_r).  Loading
uploads the arena and rebuilds the executor's layout from it on the device, checking every unit
(counts, column range, value count) -- a serving process restarts without the original weights.
"""
from __future__ import annotations

import json
import os
import struct
import zlib
from typing import Tuple

import numpy as np

Csr = Tuple[int, int, np.ndarray, np.ndarray, np.ndarray]  # rows, cols, row_ptrs, col_indices, values


def _tokens(line: str) -> list[str]:
    return line.replace(",", " ").split()


def load_smtx(path: str) -> Tuple[int, int, np.ndarray, np.ndarray]:
    """(rows, cols, row_ptrs int32[rows + 1], col_indices int32[nnz]) of a .smtx file."""
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    with open(path) as f:
        head = _tokens(f.readline())
        if len(head) < 3:
            raise ValueError(f"{path}: first line must hold rows, cols, nnz")
        rows, cols, nnz = (int(x) for x in head[:3])
        toks: list[str] = []
        while len(toks) < rows + 1:
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: {rows + 1} row pointers expected, {len(toks)} found")
            toks += line.split()
        row_ptrs = np.asarray(toks[: rows + 1], dtype=np.int64)
        cols_t: list[str] = []  # the rest of the row-pointer line is skipped, as the reference does
        while len(cols_t) < nnz:
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: {nnz} column indices expected, {len(cols_t)} found")
            cols_t += line.split()
    col_indices = np.asarray(cols_t[:nnz], dtype=np.int64)
    _check_csr(path, rows, cols, row_ptrs, col_indices)
    return rows, cols, row_ptrs.astype(np.int32), col_indices.astype(np.int32)


def read_smtx(path: str) -> Csr:
    """CSR of a .smtx file with every value 1.0 (ParseSMTX.h:52)."""
    rows, cols, rp, ci = load_smtx(path)
    return rows, cols, rp, ci, np.ones(ci.size, dtype=np.float32)


def write_smtx(path: str, rows: int, cols: int, row_ptrs, col_indices) -> None:
    with open(path, "w") as f:
        f.write(f"{rows}, {cols}, {len(col_indices)}\n")
        f.write(" ".join(str(int(x)) for x in row_ptrs) + "\n")
        f.write(" ".join(str(int(x)) for x in col_indices) + "\n")


def read_mtx(path: str) -> Csr:
    """CSR (values float32) of a Matrix Market coordinate file."""
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    with open(path) as f:
        header = f.readline().split()
        if len(header) < 4 or header[0].lower() != "%%matrixmarket":
            raise ValueError(f"{path}: not a Matrix Market file")
        if header[2].lower() != "coordinate":
            raise ValueError(f"{path}: only coordinate matrices are read")
        field = header[3].lower()
        sym = len(header) > 4 and header[4].lower() == "symmetric"
        if field not in ("real", "integer", "pattern", "double"):
            raise ValueError(f"{path}: field {field!r} is not read")
        line = f.readline()
        while line and line.lstrip().startswith("%"):
            line = f.readline()
        rows, cols, nnz = (int(x) for x in line.split()[:3])
        ncol = 2 if field == "pattern" else 3
        data = np.loadtxt(f, dtype=np.float64, comments="%", ndmin=2, max_rows=nnz) if nnz else np.zeros((0, ncol))
    if data.shape[0] != nnz or data.shape[1] < ncol:
        raise ValueError(f"{path}: {nnz} entries expected, {data.shape[0]} read")
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = data[:, 2] if ncol == 3 else np.ones(nnz)
    if sym:
        off = r != c
        r, c, v = np.concatenate([r, c[off]]), np.concatenate([c, r[off]]), np.concatenate([v, v[off]])
    if r.size and (r.min() < 0 or r.max() >= rows or c.min() < 0 or c.max() >= cols):
        raise ValueError(f"{path}: an entry lies outside the {rows} x {cols} matrix")
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    if r.size > 1 and np.any((r[1:] == r[:-1]) & (c[1:] == c[:-1])):
        raise ValueError(f"{path}: repeated coordinate")
    row_ptrs = np.zeros(rows + 1, dtype=np.int64)
    np.add.at(row_ptrs, r + 1, 1)
    row_ptrs = np.cumsum(row_ptrs)
    return rows, cols, row_ptrs.astype(np.int32), c.astype(np.int32), v.astype(np.float32)


def write_mtx(path: str, rows: int, cols: int, row_ptrs, col_indices, values, symmetric: bool = False) -> None:
    rp = np.asarray(row_ptrs)
    with open(path, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate real {'symmetric' if symmetric else 'general'}\n%\n")
        ent = [(i, int(col_indices[j]), float(values[j])) for i in range(rows) for j in range(rp[i], rp[i + 1])
               if not symmetric or int(col_indices[j]) <= i]
        f.write(f"{rows} {cols} {len(ent)}\n")
        for i, j, x in ent:
            f.write(f"{i + 1} {j + 1} {x!r}\n")


def csr_to_dense(rows: int, cols: int, row_ptrs, col_indices, values) -> np.ndarray:
    out = np.zeros((rows, cols), dtype=np.float32)
    rp = np.asarray(row_ptrs, dtype=np.int64)
    r = np.repeat(np.arange(rows), np.diff(rp))
    out[r, np.asarray(col_indices, dtype=np.int64)] = values
    return out


def _check_csr(path, rows, cols, rp, ci):
    if rp.size != rows + 1 or rp[0] != 0 or np.any(np.diff(rp) < 0) or rp[-1] != ci.size:
        raise ValueError(f"{path}: row pointers are not a CSR of {ci.size} entries")
    if ci.size and (ci.min() < 0 or ci.max() >= cols):
        raise ValueError(f"{path}: a column index lies outside [0, {cols})")


# ---------------------------------------------------------------------------- packed format
MAGIC = b"SPREGPK\0"
FORMAT_VERSION = 1


def save_packed(pm, path: str, nr: int = 0) -> None:
    """Write a PackedMatrix: magic, format version, a JSON header (geometry, mapping id and text,
    value type, sizes, CRC-32 of the payload, suggested N_r), then arena | descriptors | scales."""
    from . import _lib
    arena, descs, scales = pm.to_host()
    info = pm.info
    payload = [arena.tobytes(), descs.tobytes(), scales.tobytes() if scales is not None else b""]
    header = {
        "format": "spreg-packed", "version": FORMAT_VERSION,
        "rows": int(info["rows"]), "cols": int(info["cols"]), "mr": int(info["mr"]),
        "m_tile": int(info["m_tile"]), "k_tile": int(info["k_tile"]), "col_offset": int(info["col_offset"]),
        "value_dtype": {_lib.F32: "f32", _lib.BF16: "bf16", _lib.F16: "f16"}[int(info["value_dtype"])],
        "mapping_id": pm.mapping.mapping_id, "mapping_text": pm.mapping.text(),
        "nanokernels": [int(x) for x in pm.mapping.nanokernels],
        "num_units": int(info["num_units"]), "num_panels": int(info["num_panels"]),
        "arena_bytes": len(payload[0]), "descs_bytes": len(payload[1]), "scales_bytes": len(payload[2]),
        "nnz": int(info["nnz"]), "padding": int(info["padding"]), "nr": int(nr),
        "crc32": [zlib.crc32(b) for b in payload],
    }
    hb = json.dumps(header, sort_keys=True).encode()
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<II", FORMAT_VERSION, len(hb)))
        f.write(hb)
        for b in payload:
            f.write(b)


def read_packed_header(path: str) -> dict:
    with open(path, "rb") as f:
        return _read_header(f, path)


def _read_header(f, path):
    if f.read(8) != MAGIC:
        raise ValueError(f"{path}: not a packed-weight file")
    version, hlen = struct.unpack("<II", f.read(8))
    if version != FORMAT_VERSION:
        raise ValueError(f"{path}: format version {version}, this library reads {FORMAT_VERSION}")
    return json.loads(f.read(hlen).decode())


def load_packed(path: str, stream=None):
    """Read a file written by `save_packed` back into a device-resident PackedMatrix."""
    import ctypes as C
    from . import _lib
    from .mapping import Mapping
    from .packed import DESC_DTYPE, PackedMatrix
    with open(path, "rb") as f:
        h = _read_header(f, path)
        parts = [f.read(h["arena_bytes"]), f.read(h["descs_bytes"]), f.read(h["scales_bytes"])]
    for b, n, crc in zip(parts, (h["arena_bytes"], h["descs_bytes"], h["scales_bytes"]), h["crc32"]):
        if len(b) != n or zlib.crc32(b) != crc:
            raise ValueError(f"{path}: payload is truncated or corrupt")
    t = Mapping.from_text(h["mapping_text"])
    m = Mapping(t.mr, t.table, h.get("nanokernels"))
    if m.mapping_id != h["mapping_id"] or m.mr != h["mr"]:
        raise ValueError(f"{path}: mapping text does not match its id")
    vd = {"f32": _lib.F32, "bf16": _lib.BF16, "f16": _lib.F16}[h["value_dtype"]]
    arena = np.frombuffer(parts[0], dtype=np.uint8).copy()
    descs = np.frombuffer(parts[1], dtype=DESC_DTYPE).copy()
    scales = np.frombuffer(parts[2], dtype=np.float32).copy() if parts[2] else np.ones(1, dtype=np.float32)
    if descs.size != h["num_units"]:
        raise ValueError(f"{path}: {descs.size} descriptors for {h['num_units']} units")
    g = _lib.ArenaGeom(h["rows"], h["cols"], h["m_tile"], h["k_tile"], h["col_offset"], vd, 0)
    out = C.c_void_p()
    _lib.check(_lib.lib().spreg_pack_from_arena(
        m.handle, C.byref(g), arena.ctypes.data, arena.size, descs.ctypes.data, descs.size, scales.ctypes.data,
        scales.size if parts[2] else 0, C.byref(out), _lib.stream_handle(stream)))
    return PackedMatrix(out, m)
