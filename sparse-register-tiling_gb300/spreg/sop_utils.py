"""Helpers of the reference's Python side around the packer, under the reference's names:
sbench/SOP/sop_utils.py (Acc, Codelet, popcount, pattern_code, get_codelets_from_panel,
tile_matrix), sbench/SOP/distribution.py (compute_histogram) and sbench/SOP/mapping.py
(save_mapping).  Reference scripts switch their import and keep their calls.

The per-element Python loops of the reference become array operations; the results are the same
(tests/test_sop_utils.py checks them against direct restatements of the loops).
"""
from __future__ import annotations

import hashlib
import os
from dataclasses import dataclass
from typing import Callable, List

import numpy as np

# pattern_code: bit i set iff vec[i] != 0 (distribution.py:10-15); sop_utils.py:25-30 casts to int
# instead, which agrees on the 0/1 masks the reference calls it with.
from .sop_driver import Acc, pattern_code  # noqa: F401  (re-exported under the reference's module)

PKG_DIR = os.path.dirname(os.path.abspath(__file__))


@dataclass
class Codelet:
    """sop_utils.py:12-14: `cols` columns of a panel holding `nnz` nonzeros each."""
    nnz: int = 4
    cols: int = 4


class CodeletDict(dict):
    """sop_utils.py:17-20: a missing popcount key starts a Codelet with no columns."""

    def __missing__(self, key):
        ret = self[key] = Codelet(nnz=key, cols=0)
        return ret


def popcount(x: int) -> int:
    return bin(int(x)).count("1")


def _as_numpy(t) -> np.ndarray:
    return t.detach().cpu().numpy() if hasattr(t, "detach") else np.asarray(t)


def get_codelets_from_panel(panel) -> List[Codelet]:
    """sop_utils.py:33-40: for each column of the panel (M_r x K) with nonzeros, count it under its
    nonzero count; Codelets in order of first appearance."""
    nz = (_as_numpy(panel) != 0).sum(axis=0)
    codelets = CodeletDict()
    for c in nz:
        if c == 0:
            continue
        codelets[int(c)].cols += 1
    return list(codelets.values())


def tile_matrix(mtx, tile_shape):
    """sop_utils.py:43-46: [(i, j, tile)] over row blocks of tile_shape[0] and column blocks of
    tile_shape[1] (torch.split semantics: the last block of each dimension may be smaller)."""
    import torch
    return [(i, j, tile)
            for i, x in enumerate(torch.split(mtx, tile_shape[0], 0))
            for j, tile in enumerate(torch.split(x, tile_shape[1], 1))]


def compute_histogram(M_r: int, matrix) -> np.ndarray:
    """distribution.py:18-26: the frequency of each M_r-row pattern code over the panels' columns,
    normalised by cols x (rows // M_r).  A last panel of fewer than M_r rows counts with its rows."""
    A = _as_numpy(matrix) != 0
    rows, cols = A.shape
    counts = np.zeros(2 ** M_r, dtype=np.int64)
    for i in range(0, rows, M_r):
        blk = A[i:i + M_r]
        w = (1 << np.arange(blk.shape[0], dtype=np.int64))[:, None]
        codes = (blk.astype(np.int64) * w).sum(axis=0)
        counts += np.bincount(codes, minlength=2 ** M_r)
    return counts / (cols * rows // M_r)


def save_mapping(M_r: int, mapping: Callable[[int], object], subdir: str = "mappings", root: str = PKG_DIR) -> str:
    """mapping.py:5-20: evaluate `mapping` on every pattern 1 .. 2^M_r - 1, name the file by the last
    5 hex digits of md5(str({pattern: mapping(pattern)})) and write `M_r` then `pattern: [codes]`
    lines into root/subdir/mapping_<id>.txt; returns the id."""
    mapping_dict = {i: mapping(i) for i in range(1, 2 ** M_r)}
    mid = hashlib.md5(str(mapping_dict).encode("utf-8")).hexdigest()[-5:]
    os.makedirs(os.path.join(root, subdir), exist_ok=True)
    with open(os.path.join(root, subdir, f"mapping_{mid}.txt"), "w+") as f:
        f.write(f"{M_r}\n")
        for k, v in mapping_dict.items():
            f.write(f"{k}: {list(v)}\n")  # an int result raises here, as in the reference
    return mid
