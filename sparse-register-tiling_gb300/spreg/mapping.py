"""Pattern -> nanokernel mappings (the reference's mapping files and `pattern_mapping` callables).

A mapping file (sbench/SOP/mapping.py:5-19) is ``M_r`` on the first line, then one line
``<pattern>: [<nanokernel pattern>, ...]`` for every pattern 1 .. 2^M_r - 1.  Its id is the
last five hex digits of the md5 of ``str({pattern: list, ...})``; ``Mapping.mapping_id``
recomputes it.  ``load_mapping`` follows sbench/SOP/sop_bench.py:72-95 (a defaultdict of
lists: patterns absent from the file, and pattern 0, map to nothing).
"""
from __future__ import annotations

import ast
import ctypes as C
import hashlib
import os
from typing import Callable, Iterable, Sequence

import numpy as np

from . import _lib

MAPPING_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mappings")

# Named nanokernel sets of the reference's method grammar (tools/paper/configs.py:84-87).
# "da01e" (M_r = 4 "orig") is named there but its file is not part of the reference.
NAMED_MAPPINGS = {4: {"identity": "61fee", "orig": "da01e"}, 8: {"orig": "400fa", "alt": "747f9"}}


def popcount(x: int) -> int:
    return bin(int(x)).count("1")


def nkern_id_order(patterns: Iterable[int]) -> list[int]:
    """Nanokernel id order of a set: by (popcount, value)."""
    return sorted(set(int(p) for p in patterns if int(p) != 0), key=lambda p: (popcount(p), p))


class Mapping:
    """A pattern -> list-of-nanokernel-patterns table for panel height ``mr``."""

    def __init__(self, mr: int, table: dict[int, list[int]], nanokernels: Sequence[int] | None = None):
        if mr not in (2, 4, 6, 8):
            raise ValueError(f"M_r must be 2, 4, 6 or 8, got {mr}")
        self.mr = mr
        self.table = {int(p): [int(c) for c in v] for p, v in table.items()}
        listed = {c for v in self.table.values() for c in v if c}
        self.nanokernels = nkern_id_order(nanokernels if nanokernels is not None else listed)
        self._handle = None

    # ---------------------------------------------------------------- constructors
    @classmethod
    def identity(cls, mr: int) -> "Mapping":
        return cls(mr, {p: [p] for p in range(1, 2 ** mr)})

    @classmethod
    def from_callable(cls, mr: int, fn: Callable[[int], int | list[int]],
                      nanokernels: Sequence[int] | None = None) -> "Mapping":
        """Evaluate a reference-style ``pattern_mapping`` (int or list result, sop_driver.py:55-62)."""
        table = {}
        for p in range(0, 2 ** mr):
            r = fn(p)
            table[p] = [int(r)] if isinstance(r, (int, np.integer)) else [int(c) for c in r]
        return cls(mr, table, nanokernels)

    @classmethod
    def from_text(cls, text: str) -> "Mapping":
        lines = [ln for ln in text.splitlines() if ln.strip()]
        mr = int(lines[0])
        table = {}
        for ln in lines[1:]:
            k, v = ln.split(":", 1)
            table[int(k)] = [int(c) for c in ast.literal_eval(v.strip())]
        return cls(mr, table)

    @classmethod
    def load(cls, mapping_id: str, dirs: Sequence[str] | None = None) -> "Mapping":
        """read_pattern_mapping(mapping_id, dirs) (count_nkerns.cpp:54-55): first mapping_<id>.txt found."""
        for d in list(dirs or []) + [MAPPING_DIR]:
            path = os.path.join(d, f"mapping_{mapping_id}.txt")
            if os.path.exists(path):
                with open(path) as f:
                    return cls.from_text(f.read())
        raise FileNotFoundError(f"mapping {mapping_id!r} not found in {list(dirs or []) + [MAPPING_DIR]}")

    @classmethod
    def named(cls, mr: int, name: str) -> "Mapping":
        if name == "identity":
            return cls.identity(mr)
        return cls.load(NAMED_MAPPINGS.get(mr, {}).get(name, name))

    # ---------------------------------------------------------------- reference behaviour
    def __call__(self, pattern: int) -> list[int]:
        return list(self.table.get(int(pattern), []))

    def text(self) -> str:
        """File text in the format of save_mapping (mapping.py:16-18)."""
        out = [f"{self.mr}"]
        for p in range(1, 2 ** self.mr):
            out.append(f"{p}: {list(self.table.get(p, []))}")
        return "\n".join(out) + "\n"

    @property
    def mapping_id(self) -> str:
        """md5(str({pattern: list}))[-5:] (mapping.py:9)."""
        d = {p: list(self.table.get(p, [])) for p in range(1, 2 ** self.mr)}
        return hashlib.md5(str(d).encode("utf-8")).hexdigest()[-5:]

    def save(self, directory: str) -> str:
        os.makedirs(directory, exist_ok=True)
        mid = self.mapping_id
        with open(os.path.join(directory, f"mapping_{mid}.txt"), "w") as f:
            f.write(self.text())
        return mid

    def padding_for(self, pattern: int) -> int:
        """Zeros emitted for a column of this pattern: popcount(code & ~pattern) summed over its codes."""
        return sum(popcount(c & ~pattern) for c in self(pattern))

    def offsets_codes(self) -> tuple[np.ndarray, np.ndarray]:
        offs = [0]
        codes: list[int] = []
        for p in range(2 ** self.mr):
            codes += self.table.get(p, [])
            offs.append(len(codes))
        return np.asarray(offs, dtype=np.int32), np.asarray(codes if codes else [0], dtype=np.int32)

    # ---------------------------------------------------------------- C handle
    @property
    def handle(self):
        """spreg_mapping* (host-only object; created without touching the GPU)."""
        if self._handle is None:
            L = _lib.lib()
            offs, codes = self.offsets_codes()
            nks = np.asarray(self.nanokernels if self.nanokernels else [0], dtype=np.int32)
            h = C.c_void_p()
            _lib.check(L.spreg_mapping_create(self.mr, offs.ctypes.data, codes.ctypes.data, nks.ctypes.data,
                                              len(self.nanokernels), C.byref(h)))
            self._handle = h
        return self._handle

    def num_nkern(self) -> int:
        return int(_lib.lib().spreg_mapping_num_nkern(self.handle))

    def nkern_patterns(self) -> list[int]:
        n = self.num_nkern()
        out = np.zeros(max(n, 1), dtype=np.int32)
        _lib.check(_lib.lib().spreg_mapping_nkern_patterns(self.handle, out.ctypes.data))
        return [int(x) for x in out[:n]]

    def encode(self, pattern: int) -> int:
        """MicroKernel::encode_nkern_pattern: id, ZERO_PATTERN_ID for 0, -1 if not a nanokernel."""
        return int(_lib.lib().spreg_mapping_encode(self.handle, int(pattern)))

    def __del__(self):
        try:
            if self._handle is not None:
                _lib.lib().spreg_mapping_destroy(self._handle)
        except Exception:
            pass
