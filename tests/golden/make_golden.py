"""Generate tests/golden/*.npz from the reference's own code (run in a container that has the
reference checkout; the fixtures are committed so machines without it can still use them).

Each fixture holds a seeded sparse A (CSR), a dense B and C = A . B computed by the reference's
cpp_testbed/src/spmm/baselines/spmm_naive.cpp (compiled unchanged by `make -C oracle ref`).
One fixture slices a matrix the reference ships (bundled_datasets/random/random_90_768_768.mtx),
read with numpy (values as stored), so the golden input is the reference's own data.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "sparse-register-tiling_gb300"))

from oracle import oracle as O  # noqa: E402
from spreg import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
MTX = os.path.join(O.REFERENCE_ROOT, "bundled_datasets/random/random_90_768_768.mtx")


def read_mtx_rows(path: str, row_lo: int, row_hi: int):
    """Rows [row_lo, row_hi) of a MatrixMarket coordinate real general file as a dense array."""
    with open(path) as f:
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        m, k, _ = (int(x) for x in line.split())
        data = np.loadtxt(f, dtype=np.float64, ndmin=2)
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = data[:, 2].astype(np.float32)
    sel = (r >= row_lo) & (r < row_hi)
    A = np.zeros((row_hi - row_lo, k), dtype=np.float32)
    A[r[sel] - row_lo, c[sel]] = v[sel]
    return A


def cases():
    yield "bern80_64x96_n40", synth.bernoulli(64, 96, 0.8, seed=11), synth.dense(96, 40, seed=12)
    yield "skew90_130x200_n72", synth.row_skew(130, 200, 0.9, seed=13, std=1.0), synth.dense(200, 72, seed=14)
    yield "dense_30x17_n9", synth.bernoulli(30, 17, 0.0, seed=15), synth.dense(17, 9, seed=16)
    if os.path.exists(MTX):
        yield "mtx_random90_rows0_96_n16", read_mtx_rows(MTX, 0, 96), synth.dense(768, 16, seed=17)


def main() -> int:
    O.build(with_reference=True)
    if not O.has_ref():
        print("reference not available; fixtures not regenerated", file=sys.stderr)
        return 1
    for name, A, B in cases():
        rp, ci, v = synth.to_csr(A)
        Cn = O.ref_naive(rp, ci, v, B)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), shape=np.asarray(A.shape), row_ptrs=rp,
                            col_inds=ci, values=v, B=B, C_ref_naive=Cn)
        print(name, A.shape, B.shape, int(v.size))
    return 0


if __name__ == "__main__":
    sys.exit(main())
