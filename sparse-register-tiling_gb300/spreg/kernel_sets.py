"""Nanokernel sets chosen from a matrix's pattern histogram (set cover, greedy form).

The reference chooses a panel height's nanokernel set by a weighted set cover solved as an ILP
(sbench/ilp_pad/nano_solver.py: cost model :77-115, universe :174-221, ILP :226-279; the solver,
MOSEK, is not available here).  In its MERGE_ONLY form every pattern q runs as exactly one
nanokernel k with k a superset of q (the rows of k missing from q are padding), and a nanokernel
costs

    nCheck + F_k * (nBase + nCnz * popcount(k))

with F_k the expected number of columns per K_c-wide tile of a panel whose pattern runs as k.
The total over the chosen set is minimised with at most `budget` nanokernels.

`greedy_kernel_set` solves that model by agglomeration.  It starts from one nanokernel per pattern
present, then repeatedly merges the pair whose union increases the cost least (decreases it most)
until the budget holds and no merge lowers the cost.  Patterns absent from the histogram are mapped
to their cheapest superset in the set, which always includes the all-rows nanokernel.  The result
is a `Mapping` the packer and executors take like any mapping file.

`pattern_histogram` counts (panel, column) patterns on the device when A is a CUDA tensor.
"""
from __future__ import annotations

import dataclasses
from typing import Callable, Optional

import numpy as np

from .mapping import Mapping, popcount


@dataclasses.dataclass(frozen=True)
class KernelCost:
    """Coefficients of the set-cover cost; defaults are the reference's (nano_solver.py:77-80)."""
    n_check: float = 2.0
    n_base: float = 1.15
    n_cnz: float = 0.2
    k_c: int = 128


# Nanokernels the executor runs with a specialised FMA block (exec_kernel.cuh, fast_pattern): every
# pattern for M_r <= 4, single rows for M_r = 6, and for M_r = 8 the single rows plus the nanokernels
# of the reference's "orig" / "alt" sets.  Others take a slower path (two 16-way switches per entry).
FAST_MR8 = frozenset([1, 2, 4, 8, 16, 32, 64, 128, 15, 60, 85, 170, 195, 240, 63, 207, 243, 252, 255])


def executor_fast(mr: int, k: int) -> bool:
    if mr <= 4:
        return True
    if mr == 6:
        return k & (k - 1) == 0
    return k in FAST_MR8


def tile_hot(mr: int, k: int) -> bool:
    """Nanokernels with their own group loop in the shared-memory B-tile executor (M_r 2 and 4):
    the single rows and the all-rows kernel.  Other patterns dispatch per step there."""
    return mr in (2, 4) and (k & (k - 1) == 0 or k == (1 << mr) - 1)


def executor_penalty(mr: int, per_column: float = 1.0, tile: bool = False,
                     tile_per_column: float = 0.5) -> Callable[[int], float]:
    """Extra per-column cost of nanokernels without a specialised FMA block in this executor; with
    `tile` (K-tiled packs, which the B-tile executor runs), also of M_r 2 / 4 nanokernels without
    their own group loop there.  tile_per_column = 0.5 (from 0.25 up the same sets result) measured
    on GB300, 2048 x 512 at 70 % sparsity: 21.2 -> 18.4 us (FP32), 25.2 -> 17.7 us (BF16) per
    SpMM; at 98 %, BF16 6.9 -> 4.5 us."""
    def pen(k: int) -> float:
        p = 0.0 if executor_fast(mr, k) else per_column
        if tile and mr in (2, 4) and not tile_hot(mr, k):
            p += tile_per_column
        return p
    return pen


def pattern_histogram(A, mr: int) -> np.ndarray:
    """Number of (row panel, column) positions of each pattern code 0 .. 2^mr - 1.

    A: dense matrix (numpy, or a CUDA tensor: counted there with one bincount); its zeros are
    the pruned entries; the last panel is zero-padded to mr rows."""
    try:
        import torch
        is_t = isinstance(A, torch.Tensor)
    except ImportError:  # pragma: no cover - torch is always present here
        is_t = False
    if is_t:
        import torch
        m, k = A.shape
        P = (m + mr - 1) // mr
        mask = torch.zeros((P * mr, k), dtype=torch.int32, device=A.device)
        mask[:m] = (A != 0).to(torch.int32)
        w = (1 << torch.arange(mr, device=A.device, dtype=torch.int32)).view(1, mr, 1)
        codes = (mask.view(P, mr, k) * w).sum(dim=1)
        return torch.bincount(codes.flatten(), minlength=2 ** mr).cpu().numpy().astype(np.int64)
    from .autotune import panel_codes
    codes = panel_codes(np.asarray(A) != 0, mr)
    return np.bincount(codes.ravel(), minlength=2 ** mr).astype(np.int64)


def set_cost(kernels: dict, cost: KernelCost, penalty: Optional[Callable[[int], float]] = None) -> float:
    """Cost of {kernel: F_k}."""
    tot = 0.0
    for k, F in kernels.items():
        per = cost.n_base + cost.n_cnz * popcount(k) + (penalty(k) if penalty else 0.0)
        tot += cost.n_check + F * per
    return tot


def greedy_kernel_set(hist: np.ndarray, mr: int, budget: int, units: int, cost: KernelCost = KernelCost(),
                      penalty: Optional[Callable[[int], float]] = None) -> Mapping:
    """Mapping for panel height mr with at most `budget` nanokernels (>= 1).

    hist: pattern counts (`pattern_histogram`); units: (panel, K_c tile) units they were counted
    over, so that F_k = columns per unit; penalty(k): extra per-column cost of running nanokernel k
    (e.g. for kernels without a specialised FMA block)."""
    full = 2 ** mr - 1
    if budget < 1:
        raise ValueError("budget must be >= 1")
    if hist.shape[0] != 2 ** mr:
        raise ValueError(f"histogram must have {2 ** mr} entries")
    per_unit = np.asarray(hist, dtype=np.float64) / max(units, 1)
    # current nanokernels: kernel -> (F, member patterns)
    ks = {q: [float(per_unit[q]), {q}] for q in range(1, full + 1) if hist[q] > 0}
    keep_full = full not in ks
    slots = budget - (1 if keep_full else 0)
    if slots < 1:
        ks = {}
    pc = np.array([popcount(x) for x in range(full + 1)], dtype=np.float64)
    pen = np.array([penalty(x) if penalty else 0.0 for x in range(full + 1)])

    while len(ks) > 1:
        keys = np.array(list(ks.keys()), dtype=np.int64)
        F = np.array([ks[k][0] for k in keys])
        U = keys[:, None] | keys[None, :]
        FF = F[:, None] + F[None, :]
        base = cost.n_check + F * (cost.n_base + cost.n_cnz * pc[keys] + pen[keys])
        merged = cost.n_check + FF * (cost.n_base + cost.n_cnz * pc[U] + pen[U])
        delta = merged - base[:, None] - base[None, :]
        # a union equal to a third current kernel also absorbs that kernel and its cost
        n = len(keys)
        pos = np.full(full + 1, -1, dtype=np.int64)
        pos[keys] = np.arange(n)
        C = pos[U]
        ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        third = (C >= 0) & (C != ii) & (C != jj)
        if third.any():
            Cc = np.where(third, C, 0)
            absorbed = cost.n_check + (FF + F[Cc]) * (cost.n_base + cost.n_cnz * pc[U] + pen[U])
            delta = np.where(third, absorbed - base[:, None] - base[None, :] - base[Cc], delta)
        np.fill_diagonal(delta, np.inf)
        i, j = np.unravel_index(np.argmin(delta), delta.shape)
        if len(ks) <= max(slots, 0) and delta[i, j] >= 0:
            break
        a, b = int(keys[i]), int(keys[j])
        u = a | b
        Fa, Ma = ks.pop(a)
        Fb, Mb = ks.pop(b)
        if u in ks:
            Fc, Mc = ks.pop(u)
            ks[u] = [Fa + Fb + Fc, Ma | Mb | Mc]
        else:
            ks[u] = [Fa + Fb, Ma | Mb]
    if len(ks) > max(slots, 0):  # budget 1 with patterns present: everything runs as the full kernel
        ks = {}
    kernels = set(ks) | {full}
    table = {}
    for k, (_, members) in ks.items():
        for q in members:
            table[q] = [k]
    for q in range(1, full + 1):
        if q not in table:
            sup = [k for k in kernels if k & q == q]
            table[q] = [min(sup, key=lambda k: (pc[k] + pen[k], k))]
    return Mapping(mr, table, sorted(kernels))


def mapping_cost(hist: np.ndarray, m: Mapping, units: int, cost: KernelCost = KernelCost(),
                 penalty: Optional[Callable[[int], float]] = None) -> float:
    """The set-cover cost of an existing mapping on a histogram (list mappings: every code counts)."""
    per_unit = np.asarray(hist, dtype=np.float64) / max(units, 1)
    F: dict = {k: 0.0 for k in m.nanokernels}
    for q in range(1, 2 ** m.mr):
        for k in m(q):
            F[k] = F.get(k, 0.0) + per_unit[q]
    return set_cost(F, cost, penalty)
