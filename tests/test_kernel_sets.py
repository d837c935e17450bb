"""Nanokernel sets from a pattern histogram: coverage, budget, cost, packing and execution."""
import numpy as np
import pytest

from oracle import oracle as O
from spreg import synth
from spreg.kernel_sets import (KernelCost, executor_fast, executor_penalty, greedy_kernel_set, mapping_cost,
                               pattern_histogram)
from spreg.mapping import Mapping, popcount


@pytest.mark.parametrize("mr,budget", [(4, 6), (8, 19), (8, 8), (2, 2), (8, 1)])
def test_greedy_set_covers_every_pattern_within_budget(mr, budget):
    A = synth.row_skew(240, 300, 0.85, seed=mr + budget, std=1.0)
    h = pattern_histogram(A, mr)
    m = greedy_kernel_set(h, mr, budget, units=(240 // mr + 1) * 3)
    assert len(m.nanokernels) <= max(budget, 1)
    assert (2 ** mr - 1) in m.nanokernels
    for q in range(1, 2 ** mr):
        ks = m(q)
        assert len(ks) == 1 and ks[0] & q == q and ks[0] in m.nanokernels
    # the oracle packs it (the packer invariant holds) with the padding the mapping implies
    pk = O.Packed(O.Tables.of(m), A)
    assert pk.sizes["padding"] == int(sum(h[q] * m.padding_for(q) for q in range(1, 2 ** mr)))
    assert pk.sizes["nnz"] == int(np.count_nonzero(A))


def test_greedy_cost_not_above_identity_and_reference_sets():
    A = synth.row_skew(2048, 512, 0.9, seed=1)
    h = pattern_histogram(A, 8)
    units = 256 * 4
    g = greedy_kernel_set(h, 8, 19, units)
    c = mapping_cost(h, g, units)
    assert c <= mapping_cost(h, Mapping.identity(8), units)
    assert c <= mapping_cost(h, Mapping.load("400fa"), units) + 1e-9
    assert c <= mapping_cost(h, Mapping.load("747f9"), units) + 1e-9


def test_greedy_finds_planted_superset_kernels():
    """Panels whose columns hold sub-patterns of 0b0011 and 0b1100 only: with a budget of 3 the set
    is those two kernels plus the all-rows one."""
    g = np.random.default_rng(0)
    A = np.zeros((400, 600), dtype=np.float32)
    for p in range(100):
        for c in range(600):
            code = [0b01, 0b10, 0b11, 0b0100, 0b1000, 0b1100][g.integers(6)]
            if g.random() < 0.5:
                for r in range(4):
                    if (code >> r) & 1:
                        A[4 * p + r, c] = 1.0
    h = pattern_histogram(A, 4)
    m = greedy_kernel_set(h, 4, 3, units=100 * 5)
    assert set(m.nanokernels) == {0b0011, 0b1100, 0b1111}
    # a per-kernel cost large enough makes one all-rows kernel the cheapest set
    assert set(greedy_kernel_set(h, 4, 3, units=100 * 5, cost=KernelCost(n_check=500.0)).nanokernels) == {0b1111}


def test_histogram_numpy_matches_counting():
    A = synth.bernoulli(13, 21, 0.6, seed=4)
    h = pattern_histogram(A, 4)
    assert h.sum() == 4 * 21 and h.shape == (16,)
    codes = [sum(1 << r for r in range(4) if 4 * p + r < 13 and A[4 * p + r, c] != 0)
             for p in range(4) for c in range(21)]
    np.testing.assert_array_equal(h, np.bincount(codes, minlength=16))


def test_executor_penalty_marks_slow_kernels():
    assert executor_fast(4, 0b1011) and executor_fast(8, 0xFF) and not executor_fast(8, 0b111)
    assert executor_fast(6, 0b100) and not executor_fast(6, 0b101)
    pen = executor_penalty(8, 2.0)
    assert pen(0b111) == 2.0 and pen(0b1111) == 0.0
    m = greedy_kernel_set(pattern_histogram(synth.row_skew(512, 256, 0.9, seed=3), 8), 8, 19, 64 * 2,
                          penalty=executor_penalty(8, 100.0))
    assert all(executor_fast(8, k) for k in m.nanokernels)
    assert all(popcount(k) >= 1 for k in m.nanokernels)


def test_tile_penalty_keeps_the_b_tile_kernel_hot_set():
    """For K-tiled packs the B-tile executor has its own loop only for the single rows and the
    all-rows kernel: with the tile penalty the 70 %-sparse FFN weight keeps to those (without it
    the reference cost model adds six two- and three-row kernels)."""
    from spreg.kernel_sets import tile_hot
    assert tile_hot(4, 0b1000) and tile_hot(4, 0b1111) and not tile_hot(4, 0b0110) and tile_hot(2, 0b11)
    assert not tile_hot(8, 1)
    pen = executor_penalty(4, tile=True)
    assert pen(0b0110) == 0.5 and pen(0b0100) == 0.0 and executor_penalty(8, 2.0, tile=True)(0b111) == 2.0
    A = synth.row_skew(2048, 512, 0.7, seed=7070, sigma=0.5, std=0.02)
    h = pattern_histogram(A, 4)
    plain = greedy_kernel_set(h, 4, 15, 512 * 4, penalty=executor_penalty(4))
    tiled = greedy_kernel_set(h, 4, 15, 512 * 4, penalty=executor_penalty(4, tile=True))
    assert any(not tile_hot(4, k) for k in plain.nanokernels)
    assert all(tile_hot(4, k) for k in tiled.nanokernels)


@pytest.mark.gpu
def test_greedy_set_packs_and_executes_bit_exact(cuda):
    import torch
    from spreg.packed import PackedMatrix
    A = synth.row_skew(300, 400, 0.9, seed=7, std=1.0)
    At = torch.from_numpy(A).cuda()
    np.testing.assert_array_equal(pattern_histogram(At, 8), pattern_histogram(A, 8))
    m = greedy_kernel_set(pattern_histogram(At, 8), 8, 12, units=38 * 4, penalty=executor_penalty(8))
    pm = PackedMatrix.from_dense(At, m)
    ref = O.Packed(O.Tables.of(m), A)
    arena, descs, _ = pm.to_host()
    assert np.array_equal(arena, ref.arena) and np.array_equal(descs, ref.descs)
    B = synth.dense(400, 96, seed=8)
    got = pm.execute(torch.from_numpy(B).cuda()).cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.execute(B).view(np.uint32))
