"""Pins the CPU oracle (oracle/spreg_oracle.c) against the reference: mapping-file ids, the
reference's known-answer tests, the packer invariant, a hand-derived pack_panel case, and
outputs of the reference's own spmm_naive (live when the reference is present, else the
committed golden fixtures)."""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from spreg import synth
from spreg.mapping import MAPPING_DIR, Mapping, nkern_id_order, popcount

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def all_mapping_ids():
    return sorted(os.path.basename(p)[8:13] for p in glob.glob(os.path.join(MAPPING_DIR, "mapping_*.txt")))


@pytest.mark.parametrize("mid", all_mapping_ids())
def test_mapping_file_id_is_content_md5(mid):
    m = Mapping.load(mid)
    assert m.mapping_id == mid
    assert Mapping.from_text(m.text()).table == {p: v for p, v in m.table.items()}


def test_mapping_fixtures_cover_and_do_not_overlap():
    for mid in all_mapping_ids():
        m = Mapping.load(mid)
        for p in range(1, 2 ** m.mr):
            union, overlap = 0, 0
            for c in m(p):
                overlap |= union & c
                union |= c
            assert overlap == 0 and union & p == p, (mid, p)


def test_identity_ids_sorted_by_popcount_then_value():
    t = O.Tables.of(Mapping.identity(4))
    assert list(t.id_to_pattern[:15]) == [1, 2, 4, 8, 3, 5, 6, 9, 10, 12, 7, 11, 13, 14, 15]
    assert t.code_to_id[0] == O.ZERO
    m8 = Mapping.load("400fa")
    t8 = O.Tables.of(m8)
    assert list(t8.id_to_pattern[: t8.num_nkern]) == nkern_id_order(m8.nanokernels)
    assert t8.num_nkern == 19


def _stable_sort_reference(enc):
    # comparator of template:76-78 through Python's stable sort
    key = [(e == O.ZERO, e) for e in enc]
    return sorted(range(len(enc)), key=lambda i: key[i])


@pytest.mark.parametrize("seed", range(5))
def test_sort_and_encode_is_stable_with_zero_last(seed):
    g = np.random.default_rng(seed)
    m = Mapping.identity(4)
    t = O.Tables.of(m)
    codes = g.integers(0, 16, size=int(g.integers(1, 300))).astype(np.int32)
    enc, order = O.sort_and_encode(t, codes)
    raw = [int(t.code_to_id[c]) for c in codes]
    expect_order = _stable_sort_reference(raw)
    assert list(order) == expect_order
    assert list(enc) == [raw[i] for i in expect_order]


def test_permute_inplace_equals_gather():
    g = np.random.default_rng(7)
    for n in (1, 2, 17, 256):
        order = g.permutation(n).astype(np.int32)
        v = g.integers(-1000, 1000, size=n).astype(np.int32)
        assert np.array_equal(O.permute_inplace(order, v), v[order])


def test_pack_panel_hand_example():
    # Mr = 4 panel, 5 columns; patterns [0101, 0000, 0001, 1111, 0101] (bit r = row r)
    dense = np.zeros((5, 4), np.float32)
    dense[0, [0, 2]] = [1.0, 2.0]
    dense[2, 0] = 3.0
    dense[3, :] = [4.0, 5.0, 6.0, 7.0]
    dense[4, [0, 2]] = [8.0, 9.0]
    t = O.Tables.of(Mapping.identity(4))
    codes = [0b0101, 0, 0b0001, 0b1111, 0b0101]
    r = O.pack_panel(t, 100, codes, list(range(5)), dense)
    counts = np.zeros(15, np.int32)
    counts[0], counts[5], counts[14] = 1, 2, 1   # ids: 0001 -> 0, 0101 -> 5, 1111 -> 14
    assert np.array_equal(r["counts"], counts)
    assert list(r["cols"]) == [102, 100, 104, 103]
    assert list(r["values"]) == [3.0, 1.0, 2.0, 8.0, 9.0, 4.0, 5.0, 6.0, 7.0]
    assert r["padding"] == 0


@pytest.mark.parametrize("mid", ["400fa", "747f9", "33960", "75f82", "dcfff"])
def test_pack_panel_padding_and_invariant(mid):
    m = Mapping.load(mid)
    t = O.Tables.of(m)
    g = np.random.default_rng(3)
    K = 300
    dense = np.where(g.random((K, m.mr)) < 0.3, g.standard_normal((K, m.mr)), 0).astype(np.float32)
    pats = [(int(sum(1 << r for r in range(m.mr) if dense[c, r] != 0))) for c in range(K)]
    codes, cols = [], []
    for c, p in enumerate(pats):
        for k in m(p):
            codes.append(k)
            cols.append(c)
    r = O.pack_panel(t, 0, codes, cols, dense)
    assert r["padding"] == sum(m.padding_for(p) for p in pats)
    assert r["values"].size == r["padding"] + np.count_nonzero(dense)   # template:214
    assert int(r["counts"].sum()) == r["cols"].size


def test_pack_panel_rejects_uncovered_pattern():
    t = O.Tables.of(Mapping.identity(4))
    dense = np.ones((1, 4), np.float32)
    with pytest.raises(ValueError):
        O.pack_panel(t, 0, [0b0011], [0], dense)   # rows 2,3 nonzero but not emitted


@pytest.mark.parametrize("mid,mr", [("identity", 4), ("400fa", 8), ("747f9", 8), ("33960", 8), ("001e3", 6),
                                    ("4af51", 2)])
def test_known_answer_ones(mid, mr):
    """A in {0,1}, B = ones -> C[i, j] = nnz(row i) exactly (sbench/SOP/sop_bench.py:49-50,187,203)."""
    m = Mapping.identity(mr) if mid == "identity" else Mapping.load(mid)
    A = (synth.bernoulli(37, 150, 0.7, seed=5) != 0).astype(np.float32)
    pk = O.Packed(O.Tables.of(m), A)
    C = pk.execute(np.ones((150, 40), np.float32))
    assert np.array_equal(C, np.repeat(A.sum(1, keepdims=True), 40, axis=1))


def test_arena_layout_and_required_storage():
    m = Mapping.load("400fa")
    t = O.Tables.of(m)
    A = synth.row_skew(77, 260, 0.85, seed=9)
    pk = O.Packed(t, A)
    d = pk.descs
    assert np.all(d["values_off"] % 64 == 0) and np.all(d["cols_off"] % 64 == 0) and np.all(d["counts_off"] % 64 == 0)
    a64 = lambda x: (x + 63) // 64 * 64  # noqa: E731
    assert np.array_equal(d["cols_off"], d["values_off"] + a64(4 * d["num_values"].astype(np.int64)))
    assert np.array_equal(d["counts_off"], d["cols_off"] + a64(4 * d["num_cols"].astype(np.int64)))
    ends = d["counts_off"] + a64(4 * t.num_nkern)
    assert np.array_equal(d["values_off"][1:], ends[:-1]) and ends[-1] == pk.sizes["arena_bytes"]
    req = int((4 * d["num_values"].astype(np.int64) + 4 * d["num_cols"] + 4 * t.num_nkern + 192).sum())
    assert req == pk.sizes["required_storage"]
    assert pk.sizes["num_values"] == pk.sizes["nnz"] + pk.sizes["padding"]


def _golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


@pytest.mark.parametrize("path", _golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
@pytest.mark.parametrize("mid,mr", [("identity", 4), ("400fa", 8), ("001e3", 6)])
def test_oracle_matches_reference_spmm_naive_golden(path, mid, mr):
    z = np.load(path)
    M, K = (int(x) for x in z["shape"])
    A = np.zeros((M, K), np.float32)
    rows = np.repeat(np.arange(M), np.diff(z["row_ptrs"]))
    A[rows, z["col_inds"]] = z["values"]
    m = Mapping.identity(mr) if mid == "identity" else Mapping.load(mid)
    C = O.Packed(O.Tables.of(m), A).execute(z["B"])
    assert O.rel_err(C, z["C_ref_naive"]) <= 1e-5
    assert O.rel_err(C, O.dense_fp64(A, z["B"])) <= 1e-5


@pytest.mark.skipif(not O.has_ref(), reason="reference spmm_naive not built (no reference checkout)")
@pytest.mark.parametrize("seed", range(3))
def test_oracle_matches_reference_spmm_naive_live(seed):
    A = synth.row_skew(96, 333, 0.8, seed=seed, std=1.0)
    B = synth.dense(333, 65, seed=seed + 10)
    rp, ci, v = synth.to_csr(A)
    Cn = O.ref_naive(rp, ci, v, B)
    C = O.Packed(O.Tables.of(Mapping.identity(4)), A).execute(B)
    assert O.rel_err(C, Cn) <= 1e-5
    assert O.within_64eps(O.csr_spmm(rp, ci, v, B), Cn) or O.rel_err(O.csr_spmm(rp, ci, v, B), Cn) <= 1e-6


def test_conversions_match_torch():
    import torch
    g = np.random.default_rng(0)
    x = np.concatenate([g.standard_normal(20000).astype(np.float32) * 10.0 ** g.integers(-9, 6, 20000),
                        np.array([0.0, -0.0, 65504.0, 65519.0, 65520.0, 1e-8, 2.0 ** -24, 2.0 ** -25, 3 * 2.0 ** -26,
                                  1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, np.inf, -np.inf, 3.4e38], np.float32)])
    t = torch.from_numpy(x)
    assert np.array_equal(O.f32_to_f16(x), t.to(torch.float16).view(torch.int16).numpy().view(np.uint16))
    assert np.array_equal(O.f32_to_bf16(x), t.to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16))
    assert np.array_equal(O.f16_to_f32(O.f32_to_f16(x)), t.to(torch.float16).float().numpy())


@pytest.mark.parametrize("m_tile,k_tile", [(8, 64), (16, 256), (4, 7), (0, 100)])
def test_tiled_packing(m_tile, k_tile):
    """M_c x K_c tiles (count_nkerns.cpp:58-128): same product, K tiles accumulate (load_c)."""
    A = synth.row_skew(50, 230, 0.9, seed=4, std=1.0)
    A[:, 64:128] = 0.0   # an all-zero K tile -> EMPTY_TILE units
    B = synth.dense(230, 33, seed=8)
    t = O.Tables.of(Mapping.identity(4))
    full = O.Packed(t, A).execute(B)
    tiled = O.Packed(t, A, m_tile=m_tile, k_tile=k_tile)
    C = tiled.execute(B)
    assert O.rel_err(C, full) <= 1e-6
    A01 = (A != 0).astype(np.float32)
    ones = O.Packed(t, A01, m_tile=m_tile, k_tile=k_tile).execute(np.ones((230, 5), np.float32))
    assert np.array_equal(ones, np.repeat(A01.sum(1, keepdims=True), 5, 1))
    if k_tile == 64:
        assert tiled.sizes["empty_units"] > 0


@pytest.mark.parametrize("shape", [(0, 5), (5, 0), (1, 1), (3, 9), (9, 3)])
def test_edge_shapes(shape):
    A = synth.bernoulli(*shape, 0.5, seed=1)
    B = synth.dense(shape[1], 7, seed=2)
    pk = O.Packed(O.Tables.of(Mapping.identity(4)), A)
    C = pk.execute(B)
    assert C.shape == (shape[0], 7)
    assert O.rel_err(C, O.dense_fp64(A, B)) <= 1e-6


def test_popcount_helper():
    assert [popcount(x) for x in (0, 1, 255, 0b1010)] == [0, 1, 8, 2]


@pytest.mark.parametrize("mapping_id,mr", [("61fee", 4), ("400fa", 8), (None, 2), (None, 6)])
@pytest.mark.parametrize("k_tile,load_c,relu", [(0, False, False), (128, True, True), (64, False, True)])
def test_simd_cpu_executor_is_bit_identical_to_the_checker(mapping_id, mr, k_tile, load_c, relu):
    """The timed CPU baseline (SIMD, per-pattern FMA blocks) gives the checker's bits."""
    from spreg import synth
    from spreg.mapping import Mapping
    m = Mapping.load(mapping_id) if mapping_id else Mapping.identity(mr)
    A = synth.row_skew(130, 300, 0.85, seed=3, std=0.5)
    B = synth.dense(300, 48, seed=4)
    C0 = synth.dense(130, 48, seed=5)
    pk = O.Packed(O.Tables.of(m), A, k_tile=k_tile)
    want = pk.execute(B, C0.copy() if load_c else None, load_c=load_c, epilogue=int(relu))
    got = pk.execute_fast(B, C0.copy() if load_c else None, load_c=load_c, epilogue=int(relu), threads=3)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_simd_csr_baseline_is_bit_identical():
    from spreg import synth
    A = synth.row_skew(200, 256, 0.9, seed=8, std=1.0)
    rp, ci, v = synth.to_csr(A)
    B = synth.dense(256, 128, seed=9)
    assert np.array_equal(O.csr_spmm_fast(rp, ci, v, B, threads=3).view(np.uint32),
                          O.csr_spmm(rp, ci, v, B).view(np.uint32))


@pytest.mark.parametrize("load_c,relu", [(False, False), (True, True)])
def test_load_balanced_order_known_answers(load_c, relu):
    """The restated load-balanced order: a split at K tile 0 (zero + the whole chain from zero) or at
    K tile T (the whole chain + zero) gives the executor's own bits; a split in the middle stays within
    FP32 rounding of it, and panels that are not split keep its bits."""
    m = Mapping.identity(4)
    A = synth.row_skew(90, 384, 0.8, seed=11, std=1.0)
    B = synth.dense(384, 40, seed=12)
    C0 = synth.dense(90, 40, seed=13)
    t = O.Tables.of(m)
    plain = O.Packed(t, A, k_tile=64).execute(B, C0.copy() if load_c else None, load_c=load_c, epilogue=int(relu))
    heavy = [0, 3, 7, 22]
    if not load_c:  # from zero: 0 + chain = chain
        at0 = O.load_balanced_execute(t, A, B, heavy, 0, 64, epilogue=int(relu))
        assert np.array_equal(at0.view(np.uint32), plain.view(np.uint32))
    atT = O.load_balanced_execute(t, A, B, heavy, 6, 64, out=C0.copy() if load_c else None, load_c=load_c,
                                  epilogue=int(relu))
    assert np.array_equal(atT.view(np.uint32), plain.view(np.uint32))
    mid = O.load_balanced_execute(t, A, B, heavy, 3, 64, out=C0.copy() if load_c else None, load_c=load_c,
                                  epilogue=int(relu))
    rows = np.concatenate([np.arange(4 * p, 4 * p + 4) for p in heavy])
    rows = rows[rows < 90]  # panel 22 is the ragged last one (rows 88, 89)
    others = np.setdiff1d(np.arange(90), rows)
    assert np.array_equal(mid[others].view(np.uint32), plain[others].view(np.uint32))
    assert O.rel_err(mid[rows], plain[rows]) < 1e-6
