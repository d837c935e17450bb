"""Autotuner: statistics against the oracle packing, cost-model fitting, ranking; GPU tuning."""
import numpy as np
import pytest

from oracle import oracle as O
from spreg import synth
from spreg.autotune import (Candidate, Costs, candidates, fit_costs, heuristic_bucket, mapping_of, model_row,
                            panel_codes, panel_stats, rank, tune)

CASES = [(2, "identity"), (4, "identity"), (8, "identity"), (8, "400fa"), (8, "747f9")]


@pytest.mark.parametrize("mr,mp", CASES)
@pytest.mark.parametrize("shape,sp", [((61, 97), 0.8), ((128, 256), 0.95), ((37, 64), 0.5)])
def test_panel_stats_match_oracle_packing(mr, mp, shape, sp):
    A = synth.row_skew(*shape, sp, seed=shape[0] + mr, sigma=0.5)
    m = mapping_of(mr, mp)
    st = panel_stats(A != 0, mr, m)
    pk = O.Packed(O.Tables.of(m), A)
    assert st.P == pk.num_panels
    assert st.U == pk.sizes["num_col_indices"]
    assert st.V == pk.sizes["num_values"]
    assert st.padding == pk.sizes["padding"]
    assert st.nnz == pk.sizes["nnz"]
    # G: nonzero nkern_counts of every panel, read out of the oracle arena
    nk = pk.t.num_nkern
    G = 0
    maxU = 0
    for d in pk.descs:
        counts = pk.arena[d["counts_off"]: d["counts_off"] + 4 * nk].view(np.int32)
        G += int(np.count_nonzero(counts))
        maxU = max(maxU, int(d["num_cols"]))
    assert st.G == G
    assert st.max_panel_U == maxU


def test_panel_codes_bits():
    mask = np.zeros((5, 3), dtype=bool)
    mask[0, 0] = mask[3, 0] = mask[4, 2] = True
    c = panel_codes(mask, 4)
    assert c.shape == (2, 3)
    assert c[0, 0] == 0b1001 and c[1, 2] == 0b0001 and c[0, 1] == 0


def test_heuristic_buckets():
    assert heuristic_bucket(0.65, 32) == ("(0,0.7]", 32)
    assert heuristic_bucket(0.75, 100) == ("(0.7,0.8]", 128)
    assert heuristic_bucket(0.9, 300) == ("(0.8,0.9]", 256)
    assert heuristic_bucket(0.98, 4096) == ("(0.9,1]", 512)


def test_fit_costs_recovers_coefficients():
    true = [3000.0, 15.0, 5.0, 2.0, 0.5, 30.0]
    samples = []
    for i, (shape, sp) in enumerate([((512, 512), 0.8), ((1024, 256), 0.9), ((256, 2048), 0.95),
                                     ((2048, 512), 0.7), ((640, 640), 0.85), ((300, 900), 0.6)]):
        st = panel_stats(synth.row_skew(*shape, sp, seed=i) != 0, 4, mapping_of(4, "identity"))
        for n in (16, 64, 256, 1000):
            samples.append(("f32", st, n, 2, float(np.dot(true, model_row(st, n, 2)))))
    c = fit_costs(samples)
    np.testing.assert_allclose(c.table[Costs.key(4, 2, "f32")], true, rtol=1e-6, atol=1e-6)


def test_costs_save_load(tmp_path):
    c = Costs.default()
    c.table[Costs.key(8, 4, "bf16")] = [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]
    p = tmp_path / "c.json"
    c.save(str(p), {"samples": 3})
    d = Costs.load(str(p))
    assert d.table[Costs.key(8, 4, "bf16")] == [1.0, 2.0, 3.0, 4.0, 5.0, 6.0]


def test_rank_orders_all_candidates():
    A = synth.row_skew(512, 512, 0.9, seed=1)
    ranked, stats = rank(A != 0, 48, "f32", Costs.default(), greedy=False)
    ts = [t for t, _ in ranked]
    assert ts == sorted(ts)
    names = {c.name() for _, c in ranked}
    assert names == {c.name() for c in candidates(48, k=512)}
    assert "M4N64_identity" in names and "M8N32_400fa" in names and "M4N128_identity" not in names
    assert set(stats) == {(2, "identity"), (4, "identity"), (8, "identity"), (8, "400fa"), (8, "747f9")}
    assert Candidate(4, "identity", 64).name() == "M4N64_identity"
    assert Candidate(2, "identity", 32, 1024).name() == "M2N32_identity_K1024"
    wide = {c.name() for c in candidates(64, (2,), k=2048)}
    assert {"M2N64_identity", "M2N64_identity_K512", "M2N64_identity_K1024"} <= wide
    assert not any("_K" in c.name() for c in candidates(64, (4,), k=128))
    assert {c.k_tile for c in candidates(64, (4,), k=512)} == {0, 128, 256}
    # 256-column strips: 16-bit B, M_r <= 4, K_c <= 128, n >= 128
    w = {c.name() for c in candidates(512, (4, 8), k=1024, wide=True)}
    assert "M4N256_identity_K128" in w and not any(n.startswith("M8N256") for n in w)
    assert not any("N256" in n for n in w if "_K128" not in n)
    assert not any(c.nr == 256 for c in candidates(512, (4,), k=1024))


@pytest.mark.gpu
def test_tune_picks_a_measured_candidate_and_it_is_exact(cuda):
    import torch
    from spreg import PackedMatrix
    from spreg.autotune import tune
    A = synth.row_skew(1024, 512, 0.9, seed=4)
    res = tune(A, 128, "f32", top=3, tc=False, warps=False)
    assert res.best.name() in res.measured_ns and len(res.measured_ns) >= 3
    # every (M_r, nanokernel set) family was timed at least once
    fams = {n.split("_")[0][:2] + "_" + n.split("_")[1] for n in res.measured_ns}
    assert {"M2_identity", "M4_identity", "M8_identity", "M8_400fa", "M8_747f9"} <= fams
    assert res.measured_ns[res.best.name()] == min(res.measured_ns.values())
    m = mapping_of(res.best.mr, res.best.mapping)
    B = synth.dense(512, 128, seed=5)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m)
    got = pm.execute(torch.from_numpy(B).cuda(), nr=res.best.nr).cpu().numpy()
    want = O.Packed(O.Tables.of(m), A).execute(B)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_rank_adds_greedy_nanokernel_sets_for_mr8_and_tiled_mr4():
    from spreg.autotune import GENERATED
    A = synth.row_skew(256, 384, 0.9, seed=2)
    ranked, stats = rank(A != 0, 64, "f32", Costs.default())
    gen = {(c.mr, c.mapping) for _, c in ranked if c.mapping in GENERATED}
    assert {mr for mr, _ in gen} == {4, 8} and len(gen) == 2
    for mr, gid in gen:
        assert (mr, gid) in stats and mapping_of(mr, gid).mapping_id == gid
        assert all(c.k_tile > 0 for _, c in ranked if c.mr == 4 and c.mapping == gid)  # B-tile executor sets


def test_candidate_names_carry_cta_tiling_and_tensor_core_threshold():
    assert Candidate(4, "identity", 128, 128, warps=8).name() == "M4N128_identity_K128_W8"
    assert Candidate(2, "identity", 64, tc_fill=0.0).name() == "M2N64_identity_TC0"
    assert Candidate(2, "identity", 64).tc_fill > 1.0  # no tensor-core panels by default


def test_tensor_core_prediction_grows_with_the_panels_it_takes():
    from spreg.autotune import tc_predict_ns
    A = synth.row_skew(1024, 512, 0.9, seed=3)
    t_all, share_all = tc_predict_ns(A != 0, 256, "bf16", 0.0, 4)
    t_none, share_none = tc_predict_ns(A != 0, 256, "bf16", 1.01, 4)
    t_f32, _ = tc_predict_ns(A != 0, 256, "f32", 0.0, 4)
    assert share_all == 1.0 and share_none == 0.0 and t_all > t_none and t_f32 > t_all


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,n", [("f32", 512), ("bf16", 256), ("bf16", 32)])
def test_full_tune_best_is_measured_and_within_tolerance(cuda, dtype, n):
    """CTA tiling and tensor-core thresholds take part; the winner is the fastest measured and its
    result holds the storage's tolerance (FP32 1e-5, BF16 1e-2 against FP64)."""
    import torch
    from spreg import _lib
    from spreg.hybrid import HybridMatrix
    A = synth.row_skew(1024, 512, 0.9, seed=6, std=0.02)
    res = tune(A, n, dtype, top=2, batch=8)
    assert res.measured_ns[res.best.name()] == min(res.measured_ns.values())
    assert any("_W" in k for k in res.measured_ns)
    assert dtype == "f32" or n < 64 or any("_TC" in k for k in res.measured_ns)
    c = res.best
    m = mapping_of(c.mr, c.mapping)
    vd = _lib.F32 if dtype == "f32" else _lib.BF16
    h = HybridMatrix.from_dense(torch.from_numpy(A).cuda(), m, c.tc_fill, k_tile=c.k_tile, value_dtype=vd)
    B = synth.dense(512, n, seed=7)
    Bt = torch.from_numpy(B).cuda()
    if dtype == "bf16":
        Bt = Bt.to(torch.bfloat16)
    got = h.execute(Bt, nr=c.nr).cpu().numpy()
    Bq = Bt.float().cpu().numpy()
    Aq = A if dtype == "f32" else torch.from_numpy(A).to(torch.bfloat16).float().numpy()
    assert O.rel_err(got, O.dense_fp64(Aq, Bq)) <= (1e-5 if dtype == "f32" else 1e-2)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f32", "bf16"])
def test_tune_times_the_wide_gather_strips_at_the_sparse_end(cuda, dtype):
    """At 98 % sparsity and n = 512 the tuner times the gather kernel's 256- and 512-column strips of
    untiled packs beside its other candidates; its pick executes bit-exact with the oracle."""
    import torch
    from spreg import PackedMatrix, _lib
    A = synth.row_skew(2048, 512, 0.98, seed=11, sigma=0.5, std=0.02)
    res = tune(A, 512, dtype, top=2, batch=8, tc=False, rounds=False)
    wide = [k for k in res.measured_ns if k.split("_")[0].endswith(("N256", "N512")) and "_K" not in k]
    assert any("N512" in k for k in wide) and any("N256" in k for k in wide), sorted(res.measured_ns)
    assert res.measured_ns[res.best.name()] == min(res.measured_ns.values())
    c = res.best
    m = mapping_of(c.mr, c.mapping)
    vd = _lib.F32 if dtype == "f32" else _lib.BF16
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=c.k_tile, value_dtype=vd)
    B = synth.dense(512, 512, seed=12)
    Bt = torch.from_numpy(B).cuda()
    Bref = B
    if dtype == "bf16":
        Bt = Bt.bfloat16()
        Bref = Bt.cpu().view(torch.int16).numpy().view(np.uint16)
    got = pm.execute(Bt, nr=c.nr, warps=c.warps).cpu().numpy()
    want = O.Packed(O.Tables.of(m), A, k_tile=c.k_tile, value_dtype=vd).execute(Bref)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_candidate_names_round_trip():
    """candidate_from_name inverts Candidate.name(), greedy mapping ids included (rebuilt from A)."""
    from spreg.autotune import GENERATED, candidate_from_name, greedy_mapping, mapping_of
    A = synth.row_skew(512, 256, 0.9, seed=5, std=1.0)
    gid = greedy_mapping(A != 0, 4, budget=15, tile=True).mapping_id
    GENERATED.pop(gid, None)
    for name in ("M4N128_identity_K128", f"M4N256_{gid}_K128", "M8N64_400fa_W4_R16", "M2N32_identity_K256_TC0.1"):
        c = candidate_from_name(name, A)
        assert c.name() == name
        mapping_of(c.mr, c.mapping)  # registered, or a named mapping file
    with pytest.raises(ValueError):
        candidate_from_name("N128M4")
