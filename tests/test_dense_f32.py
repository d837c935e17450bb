"""FP32-accurate dense rows on the tensor cores (spreg_dense_rows_f32: scaled FP16 split pairs, three
MMAs per K step) and the FP32 hybrid (tensor-core panels + register-tiled panels).

The bar is the one the FP32 executor is held to: rel err <= 1e-5 against the oracle's FP32 executor
(sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:265-305, restated in oracle/) and against an FP64
product of the same FP32 inputs, on the 2048 x 512 @ 90 % row-skew headline shape, the FFN shapes
across sparsities, ragged shapes and a wide dynamic range of row and column magnitudes."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from spreg import _lib, synth

pytestmark = pytest.mark.gpu

F32_TOL = 1e-5  # the FP32 executor's tolerance against the reference executor and FP64


def _rel(a, b):
    return float((a.double() - b.double()).norm() / max(float(b.double().norm()), 1e-300))


def _fp64(a, b):
    return a.double() @ b.double()


@pytest.mark.parametrize("R,K,n", [(1, 1, 1), (128, 64, 128), (300, 100, 200), (77, 1000, 16), (256, 4096, 96),
                                   (129, 520, 257), (640, 512, 512), (100, 2500, 70)])
@pytest.mark.parametrize("load_c,relu", [(False, False), (True, True)])
def test_dense_rows_f32_matches_fp64(cuda, R, K, n, load_c, relu):
    import torch
    from spreg.hybrid import dense_rows_f32, split_rows_f32
    g = torch.Generator(device="cuda").manual_seed(R * 7 + K + n)
    M = R + 37
    a = torch.randn((R, K), device="cuda", generator=g)
    B = torch.randn((K, n), device="cuda", generator=g)
    rows = torch.randperm(M, device="cuda", generator=g)[:R].to(torch.int32)
    C0 = torch.randn((M, n), device="cuda", generator=g)
    C = C0.clone()
    a_split, scale = split_rows_f32(a)
    dense_rows_f32(a_split, scale, rows, B, C, load_c=load_c, epilogue=1 if relu else 0)
    want = _fp64(a, B)
    if load_c:
        want = want + C0[rows.long()].double()
    if relu:
        want = torch.relu(want)
    assert _rel(C[rows.long()], want) <= F32_TOL
    others = torch.ones(M, dtype=torch.bool, device="cuda")
    others[rows.long()] = False
    assert torch.equal(C[others], C0[others])  # rows the product does not own are untouched
    from spreg.packed import device_status
    assert device_status() == 0


def test_split_pair_is_exact_to_fp32_level(cuda):
    """hi + lo reproduces every scaled value to 2^-22 relative (the FP16 pair carries 22 bits)."""
    import torch
    from spreg.hybrid import split_rows_f32
    g = torch.Generator(device="cuda").manual_seed(5)
    a = torch.randn((64, 333), device="cuda", generator=g) * torch.logspace(-30, 30, 64, device="cuda")[:, None]
    a[3] = 0.0
    a_split, scale = split_rows_f32(a)
    R = a.shape[0]
    back = (a_split[:R, :333].double() + a_split[R:, :333].double()) * scale.double()[:, None]
    rel = ((back - a.double()).abs() / a.double().abs().amax(dim=1, keepdim=True).clamp_min(1e-300))
    assert float(rel.max()) <= 2.0 ** -22
    assert float(scale[3]) == 1.0 and torch.count_nonzero(a_split[[3, R + 3]]) == 0
    assert torch.count_nonzero(a_split[:, 333:]) == 0  # padding columns are zero


def test_dense_rows_f32_wide_dynamic_range(cuda):
    """Rows of A spanning 1e-20 .. 1e20 and columns of B 1e-10 .. 1e10 keep FP32-level error in every
    element, relative to the magnitudes that meet in it."""
    import torch
    from spreg.hybrid import dense_rows_f32, split_rows_f32
    g = torch.Generator(device="cuda").manual_seed(9)
    R, K, n = 200, 300, 150
    a = torch.randn((R, K), device="cuda", generator=g) * torch.logspace(-20, 20, R, device="cuda")[:, None]
    B = torch.randn((K, n), device="cuda", generator=g) * torch.logspace(-10, 10, n, device="cuda")[None, :]
    C = torch.zeros((R, n), device="cuda")
    a_split, scale = split_rows_f32(a)
    dense_rows_f32(a_split, scale, torch.arange(R, device="cuda", dtype=torch.int32), B, C)
    want = _fp64(a, B)
    err = (C.double() - want).abs()
    # per element, relative to the magnitudes that meet in it (|a_i| . |b_j|)
    scale_ij = a.double().abs() @ B.double().abs()
    assert float((err / scale_ij.clamp_min(1e-300)).max()) <= 3e-5  # K = 300 FP32 additions
    assert torch.isfinite(C).all()


def _hybrid_f32(A, n, tc_fill, k_tile=128, seed=1):
    import torch
    from spreg import Mapping
    from spreg.hybrid import HybridMatrix
    At = torch.from_numpy(A).cuda()
    h = HybridMatrix.from_dense(At, Mapping.identity(4), tc_fill, k_tile=k_tile, value_dtype=_lib.F32)
    B = synth.dense(A.shape[1], n, seed=seed)
    C = h.execute(torch.from_numpy(B).cuda())
    return h, C.cpu().numpy(), B


@pytest.mark.parametrize("tc_fill", [0.0, 0.1, 1.01])
def test_hybrid_f32_headline_shape_vs_oracle_and_fp64(cuda, tc_fill):
    """2048 x 512 at 90 % row skew, N = 512 (the FP32 headline workload): every split of the panels
    stays within 1e-5 of the oracle's FP32 executor and of FP64; register-tiled rows are bit-exact."""
    from spreg import Mapping
    A = synth.row_skew(2048, 512, 0.9, seed=0, std=0.02)
    h, got, B = _hybrid_f32(A, 512, tc_fill)
    ref = O.Packed(O.Tables.of(Mapping.identity(4)), A).execute(B)
    assert O.rel_err(got, ref) <= F32_TOL
    assert O.rel_err(got, O.dense_fp64(A, B)) <= F32_TOL
    if tc_fill == 0.0:
        assert h.tc_rows == 2048
    if h.tc_rows < 2048:
        keep = np.ones(2048, bool)
        keep[h.row_index.cpu().numpy()] = False
        A_sp = A.copy()
        A_sp[~keep] = 0
        ref_sp = O.Packed(O.Tables.of(Mapping.identity(4)), A_sp, k_tile=128).execute(B)
        assert np.array_equal(got[keep].view(np.uint32), ref_sp[keep].view(np.uint32))


@pytest.mark.parametrize("shape", [(2048, 512), (512, 2048)])
@pytest.mark.parametrize("sparsity", [0.7, 0.8, 0.9, 0.95, 0.98])
def test_hybrid_f32_ffn_sweep_all_tensor_core(cuda, shape, sparsity):
    from spreg import Mapping
    A = synth.row_skew(shape[0], shape[1], sparsity, seed=11, std=0.02)
    h, got, B = _hybrid_f32(A, 512, 0.0, seed=12)
    assert h.tc_rows == shape[0]
    ref = O.Packed(O.Tables.of(Mapping.identity(4)), A).execute(B)
    assert O.rel_err(got, ref) <= F32_TOL
    assert O.rel_err(got, O.dense_fp64(A, B)) <= F32_TOL


def _items_case(seed=21):
    """Products of many shapes plus 10 products sharing one weight (coalesced); returns the items,
    the tensors to keep alive and each product's FP64 reference."""
    import torch
    from spreg.hybrid import f32_item, split_rows_f32
    g = torch.Generator(device="cuda").manual_seed(seed)
    items, keep, refs, outs = [], [], [], []
    cases = [(128, 64, 128), (7, 300, 33), (700, 1000, 200), (256, 520, 129), (384, 64, 300), (1, 5, 1),
             (130, 2100, 96)] * 4  # K = 2100: three K chunks
    for i, (R, K, n) in enumerate(cases):
        a = torch.randn((R, K), device="cuda", generator=g)
        a_split, sc = split_rows_f32(a)
        B = torch.randn((K, n), device="cuda", generator=g)
        idx = torch.arange(R, device="cuda", dtype=torch.int32)
        C = torch.zeros((R, n), device="cuda")
        items.append(f32_item(a_split, sc, idx, B, C))
        keep += [a_split, sc, B, idx]
        refs.append(_fp64(a, B))
        outs.append(C)
    a = torch.randn((512, 320), device="cuda", generator=g)
    a_split, sc = split_rows_f32(a)
    idx = torch.randperm(512, device="cuda", generator=g).to(torch.int32)
    keep += [a_split, sc, idx]
    for j in range(10):
        n = [64, 130, 256, 33, 1][j % 5]
        Bw = torch.randn((320, n + 3), device="cuda", generator=g)
        B = Bw[:, :n]  # a row stride that is not n
        C = torch.zeros((512, n), device="cuda")
        items.append(f32_item(a_split, sc, idx, B, C))
        keep.append(Bw)
        want = torch.zeros((512, n), device="cuda", dtype=torch.float64)
        want[idx.long()] = _fp64(a, B)
        refs.append(want)
        outs.append(C)
    return items, keep, refs, outs


def test_batched_coalesced_and_plan_equal_single_calls(cuda):
    """One batched call (many shapes, coalesced products over several B), a reusable plan run twice,
    and one call per product give the same bits, each within the FP32 tolerance."""
    import torch
    items, keep, refs, outs = _items_case()
    for it, want, C in zip(items, refs, outs):
        _lib.check(_lib.lib().spreg_dense_rows_f32(ctypes.byref(it), _lib.stream_handle(None)))
    torch.cuda.synchronize()
    single = [C.clone() for C in outs]
    for C, want in zip(single, refs):
        assert _rel(C, want) <= F32_TOL
    for C in outs:
        C.fill_(-7.0)
    arr = (_lib.DenseRowsF32Item * len(items))(*items)
    _lib.check(_lib.lib().spreg_dense_rows_f32_batched(arr, len(items), _lib.stream_handle(None)))
    torch.cuda.synchronize()
    for C, S in zip(outs, single):
        assert torch.equal(C.view(torch.int32), S.view(torch.int32))
    from spreg.hybrid import DenseRowsPlan
    plan = DenseRowsPlan(items)
    for _ in range(2):
        for C in outs:
            C.fill_(3.0)
        plan.run()
        torch.cuda.synchronize()
        for C, S in zip(outs, single):
            assert torch.equal(C.view(torch.int32), S.view(torch.int32))
    plan.close()
    from spreg.packed import device_status
    assert device_status() == 0


def test_hybrid_batch_equals_single_executes(cuda):
    """HybridBatch (register-tiled parts in one batched call, tensor-core parts as one plan) gives the
    bits of each HybridMatrix.execute, for all-tensor-core, mixed and register-tiled-only matrices."""
    import torch
    from spreg import Mapping
    from spreg.hybrid import HybridBatch, HybridMatrix
    triples, single = [], []
    for i, (fill, (M, K, n)) in enumerate([(0.0, (256, 512, 512)), (0.1, (300, 256, 100)), (1.01, (128, 96, 64)),
                                           (0.0, (2048, 512, 512))]):
        A = synth.row_skew(M, K, 0.9, seed=30 + i, std=0.02)
        A[8:16] = synth.bernoulli(8, K, 0.5, seed=40 + i, std=0.02)
        h = HybridMatrix.from_dense(torch.from_numpy(A).cuda(), Mapping.identity(4), fill, k_tile=128,
                                    value_dtype=_lib.F32)
        B = torch.from_numpy(synth.dense(K, n, seed=50 + i)).cuda()
        single.append(h.execute(B).clone())
        triples.append((h, B, torch.full((M, n), -1.0, device="cuda")))
    batch = HybridBatch(triples)
    batch.run()
    torch.cuda.synchronize()
    for (_, _, C), S in zip(triples, single):
        assert torch.equal(C.view(torch.int32), S.view(torch.int32))


def test_dense_rows_f32_argument_checks(cuda):
    import torch
    from spreg.hybrid import f32_item, split_rows_f32
    a = torch.randn((4, 12), device="cuda")
    a_split, sc = split_rows_f32(a)
    B = torch.randn((12, 8), device="cuda")
    C = torch.zeros((4, 8), device="cuda")
    idx = torch.arange(4, device="cuda", dtype=torch.int32)
    it = f32_item(a_split, sc, idx, B, C)
    it.ld_split = 12  # not a multiple of 8 elements
    with pytest.raises(_lib.SpregError, match="16-byte aligned"):
        _lib.check(_lib.lib().spreg_dense_rows_f32(ctypes.byref(it), _lib.stream_handle(None)))
    it = f32_item(a_split, sc, idx, B, C)
    it.tile_n = 64
    with pytest.raises(_lib.SpregError, match="tile_n"):
        _lib.check(_lib.lib().spreg_dense_rows_f32(ctypes.byref(it), _lib.stream_handle(None)))
    it = f32_item(a_split, sc, idx, B, C)
    it.row_scale = None
    with pytest.raises(_lib.SpregError, match="null"):
        _lib.check(_lib.lib().spreg_dense_rows_f32(ctypes.byref(it), _lib.stream_handle(None)))
    st = _lib.lib().spreg_dense_rows_f32_split(a.data_ptr(), 4, 12, 12, a_split.data_ptr(), 12, sc.data_ptr(),
                                               _lib.stream_handle(None))
    assert st == _lib.SPREG_ERR_INVALID_ARG and "multiple of 8" in _lib.last_error()
