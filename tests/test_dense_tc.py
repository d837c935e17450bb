"""Dense row panels on the tensor cores (tcgen05): products against torch FP32 of the same BF16
operands, and the hybrid split (tensor-core panels + register-tiled panels) against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from spreg import _lib, synth

pytestmark = pytest.mark.gpu

FP32_ACC_TOL = 1e-5   # FP32 accumulation of BF16 products, any order
BF16_OUT_TOL = 1e-2   # output rounded to BF16


def _rel(a, b):
    import torch
    return float((a.double() - b.double()).norm() / max(float(b.double().norm()), 1e-300))


@pytest.mark.parametrize("R,K,n", [(1, 8, 1), (128, 64, 128), (300, 100, 200), (77, 1000, 16), (256, 4096, 96),
                                   (129, 520, 257)])
@pytest.mark.parametrize("c_bf16,load_c,relu", [(False, False, False), (False, True, True), (True, False, True)])
def test_dense_rows_match_torch(cuda, R, K, n, c_bf16, load_c, relu):
    import torch
    from spreg.hybrid import dense_rows_bf16
    g = torch.Generator(device="cuda").manual_seed(R * 7 + K + n)
    M = R + 37
    k8 = (K + 7) // 8 * 8
    a = torch.zeros((R, k8), device="cuda", dtype=torch.bfloat16)
    a[:, :K] = torch.randn((R, K), device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn((K, n), device="cuda", generator=g).to(torch.bfloat16)
    rows = torch.randperm(M, device="cuda", generator=g)[:R].to(torch.int32)
    dt = torch.bfloat16 if c_bf16 else torch.float32
    C0 = torch.randn((M, n), device="cuda", generator=g).to(dt)
    C = C0.clone()
    dense_rows_bf16(a, rows, B, C, load_c=load_c, epilogue=1 if relu else 0)
    want = a[:, :K].float() @ B.float()
    if load_c:
        want = want + C0[rows.long()].float()
    if relu:
        want = torch.relu(want)
    got = C[rows.long()].float()
    assert _rel(got, want) <= (BF16_OUT_TOL if c_bf16 else FP32_ACC_TOL)
    others = torch.ones(M, dtype=torch.bool, device="cuda")
    others[rows.long()] = False
    assert torch.equal(C[others], C0[others])  # rows the product does not own are untouched
    from spreg.packed import device_status
    assert device_status() == 0


def test_dense_rows_argument_checks(cuda):
    import torch
    from spreg.hybrid import dense_rows_bf16
    a = torch.zeros((4, 12), device="cuda", dtype=torch.bfloat16)  # row stride 24 bytes
    B = torch.zeros((12, 8), device="cuda", dtype=torch.bfloat16)
    C = torch.zeros((4, 8), device="cuda")
    idx = torch.arange(4, device="cuda", dtype=torch.int32)
    with pytest.raises(_lib.SpregError, match="16-byte aligned"):
        dense_rows_bf16(a, idx, B, C)


def _hybrid_case(tc_fill, load_c, relu, seed=3):
    import torch
    from spreg import Mapping
    from spreg.hybrid import HybridMatrix, panel_fill
    M, K, n = 260, 384, 72
    A = synth.row_skew(M, K, 0.9, seed=seed, std=1.0)
    A[40:48] = synth.bernoulli(8, K, 0.4, seed=seed + 1, std=1.0)    # two dense panels
    A[200:204] = synth.bernoulli(4, K, 0.1, seed=seed + 2, std=1.0)  # one very dense panel
    A = synth.round_bf16(A)
    m = Mapping.identity(4)
    At = torch.from_numpy(A).cuda()
    h = HybridMatrix.from_dense(At, m, tc_fill, k_tile=128)
    B = synth.round_bf16(synth.dense(K, n, seed=seed + 3))
    Bt = torch.from_numpy(B).cuda().to(torch.bfloat16)
    C0 = synth.dense(M, n, seed=seed + 4)
    C = torch.from_numpy(C0).cuda().clone()
    h.execute(Bt, C, load_c=load_c, epilogue=1 if relu else 0)
    want = A.astype(np.float64) @ B.astype(np.float64) + (C0 if load_c else 0)
    if relu:
        want = np.maximum(want, 0)
    return h, C.cpu().numpy(), want, A, B, C0


@pytest.mark.parametrize("load_c,relu", [(False, False), (True, False), (False, True), (True, True)])
def test_hybrid_split_matches_fp64(cuda, load_c, relu):
    h, got, want, A, B, C0 = _hybrid_case(0.3, load_c, relu)
    assert h.tc_rows == 12  # panels 10, 11 (rows 40..47) and 50 (rows 200..203)
    assert O.rel_err(got, want) <= FP32_ACC_TOL
    # the register-tiled rows are bit-identical to the oracle's execution of the sparse part
    import torch
    A_sp = A.copy()
    A_sp[40:48] = 0
    A_sp[200:204] = 0
    from spreg import Mapping
    ref = O.Packed(O.Tables.of(Mapping.identity(4)), A_sp, k_tile=128, value_dtype=_lib.BF16)
    Bu = torch.from_numpy(B).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    Cr = C0.copy() if load_c else np.zeros_like(C0)
    ref.execute(Bu, Cr, load_c=load_c, epilogue=1 if relu else 0)
    keep = np.ones(A.shape[0], bool)
    keep[40:48] = keep[200:204] = False
    assert np.array_equal(got[keep].view(np.uint32), Cr[keep].view(np.uint32))


@pytest.mark.parametrize("fill", [0.0, 1.01])
def test_hybrid_all_or_no_panels_on_tensor_cores(cuda, fill):
    h, got, want, *_ = _hybrid_case(fill, True, True)
    assert h.tc_rows == (260 if fill == 0.0 else 0)
    assert O.rel_err(got, want) <= FP32_ACC_TOL


def test_batched_products_equal_single_calls(cuda):
    """Products of many shapes in one batched call are bit-identical to one call each."""
    import torch
    from spreg.hybrid import dense_rows_bf16
    from spreg.serving import TC_ITEM_DTYPE
    g = torch.Generator(device="cuda").manual_seed(5)
    cases = [(128, 64, 128), (7, 300, 33), (300, 1000, 200), (1, 8, 1), (256, 520, 129)] * 20  # 100 items
    ops, items = [], np.zeros(len(cases), dtype=TC_ITEM_DTYPE)
    for i, (R, K, n) in enumerate(cases):
        k8 = (K + 7) // 8 * 8
        a = torch.zeros((R, k8), device="cuda", dtype=torch.bfloat16)
        a[:, :K] = torch.randn((R, K), device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn((K, n), device="cuda", generator=g).to(torch.bfloat16)
        idx = torch.randperm(R + 5, device="cuda", generator=g)[:R].to(torch.int32)
        C1 = torch.randn((R + 5, n), device="cuda", generator=g)
        C2 = C1.clone()
        load_c, epi = i % 2, (i // 2) % 2
        dense_rows_bf16(a, idx, B, C1, load_c=bool(load_c), epilogue=epi)
        items[i] = (a.data_ptr(), R, K, a.stride(0), idx.data_ptr(), B.data_ptr(), B.stride(0), C2.data_ptr(),
                    C2.stride(0), n, _lib.F32, load_c, epi, 0)
        ops.append((a, idx, B, C1, C2))
    _lib.check(_lib.lib().spreg_dense_rows_bf16_batched(items.ctypes.data, len(cases),
                                                       _lib.stream_handle(torch.cuda.current_stream())))
    torch.cuda.synchronize()
    for a, idx, B, C1, C2 in ops:
        assert torch.equal(C1.view(torch.int32), C2.view(torch.int32))


def test_products_sharing_weights_coalesce_to_same_results(cuda):
    """Products with the same weight rows (the same layer for many requests) run as one product over
    their side-by-side B; every output equals its own single call bit for bit."""
    import torch
    from spreg.hybrid import dense_rows_bf16
    from spreg.serving import TC_ITEM_DTYPE
    g = torch.Generator(device="cuda").manual_seed(9)
    R, K = 300, 520
    a = torch.zeros((R, 520), device="cuda", dtype=torch.bfloat16)
    a[:, :K] = torch.randn((R, K), device="cuda", generator=g).to(torch.bfloat16)
    idx = torch.randperm(R, device="cuda", generator=g).to(torch.int32)
    ns = [1, 64, 130, 7, 256, 300, 33, 128, 2, 200] * 3
    items = np.zeros(len(ns), dtype=TC_ITEM_DTYPE)
    ops = []
    for i, n in enumerate(ns):
        B = torch.randn((K, n + 3), device="cuda", generator=g).to(torch.bfloat16)[:, :n]  # ldb > n
        C1 = torch.randn((R, n), device="cuda", generator=g)
        C2 = C1.clone()
        load_c, epi = i % 2, (i // 3) % 2  # three coalesced groups of mixed widths
        dense_rows_bf16(a, idx, B, C1, load_c=bool(load_c), epilogue=epi)
        items[i] = (a.data_ptr(), R, K, a.stride(0), idx.data_ptr(), B.data_ptr(), B.stride(0), C2.data_ptr(),
                    C2.stride(0), n, _lib.F32, load_c, epi, 0)
        ops.append((B, C1, C2))
    _lib.check(_lib.lib().spreg_dense_rows_bf16_batched(items.ctypes.data, len(ns),
                                                       _lib.stream_handle(torch.cuda.current_stream())))
    torch.cuda.synchronize()
    for B, C1, C2 in ops:
        assert torch.equal(C1.view(torch.int32), C2.view(torch.int32))


def test_tile_width_hint_gives_the_same_products(cuda):
    """tile_n = 128 / 256 / automatic: the same FP32 sums of BF16 products (the MMA's K order does not
    depend on the tile width), and a bad hint is refused."""
    import torch
    from spreg.serving import TC_ITEM_DTYPE
    M, K, N = 300, 200, 400
    A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
    B = torch.randn(K, N, device="cuda").to(torch.bfloat16)
    ri = torch.arange(M, dtype=torch.int32, device="cuda")
    outs = []
    for tn in (0, 128, 256):
        C = torch.empty(M, N, device="cuda")
        it = np.zeros(1, dtype=TC_ITEM_DTYPE)
        it[0] = (A.data_ptr(), M, K, K, ri.data_ptr(), B.data_ptr(), N, C.data_ptr(), N, N, _lib.F32, 0, 0, tn)
        _lib.check(_lib.lib().spreg_dense_rows_bf16_batched(it.ctypes.data, 1, _lib.stream_handle(None)))
        outs.append(C)
    torch.cuda.synchronize()
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], outs[2])
    ref = A.float() @ B.float()
    assert float((outs[0] - ref).norm() / ref.norm()) <= 1e-5
    it[0]["tile_n"] = 64
    with pytest.raises(_lib.SpregError, match="tile_n"):
        _lib.check(_lib.lib().spreg_dense_rows_bf16_batched(it.ctypes.data, 1, _lib.stream_handle(None)))


def _shapes_run():
    """Single products (odd and even row block counts, 128- and 256-wide tiles, B read in place), a
    batched call of many shapes and a coalesced call over several B (transposed B); returns every
    output."""
    import torch
    from spreg.hybrid import dense_rows_bf16
    from spreg.serving import TC_ITEM_DTYPE
    mode = "single CTAs"
    g = torch.Generator(device="cuda").manual_seed(21)
    outs = []
    for R, K, n, c_bf16, load_c, relu in [(1, 8, 1, False, False, False), (300, 100, 200, False, True, True),
                                          (640, 520, 384, False, False, False), (129, 1000, 257, True, True, False),
                                          (1024, 256, 128, False, False, True), (2048, 512, 512, False, True, False)]:
        k8 = (K + 7) // 8 * 8
        a = torch.zeros((R, k8), device="cuda", dtype=torch.bfloat16)
        a[:, :K] = torch.randn((R, K), device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn((K, n), device="cuda", generator=g).to(torch.bfloat16)
        rows = torch.randperm(R + 9, device="cuda", generator=g)[:R].to(torch.int32)
        dt = torch.bfloat16 if c_bf16 else torch.float32
        C0 = torch.randn((R + 9, n), device="cuda", generator=g).to(dt)
        C = C0.clone()
        dense_rows_bf16(a, rows, B, C, load_c=load_c, epilogue=1 if relu else 0)
        want = a[:, :K].float() @ B.float()
        if load_c:
            want = want + C0[rows.long()].float()
        if relu:
            want = torch.relu(want)
        assert _rel(C[rows.long()].float(), want) <= (BF16_OUT_TOL if c_bf16 else FP32_ACC_TOL), (mode, R, K, n)
        others = torch.ones(R + 9, dtype=torch.bool, device="cuda")
        others[rows.long()] = False
        assert torch.equal(C[others], C0[others])
        outs.append(C)
    # B rows of 602 bytes cannot be read in place: transposed into a K-major buffer, 256-wide tiles
    a = torch.randn((700, 264), device="cuda", generator=g).to(torch.bfloat16)
    Bu = torch.randn((264, 301), device="cuda", generator=g).to(torch.bfloat16)[:, :300]
    C = torch.zeros((700, 300), device="cuda")
    dense_rows_bf16(a, torch.arange(700, device="cuda", dtype=torch.int32), Bu, C)
    assert _rel(C, a.float() @ Bu.float()) <= FP32_ACC_TOL, mode
    outs.append(C)
    # many shapes in one launch, and 12 products sharing one weight (coalesced, B transposed)
    cases = [(128, 64, 128), (7, 300, 33), (700, 1000, 200), (256, 520, 129), (384, 64, 300)] * 8
    a_sh = torch.randn((512, 320), device="cuda", generator=g).to(torch.bfloat16)
    i_sh = torch.randperm(512, device="cuda", generator=g).to(torch.int32)
    items = np.zeros(len(cases) + 12, dtype=TC_ITEM_DTYPE)
    keep = []
    for i, (R, K, n) in enumerate(cases):
        k8 = (K + 7) // 8 * 8
        a = torch.zeros((R, k8), device="cuda", dtype=torch.bfloat16)
        a[:, :K] = torch.randn((R, K), device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn((K, n), device="cuda", generator=g).to(torch.bfloat16)
        idx = torch.arange(R, device="cuda", dtype=torch.int32)
        C = torch.randn((R, n), device="cuda", generator=g)
        items[i] = (a.data_ptr(), R, K, a.stride(0), idx.data_ptr(), B.data_ptr(), B.stride(0), C.data_ptr(),
                    C.stride(0), n, _lib.F32, i % 2, (i // 2) % 2, 0)
        keep += [a, B, idx]
        outs.append(C)
    for j in range(12):
        n = [64, 130, 256, 33][j % 4]
        B = torch.randn((320, n + 5), device="cuda", generator=g).to(torch.bfloat16)[:, :n]
        C = torch.zeros((512, n), device="cuda")
        items[len(cases) + j] = (a_sh.data_ptr(), 512, 320, 320, i_sh.data_ptr(), B.data_ptr(), B.stride(0),
                                 C.data_ptr(), n, n, _lib.F32, 0, 0, 0)
        keep.append(B)
        outs.append(C)
    _lib.check(_lib.lib().spreg_dense_rows_bf16_batched(items.ctypes.data, len(items),
                                                       _lib.stream_handle(torch.cuda.current_stream())))
    torch.cuda.synchronize()
    from spreg.packed import device_status
    assert device_status() == 0
    return outs


def test_products_of_many_shapes_alone_batched_and_coalesced_are_repeatable(cuda):
    """Every shape family (single products, one launch of many shapes, coalesced products over
    several B) meets its tolerance, and a second run gives the same bits."""
    import torch
    first = _shapes_run()
    again = _shapes_run()
    for x, y in zip(first, again):
        assert torch.equal(x.view(torch.int16) if x.dtype == torch.bfloat16 else x.view(torch.int32),
                           y.view(torch.int16) if y.dtype == torch.bfloat16 else y.view(torch.int32))


def test_bf16_plan_equals_batched_call(cuda):
    """spreg_dense_rows_bf16_plan_create: the same products as one batched call (many shapes, products
    coalesced over one weight, B read in place and transposed), run twice."""
    import torch
    from spreg.hybrid import DenseRowsPlan, bf16_items
    g = torch.Generator(device="cuda").manual_seed(44)
    rows, outs, keep = [], [], []
    a_sh = torch.randn((300, 264), device="cuda", generator=g).to(torch.bfloat16)
    i_sh = torch.arange(300, device="cuda", dtype=torch.int32)
    for j, (R, K, n) in enumerate([(128, 64, 128), (7, 300, 33), (700, 1000, 200), (256, 520, 257)] * 2):
        k8 = (K + 7) // 8 * 8
        a = torch.zeros((R, k8), device="cuda", dtype=torch.bfloat16)
        a[:, :K] = torch.randn((R, K), device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn((K, n), device="cuda", generator=g).to(torch.bfloat16)
        idx = torch.arange(R, device="cuda", dtype=torch.int32)
        C = torch.zeros((R, n), device="cuda")
        rows.append((a, idx, B, C, n, K, j % 2, (j // 2) % 2))
        keep += [a, B, idx]
        outs.append(C)
    for n in (64, 130, 33):
        B = torch.randn((264, n), device="cuda", generator=g).to(torch.bfloat16)
        C = torch.zeros((300, n), device="cuda")
        rows.append((a_sh, i_sh, B, C, n, 264, 0, 0))
        keep.append(B)
        outs.append(C)
    items = bf16_items(rows)
    _lib.check(_lib.lib().spreg_dense_rows_bf16_batched(items.ctypes.data, len(items), _lib.stream_handle(None)))
    torch.cuda.synchronize()
    want = [C.clone() for C in outs]
    plan = DenseRowsPlan(items)
    for _ in range(2):
        for C in outs:
            C.zero_()
        plan.run()
        torch.cuda.synchronize()
        for C, W in zip(outs, want):
            assert torch.equal(C.view(torch.int32), W.view(torch.int32))
    plan.close()
