"""spreg_execute_batched_noalloc: the executor entry point for callers that cannot allocate device
memory while it runs (for example a serving loop whose device memory is owned by another
allocator).  It must give the bits of spreg_execute_batched and of the oracle's FP32 / 16-bit
executor (sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:265-305, restated in oracle/), call
after call, with its scratch in the library's static device array, and report its status word
through spreg_device_status.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.packed import PackedMatrix

pytestmark = pytest.mark.gpu


def _work(items):
    arr = (_lib.WorkItem * len(items))()
    for i, (pm, B, C, kw) in enumerate(items):
        arr[i].a = pm.handle
        arr[i].args = pm.exec_args(B, C, **kw)
    return arr


def _torch_dt(code):
    return {_lib.F32: torch.float32, _lib.BF16: torch.bfloat16, _lib.F16: torch.float16}[code]


# (M, K, N, mapping, value dtype, k_tile, exec kwargs, ldb pad, ldc pad, out BF16)
CASES = [
    (256, 512, 128, "61fee", _lib.F32, 0, {}, 0, 0, False),
    (130, 300, 77, "400fa", _lib.F32, 0, {}, 0, 0, False),
    (512, 256, 96, "61fee", _lib.BF16, 0, {}, 0, 0, False),
    (384, 520, 200, "61fee", _lib.F32, 128, {}, 0, 0, False),             # K-tiled, automatic staging
    (200, 256, 64, "61fee", _lib.F32, 0, {"nr": 32}, 3, 5, False),       # explicit N_r, odd ldb / ldc
    (160, 192, 90, "61fee", _lib.F32, 64, {"load_c": True, "epilogue": 1}, 1, 2, False),
    (96, 128, 20, "61fee", _lib.F32, 0, {}, 0, 0, False),                # N < 32
    (128, 256, 128, "61fee", _lib.F16, 0, {"nr": 64}, 0, 0, False),       # FP16 values with panel scales
    (144, 200, 72, "61fee", _lib.BF16, 0, {"epilogue": 1}, 0, 0, True),   # BF16 out
    (256, 512, 512, "61fee", _lib.F32, 0, {"nr": 512}, 0, 0, False),      # wide FP32 strips (512 columns)
    (300, 256, 600, "400fa", _lib.F32, 0, {"nr": 256}, 0, 4, False),      # 256-column FP32, M_r 8, tail
    (260, 512, 512, "61fee", _lib.BF16, 0, {"nr": 512}, 0, 0, False),     # 512-column 16-bit strips
    (128, 256, 512, "61fee", _lib.F16, 0, {"nr": 256}, 0, 0, False),      # 256-column, FP16 panel scales
    (144, 200, 512, "61fee", _lib.BF16, 0, {"nr": 512, "epilogue": 1}, 0, 0, True),  # wide, BF16 out
]


def _build(case, i):
    M, K, N, mid, vd, kt, kw, pb, pc, out_bf16 = case
    m = Mapping.identity(4) if mid == "61fee" else Mapping.load(mid)
    A = synth.row_skew(M, K, 0.85, seed=40 + i, std=1.0)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=kt, value_dtype=vd)
    Bf = synth.dense(K, N, seed=50 + i)
    bt = torch.float32 if vd == _lib.F32 else _torch_dt(vd)
    Bw = torch.zeros((K, N + pb), dtype=bt, device="cuda")
    Bw[:, :N] = torch.from_numpy(Bf).cuda().to(bt)
    C0 = synth.dense(M, N, seed=60 + i)
    ct = torch.bfloat16 if out_bf16 else torch.float32
    return m, A, pm, Bw[:, :N], C0, ct, pc


def _fresh_c(C0, ct, pc):
    Cw = torch.zeros((C0.shape[0], C0.shape[1] + pc), dtype=ct, device="cuda")
    Cw[:, :C0.shape[1]] = torch.from_numpy(C0).cuda().to(ct)
    return Cw[:, :C0.shape[1]]


def _oracle(case, m, A, pm, B, C0):
    M, K, N, mid, vd, kt, kw, pb, pc, out_bf16 = case
    ref = O.Packed(O.Tables.of(m), A, k_tile=kt, value_dtype=vd)
    if vd == _lib.F32:
        Bh = B.cpu().numpy()
    else:
        Bh = B.contiguous().view(torch.int16).cpu().numpy().view(np.uint16)
    Cr = C0.copy() if kw.get("load_c") else np.zeros_like(C0)
    ref.execute(Bh, Cr, load_c=bool(kw.get("load_c")), epilogue=int(kw.get("epilogue", 0)))
    return Cr


def test_noalloc_matches_batched_and_oracle_twice(cuda):
    built = [_build(c, i) for i, c in enumerate(CASES)]
    ref_items, na_items = [], []
    for case, (m, A, pm, B, C0, ct, pc) in zip(CASES, built):
        kw = case[6]
        ref_items.append((pm, B, _fresh_c(C0, ct, pc), kw))
        na_items.append((pm, B, _fresh_c(C0, ct, pc), kw))
    L = _lib.lib()
    stream = _lib.stream_handle(None)
    _lib.check(L.spreg_execute_batched(_work(ref_items), len(ref_items), stream))
    torch.cuda.synchronize()
    # the regular entry point against the oracle (FP32 results bit-exact; BF16 output rounded once)
    for case, (m, A, pm, B, C0, ct, pc), (_, _, Cr, _) in zip(CASES, built, ref_items):
        want = _oracle(case, m, A, pm, B, C0)
        got = Cr.float().cpu().numpy()
        if ct == torch.float32:
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), case
        else:
            assert O.rel_err(got, want) <= 1e-2, case
    na = _work(na_items)
    for call in range(2):
        for (_, _, C, kw), (case, (m, A, pm, B, C0, ct, pc)) in zip(na_items, zip(CASES, built)):
            C.copy_(torch.from_numpy(C0).cuda().to(ct) if kw.get("load_c") else torch.full_like(C, -1.0))
        _lib.check(L.spreg_execute_batched_noalloc(na, len(na_items), stream))
        torch.cuda.synchronize()
        for (_, _, Cr, _), (_, _, Cn, _), case in zip(ref_items, na_items, CASES):
            assert torch.equal(Cr, Cn), f"call {call}: {case}"
    status = ctypes.c_int32()
    _lib.check(L.spreg_device_status(ctypes.byref(status), 0))
    assert status.value == 0


def test_noalloc_rejects_more_launches_than_its_scratch(cuda):
    m = Mapping.identity(4)
    pm = PackedMatrix.from_dense(torch.from_numpy(synth.bernoulli(8, 32, 0.5, seed=1)).cuda(), m)
    B = torch.ones((32, 32), device="cuda")
    C = torch.zeros((8, 32), device="cuda")
    n = 224 * 64 + 1  # 65 launches of the batched kernel
    arr = (_lib.WorkItem * n)()
    args = pm.exec_args(B, C)
    for i in range(n):
        arr[i].a = pm.handle
        arr[i].args = args
    st = _lib.lib().spreg_execute_batched_noalloc(arr, n, _lib.stream_handle(None))
    assert st == _lib.SPREG_ERR_INVALID_ARG
    assert "at most 64" in _lib.last_error()


@pytest.mark.parametrize("kw", [dict(rounds=2, nr=32), dict(balance=1), dict(staging=1)])
def test_noalloc_refuses_the_b_tile_kernel_options(cuda, kw):
    """The no-allocation entry point runs the batched kernel alone: panel rounds, the load-balanced
    split and forced B tiles are refused with an error, nothing launched."""
    m = Mapping.identity(4)
    pm = PackedMatrix.from_dense(torch.from_numpy(synth.row_skew(256, 256, 0.9, seed=3)).cuda(), m, k_tile=64)
    B = torch.ones((256, 64), device="cuda")
    C = torch.zeros((256, 64), device="cuda")
    st = _lib.lib().spreg_execute_batched_noalloc(_work([(pm, B, C, kw)]), 1, _lib.stream_handle(None))
    assert st == _lib.SPREG_ERR_INVALID_ARG
    assert "batched execution-layout kernel only" in _lib.last_error()
    assert float(C.abs().sum()) == 0.0
