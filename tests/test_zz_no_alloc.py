"""spreg_execute_batched_noalloc: the executor entry point for callers that cannot allocate device
memory while it runs (for example a serving loop whose device memory is owned by another
allocator).  It must give the same bits as spreg_execute_batched, call after call, with its
scratch in the library's static device array.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.packed import PackedMatrix

pytestmark = pytest.mark.gpu


def _work(items):
    arr = (_lib.WorkItem * len(items))()
    for i, (pm, B, C) in enumerate(items):
        arr[i].a = pm.handle
        arr[i].args = pm.exec_args(B, C)
    return arr


def test_noalloc_matches_batched_twice(cuda):
    cases = [(256, 512, 128, Mapping.identity(4), _lib.F32), (130, 300, 77, Mapping.load("400fa"), _lib.F32),
             (512, 256, 96, Mapping.identity(4), _lib.BF16)]
    ref_items, na_items = [], []
    for i, (M, K, N, m, vd) in enumerate(cases):
        A = synth.row_skew(M, K, 0.85, seed=40 + i, std=1.0)
        tdt = torch.float32 if vd == _lib.F32 else torch.bfloat16
        B = torch.from_numpy(synth.dense(K, N, seed=50 + i)).to(tdt).cuda()
        pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, value_dtype=vd)
        ref_items.append((pm, B, torch.zeros((M, N), device="cuda")))
        na_items.append((pm, B, torch.zeros((M, N), device="cuda")))
    L = _lib.lib()
    stream = _lib.stream_handle(None)
    ref = _work(ref_items)
    _lib.check(L.spreg_execute_batched(ref, len(ref_items), stream))
    na = _work(na_items)
    for call in range(2):
        for _, _, C in na_items:
            C.fill_(-1.0)
        _lib.check(L.spreg_execute_batched_noalloc(na, len(na_items), stream))
        torch.cuda.synchronize()
        for (_, _, Cr), (_, _, Cn) in zip(ref_items, na_items):
            assert torch.equal(Cr, Cn), f"call {call}"
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
