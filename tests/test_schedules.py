"""Outer schedules (tools/paper/configs.py:9-25; SOPConfig's schedule, cpp_testbed/src/spmm/nano/
SpMM_SOP.h:33-54): on the GPU the K loop runs inside every job, so a schedule decides whether column
strips or row panels are handed out outermost (spreg_exec_args.job_order).  The order changes which
jobs run together, never an element's FMA chain, so every order gives the oracle's bits."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.matmul import SCHEDULES, MatMulSpecialized, TileConfig
from spreg.packed import PackedMatrix, execute_batched

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k_tile,staging", [(0, 0), (0, 2), (128, 0), (128, 1)])
@pytest.mark.parametrize("dtype", [_lib.F32, _lib.BF16])
def test_job_orders_give_the_oracle_bits(cuda, k_tile, staging, dtype):
    import torch
    m = Mapping.identity(4)
    A = synth.row_skew(700, 384, 0.85, seed=3, std=1.0)
    tdt = torch.float32 if dtype == _lib.F32 else torch.bfloat16
    B = torch.from_numpy(synth.dense(384, 296, seed=4)).cuda().to(tdt)  # 16-byte rows in both types
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=k_tile, value_dtype=dtype)
    Bref = B.cpu().numpy() if dtype == _lib.F32 else B.cpu().view(torch.int16).numpy().view(np.uint16)
    want = O.Packed(O.Tables.of(m), A, k_tile=k_tile, value_dtype=dtype).execute(Bref)
    outs = []
    for order in (0, 1):
        C = pm.execute(B, staging=staging, order=order)
        outs.append(C)
        assert np.array_equal(C.cpu().numpy().view(np.uint32), want.view(np.uint32)), order
    # in one batched launch with other SpMMs, both orders mixed
    Cs = [torch.empty_like(outs[0]) for _ in range(4)]
    execute_batched([(pm, B, C, dict(order=i % 2, staging=staging)) for i, C in enumerate(Cs)])
    torch.cuda.synchronize()
    for C in Cs:
        assert torch.equal(C, outs[0])


def test_bad_job_order_is_refused(cuda):
    import torch
    pm = PackedMatrix.from_dense(torch.from_numpy(synth.bernoulli(8, 32, 0.5, seed=1)).cuda(), Mapping.identity(4))
    B = torch.ones((32, 32), device="cuda")
    with pytest.raises(_lib.SpregError, match="job_order"):
        pm.execute(B, order=2)


@pytest.mark.parametrize("schedule", ["KNM", "NKM", "MNK", "KMN"])
def test_matmul_outer_schedules(cuda, schedule):
    import torch
    m = Mapping.identity(4)
    A = synth.row_skew(300, 200, 0.9, seed=5, std=1.0)
    B = synth.dense(200, 96, seed=6)
    rp, ci, v = synth.to_csr(A)
    mm = MatMulSpecialized(300, 200, 96, v, rp, ci, TileConfig(K_c=64, runtimeSchedule=SCHEDULES[schedule]), 1, "", m)
    C = torch.zeros((300, 96))
    mm(C, torch.from_numpy(B))
    want = O.Packed(O.Tables.of(m), A, k_tile=64).execute(B)
    assert np.array_equal(C.numpy().view(np.uint32), want.view(np.uint32))
