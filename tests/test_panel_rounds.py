"""Panel rounds of the B-tile kernel (spreg_exec_args.panel_rounds > 1): a job keeps its strip of B
for every K tile in shared memory while R rounds of its consumer warps' panels run against it.
Each output element is still one FMA chain (K tiles in order, entries in packed order), so every
case is compared bit for bit with the oracle's execution of the same packing
(sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:265-305) and with the kernel without rounds."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.packed import PackedMatrix, device_status, execute_batched

pytestmark = pytest.mark.gpu

TORCH = {_lib.F32: torch.float32, _lib.BF16: torch.bfloat16, _lib.F16: torch.float16}


def case(M, K, n, sparsity, seed, *, mr=4, k_tile=0, vd=_lib.F32, col_offset=0):
    m = Mapping.identity(mr)
    A = synth.row_skew(M, K, sparsity, seed=seed, std=1.0)
    B = synth.dense(K + col_offset, n, seed=seed + 1)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=k_tile, col_offset=col_offset, value_dtype=vd)
    ref = O.Packed(O.Tables.of(m), A, k_tile=k_tile, col_offset=col_offset, value_dtype=vd)
    Bt = torch.from_numpy(B).cuda().to(TORCH[vd])
    Bref = B if vd == _lib.F32 else Bt.cpu().view(torch.int16).numpy().view(np.uint16)
    return pm, Bt, ref.execute(Bref)


def bits(C):
    return C.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("k_tile", [0, 128, 200])
@pytest.mark.parametrize("nr", [32, 64])
@pytest.mark.parametrize("rounds", [2, 3, 8])
def test_rounds_fp32_bit_exact(cuda, k_tile, nr, rounds):
    # 1001 rows: 251 panels of M_r = 4 (the last one ragged), not a multiple of 15 x rounds
    pm, B, want = case(1001, 512, 160, 0.97, seed=rounds + nr + k_tile, k_tile=k_tile)
    C = pm.execute(B, nr=nr, rounds=rounds)
    assert np.array_equal(bits(C), want.view(np.uint32))
    assert torch.equal(C, pm.execute(B, nr=nr))  # the executor's own choice, without rounds
    assert device_status() == 0


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("warps", [0, 4])
def test_rounds_orders_and_cta_tiling(cuda, order, warps):
    pm, B, want = case(700, 384, 256, 0.95, seed=11, k_tile=128)
    C = pm.execute(B, nr=64, rounds=4, order=order, warps=warps)
    assert np.array_equal(bits(C), want.view(np.uint32))
    assert device_status() == 0


@pytest.mark.parametrize("vd", [_lib.BF16, _lib.F16])
@pytest.mark.parametrize("nr", [64, 128])
def test_rounds_16bit_storage(cuda, vd, nr):
    pm, B, want = case(513, 512, 296, 0.9, seed=5, vd=vd)  # 16-byte rows of 16-bit B
    C = pm.execute(B, nr=nr, rounds=4)
    assert np.array_equal(bits(C), want.view(np.uint32))
    assert device_status() == 0


def test_rounds_one_resident_strip(cuda):
    """FP32, K = 512, 64-column strips: a strip is 128 KB, so one resident strip and the producer
    waits for a job's last stage before it loads the next job's strip."""
    pm, B, want = case(2048, 512, 512, 0.98, seed=21)
    for rounds in (2, 8, 64):
        C = pm.execute(B, nr=64, rounds=rounds)
        assert np.array_equal(bits(C), want.view(np.uint32)), rounds
    assert device_status() == 0


def test_rounds_column_offset_and_automatic_width(cuda):
    pm, B, want = case(300, 256, 200, 0.9, seed=8, k_tile=64, col_offset=24)
    C = pm.execute(B, rounds=5)  # nr = 0: the widest strip whose K tiles all fit
    assert np.array_equal(bits(C), want.view(np.uint32))


def test_rounds_in_a_batched_launch(cuda):
    """Several SpMMs of different shapes in one launch, with and without rounds."""
    cases = [case(600 + 64 * i, 512, 256, 0.97 - 0.02 * (i % 3), seed=30 + i, k_tile=(0, 128)[i % 2])
             for i in range(6)]
    Cs = [torch.empty((pm.info["rows"], 256), device="cuda") for pm, _, _ in cases]
    execute_batched([(pm, B, C, dict(nr=64, rounds=(4, 1, 8)[i % 3])) for i, ((pm, B, _), C) in
                     enumerate(zip(cases, Cs))])
    torch.cuda.synchronize()
    for (_, _, want), C in zip(cases, Cs):
        assert np.array_equal(bits(C), want.view(np.uint32))
    assert device_status() == 0


def test_rounds_refusals(cuda):
    pm, B, _ = case(256, 1024, 128, 0.95, seed=2)
    with pytest.raises(_lib.SpregError, match="does not fit"):
        pm.execute(B, nr=128, rounds=4)  # 1024 x 128 FP32 = 512 KB
    with pytest.raises(_lib.SpregError, match="panel_rounds"):
        pm.execute(B, nr=32, rounds=4, staging=2)
    with pytest.raises(_lib.SpregError, match="panel_rounds"):
        pm.execute(B, nr=32, rounds=65)
