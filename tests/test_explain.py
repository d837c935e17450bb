"""spreg_execute_explain: the plan spreg_execute makes for a call (kernel, strip width, columns of
the whole strips and of the 32-column tail, K tiles, warps, panel rounds, load-balanced split), with
no launch."""
import pytest
import torch

from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.packed import PackedMatrix

pytestmark = pytest.mark.gpu


def packed(M, K, k_tile, vd=_lib.F32, sparsity=0.9):
    A = synth.row_skew(M, K, sparsity, seed=1, std=1.0)
    return PackedMatrix.from_dense(torch.from_numpy(A).cuda(), Mapping.identity(4), k_tile=k_tile, value_dtype=vd)


def test_strip_width_and_tail_follow_nr(cuda):
    pm = packed(2048, 512, 128)
    B = torch.randn((512, 3136), device="cuda")
    C = torch.empty((2048, 3136), device="cuda")
    e = pm.explain(B, C, nr=128)
    assert e["kernel"] == "exec_tile_kernel" and e["k_tiles"] == 4 and e["k_tile"] == 128
    # the 64 columns past the last whole 128-column strip are one more (masked) strip of the same launch
    assert (e["nv"], e["main_columns"], e["tail_columns"]) == (4, 3136, 0), e
    e = pm.explain(B, C, nr=64)
    assert (e["nv"], e["main_columns"], e["tail_columns"]) == (2, 3136, 0), e


def test_wide_strips_for_16bit_b(cuda):
    pm = packed(2048, 512, 128, vd=_lib.BF16)
    B = torch.randn((512, 3136), device="cuda").to(torch.bfloat16)
    C = torch.empty((2048, 3136), device="cuda")
    e = pm.explain(B, C, nr=256)
    assert e["kernel"] == "exec_tile_kernel" and e["nv"] == 8, e


def test_untiled_pack_runs_the_batched_kernel_and_rounds_the_tile_kernel(cuda):
    pm = packed(1024, 512, 0, sparsity=0.98)
    B = torch.randn((512, 512), device="cuda")
    C = torch.empty((1024, 512), device="cuda")
    assert pm.explain(B, C, nr=128)["kernel"] == "exec_batch_kernel"
    e = pm.explain(B, C, nr=64, rounds=4)
    assert (e["kernel"], e["rounds"], e["nv"]) == ("exec_tile_kernel", 4, 2), e


def test_explain_refuses_what_execute_refuses(cuda):
    pm = packed(256, 256, 64)
    B = torch.randn((256, 64), device="cuda")
    C = torch.empty((256, 64), device="cuda")
    with pytest.raises(_lib.SpregError, match="nr must be"):
        pm.explain(B, C, nr=48)


def test_tail_needs_whole_lane_columns(cuda):
    """n not a multiple of the lane's columns: the tail keeps 32-column strips of their own."""
    pm = packed(512, 256, 64)
    B = torch.randn((256, 200), device="cuda")  # 200 = 1 x 128 + 72; 200 % 4 == 0: merged
    C = torch.empty((512, 200), device="cuda")
    assert (pm.explain(B, C, nr=128)["main_columns"], pm.explain(B, C, nr=128)["tail_columns"]) == (200, 0)
    Bo = torch.randn((256, 203), device="cuda")[:, :202]  # 202: 2 leftover columns in a lane, rows 16-byte aligned
    Bp = torch.zeros((256, 204), device="cuda")
    Bp[:, :202] = Bo
    Cp = torch.empty((512, 204), device="cuda")
    e = pm.explain(Bp, Cp, n=202, nr=128, staging=1)
    assert (e["main_columns"], e["tail_columns"]) == (128, 74), e
