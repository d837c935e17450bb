"""Load-balanced SpMM (spreg_exec_args.load_balance, the reference's load-balanced kernel choice in
cpp_testbed/src/spmm/nano/runtime_yaml_config.register:84-99): when a launch leaves SMs idle, the
heaviest groups of row panels have their K tiles split between two concurrent jobs, C = (tiles
[0, split) from C or zero) + (tiles [split, T) from zero), one FP32 add per element, then the
epilogue.  Every case is compared bit for bit with the oracle's restatement of that order
(oracle.load_balanced_execute), and within FP32 rounding with the unsplit executor."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.matmul import MatMulSpecialized, TileConfig
from spreg.packed import PackedMatrix, device_status, execute_batched

pytestmark = pytest.mark.gpu

TORCH = {_lib.F32: torch.float32, _lib.BF16: torch.bfloat16}


def skewed(M, K, seed, sparsity=0.9, sigma=1.2):
    """Log-normal row skew strong enough for a heavy tail of row panels."""
    return synth.row_skew(M, K, sparsity, seed=seed, sigma=sigma, std=1.0)


def run(A, k_tile, n=256, vd=_lib.F32, load_c=False, epilogue=0, mr=4, **kw):
    m = Mapping.identity(mr)
    B = synth.dense(A.shape[1], n, seed=7)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=k_tile, value_dtype=vd)
    Bt = torch.from_numpy(B).cuda().to(TORCH[vd])
    Bref = B if vd == _lib.F32 else Bt.cpu().view(torch.int16).numpy().view(np.uint16)
    C0 = synth.dense(A.shape[0], n, seed=8)
    Cg = torch.from_numpy(C0.copy()).cuda()
    H, split, heavy = pm.load_balance_plan(Bt, Cg, **kw)
    pm.execute(Bt, Cg, load_c=load_c, epilogue=epilogue, balance=1, **kw)
    want = O.load_balanced_execute(O.Tables.of(m), A, Bref, heavy, split, k_tile, value_dtype=vd,
                                   out=C0.copy() if load_c else None, load_c=load_c, epilogue=epilogue)
    plain = O.Packed(O.Tables.of(m), A, k_tile=k_tile, value_dtype=vd).execute(
        Bref, C0.copy() if load_c else None, load_c=load_c, epilogue=epilogue)
    return Cg.cpu().numpy(), want, plain, (H, split, heavy)


@pytest.mark.parametrize("k_tile", [64, 128])
@pytest.mark.parametrize("mr", [4, 8])
def test_split_matches_the_stated_order(cuda, k_tile, mr):
    A = skewed(1500, 512, seed=k_tile + mr)
    got, want, plain, (H, split, heavy) = run(A, k_tile, mr=mr)
    assert H > 0 and split == (512 // k_tile) // 2 and len(heavy) == H
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert O.rel_err(got, plain) < 1e-6
    assert device_status() == 0


@pytest.mark.parametrize("load_c,epilogue", [(True, 0), (False, 1), (True, 1)])
def test_split_with_load_c_and_relu(cuda, load_c, epilogue):
    A = skewed(900, 384, seed=3)
    got, want, plain, (H, _, _) = run(A, 64, load_c=load_c, epilogue=epilogue)
    assert H > 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_split_bf16_values_and_ragged_columns(cuda):
    A = skewed(777, 512, seed=5)
    got, want, plain, (H, _, _) = run(A, 128, n=296, vd=_lib.BF16)
    assert H > 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_split_with_panel_rounds_and_strip_widths(cuda):
    A = skewed(1200, 512, seed=9, sparsity=0.96)
    for nr, rounds in ((32, 4), (64, 2), (128, 0)):
        got, want, _, (H, _, _) = run(A, 128, nr=nr, rounds=rounds)
        assert H > 0
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (nr, rounds)


def test_uniform_matrix_alone_is_split(cuda):
    """Uniform nonzeros, a single SpMM whose groups all fit the idle SMs twice over (128-column strips):
    every group is split (halving each job); with 32-column strips only one group would fit, which
    would not shorten the longest job, so nothing is split."""
    A = synth.bernoulli(1024, 512, 0.9, seed=1, std=1.0)
    got, want, plain, (H, split, _) = run(A, 128, nr=128)
    assert H == 256 and split == 2
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    got, _, plain, (H, split, _) = run(A, 128, nr=32)
    assert (H, split) == (0, 0)
    assert np.array_equal(got.view(np.uint32), plain.view(np.uint32))


def test_full_launch_is_not_split(cuda):
    """A launch with at least one job per SM is balanced by the work counter: nothing is split and
    the result is the executor's own chain."""
    A = skewed(8192, 512, seed=6)
    got, want, plain, (H, split, _) = run(A, 128, n=512)
    assert (H, split) == (0, 0)
    assert np.array_equal(got.view(np.uint32), plain.view(np.uint32))


def test_untiled_pack_is_not_split(cuda):
    A = skewed(1000, 256, seed=4)
    got, _, plain, (H, _, _) = run(A, 0)
    assert H == 0
    assert np.array_equal(got.view(np.uint32), plain.view(np.uint32))


def test_split_in_a_batched_launch_and_a_cuda_graph(cuda):
    m = Mapping.identity(4)
    As = [skewed(1000 + 200 * i, 512, seed=20 + i) for i in range(3)]
    packs = [PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=128) for A in As]
    Bs = [torch.from_numpy(synth.dense(512, 256, seed=30 + i)).cuda() for i in range(3)]
    Cs = [torch.empty((A.shape[0], 256), device="cuda") for A in As]
    # a fixed strip width: alone and in the launch the SpMM has the same strips
    work = [(p, B, C, dict(balance=i % 2 ^ 1, nr=128)) for i, (p, B, C) in enumerate(zip(packs, Bs, Cs))]
    execute_batched(work)
    torch.cuda.synchronize()
    # in a launch with other SpMMs fewer SMs are idle, so a balanced SpMM splits at most the groups it
    # splits alone (same strips): its result is the stated order for one of those group counts
    wants = []
    for i, (A, p, B, C) in enumerate(zip(As, packs, Bs, Cs)):
        got = C.cpu().numpy()
        if i % 2 == 0:
            H, split, heavy = p.load_balance_plan(B, C, nr=128)
            assert H > 0
            counts = sorted({min(15 * g, H) for g in range(0, H // 15 + 2)}, reverse=True)  # whole groups of 15
            cands = [O.load_balanced_execute(O.Tables.of(m), A, B.cpu().numpy(), heavy[:h], split, 128)
                     for h in counts]
            match = [w for w in cands if np.array_equal(got.view(np.uint32), w.view(np.uint32))]
            assert match, i
            wants.append(match[0])
        else:
            wants.append(O.Packed(O.Tables.of(m), A, k_tile=128).execute(B.cpu().numpy()))
            assert np.array_equal(got.view(np.uint32), wants[-1].view(np.uint32))
    # the same launch captured in a CUDA graph (the scratch is stream-ordered) and replayed
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        execute_batched(work)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        execute_batched(work)
    for C in Cs:
        C.zero_()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for C, want in zip(Cs, wants):
        assert np.array_equal(C.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert device_status() == 0


def test_matmul_specialized_load_balanced(cuda):
    m = Mapping.identity(4)
    A = skewed(800, 512, seed=12)
    B = synth.dense(512, 128, seed=13)
    rp, ci, v = synth.to_csr(A)
    mm = MatMulSpecialized(800, 512, 128, v, rp, ci, TileConfig(K_c=128, load_balance=1), 1, "", m)
    C = torch.zeros((800, 128))
    mm(C, torch.from_numpy(B))
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=128)
    H, split, heavy = pm.load_balance_plan(torch.from_numpy(B).cuda(), torch.empty((800, 128), device="cuda"))
    assert H > 0
    want = O.load_balanced_execute(O.Tables.of(m), A, B, heavy, split, 128)
    assert np.array_equal(C.numpy().view(np.uint32), want.view(np.uint32))


def test_load_balance_refusals(cuda):
    A = skewed(512, 512, seed=2)
    m = Mapping.identity(4)
    B = torch.from_numpy(synth.dense(512, 64, seed=1)).cuda()
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=128)
    with pytest.raises(_lib.SpregError, match="load_balance"):
        pm.execute(B, balance=1, staging=2)
    with pytest.raises(_lib.SpregError, match="load_balance"):
        pm.execute(B, balance=2)
    p16 = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=128, value_dtype=_lib.F16)
    with pytest.raises(_lib.SpregError, match="load_balance"):
        p16.execute(B.half(), balance=1)
