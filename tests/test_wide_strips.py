"""FP32 strips of 256 and 512 columns in the gather kernel (spreg_exec_args.nr = 256 / 512): lanes
hold 16-byte quarters of the strip, interleaved, and each packed entry's B row segment feeds 8 or
16 columns a lane.  Every output element is still one FMA chain in packed order (K tiles in order,
entries as packed), so each case is compared bit for bit with the oracle's execution of the same
packing (sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:265-305)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.packed import PackedMatrix, device_status, execute_batched

pytestmark = pytest.mark.gpu


def case(M, K, n, sparsity, seed, *, mr=4, mapping=None, k_tile=0, col_offset=0, sigma=0.5):
    m = mapping if mapping is not None else Mapping.identity(mr)
    A = synth.row_skew(M, K, sparsity, seed=seed, sigma=sigma, std=1.0)
    B = synth.dense(K + col_offset, n, seed=seed + 1)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=k_tile, col_offset=col_offset)
    ref = O.Packed(O.Tables.of(m), A, k_tile=k_tile, col_offset=col_offset)
    return pm, ref, torch.from_numpy(B).cuda(), B


def bits(C):
    return C.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("mr,nr", [(2, 256), (2, 512), (4, 256), (4, 512), (8, 256), (8, 512)])
@pytest.mark.parametrize("n", [512, 600, 1024])
def test_wide_strips_bit_exact(cuda, mr, nr, n):
    pm, ref, B, Bn = case(1001, 512, n, 0.97, seed=mr * 7 + nr + n, mr=mr)
    plan = pm.explain(B, torch.empty((1001, n), device="cuda"), nr=nr)
    width = 512 if (nr == 512 and mr <= 4) else 256
    assert plan["kernel"] == "exec_batch_kernel" and plan["strip_columns"] == width, plan
    C = pm.execute(B, nr=nr)
    assert np.array_equal(bits(C), ref.execute(Bn).view(np.uint32))
    assert device_status() == 0


@pytest.mark.parametrize("load_c,epilogue", [(True, 0), (False, 1), (True, 1)])
def test_wide_strips_load_c_relu_and_warps(cuda, load_c, epilogue):
    pm, ref, B, Bn = case(700, 384, 512, 0.95, seed=3, mr=2)
    C0 = synth.dense(700, 512, seed=99)
    for warps in (0, 1, 4, 8):
        Cg = torch.from_numpy(C0.copy()).cuda()
        pm.execute(B, Cg, load_c=load_c, epilogue=epilogue, nr=512, warps=warps)
        want = ref.execute(Bn, C0.copy() if load_c else None, load_c=load_c, epilogue=epilogue)
        assert np.array_equal(bits(Cg), want.view(np.uint32)), warps


def test_wide_strips_k_tiled_pack_through_the_gather_kernel(cuda):
    """A K-tiled pack with B staging 2 (the gather kernel): the accumulators stay in registers
    across K tiles."""
    pm, ref, B, Bn = case(513, 512, 768, 0.96, seed=8, mr=4, k_tile=128)
    C = pm.execute(B, nr=256, staging=2)
    assert pm.explain(B, C, nr=256, staging=2)["strip_columns"] == 256
    assert np.array_equal(bits(C), ref.execute(Bn).view(np.uint32))


def test_wide_strips_mapping_and_column_offset(cuda):
    pm, ref, B, Bn = case(640, 256, 512, 0.98, seed=12, mapping=Mapping.load("747f9"), col_offset=24)
    C = pm.execute(B, nr=256)
    assert np.array_equal(bits(C), ref.execute(Bn).view(np.uint32))


def test_wide_strips_strided_and_misaligned_operands_fall_back(cuda):
    """B and C row strides that are multiples of 4 floats keep the wide strips; a C that is not
    16-byte aligned takes narrower strips, with the same result."""
    pm, ref, B, Bn = case(300, 256, 520, 0.95, seed=4, mr=2)
    want = ref.execute(Bn)
    Cbig = torch.zeros((300, 528), device="cuda")
    C = Cbig[:, :520]
    assert pm.explain(B, C, nr=512)["strip_columns"] == 512
    pm.execute(B, C, nr=512)
    assert np.array_equal(bits(C.contiguous()), want.view(np.uint32))
    Codd = torch.zeros((300, 521), device="cuda")[:, 1:]
    assert pm.explain(B, Codd, nr=512)["strip_columns"] < 256
    pm.execute(B, Codd, nr=512)
    assert np.array_equal(bits(Codd.contiguous()), want.view(np.uint32))


def test_wide_strips_batched_with_other_widths_and_a_graph(cuda):
    cases = [case(400 + 96 * i, 512, 512, 0.9 + 0.02 * (i % 4), seed=40 + i, mr=(2, 4)[i % 2]) for i in range(6)]
    Cs = [torch.empty((pm.info["rows"], 512), device="cuda") for pm, _, _, _ in cases]
    work = [(pm, B, C, dict(nr=(512, 256, 128)[i % 3])) for i, ((pm, _, B, _), C) in enumerate(zip(cases, Cs))]
    execute_batched(work)
    torch.cuda.synchronize()
    wants = [ref.execute(Bn) for _, ref, _, Bn in cases]
    for C, want in zip(Cs, wants):
        assert np.array_equal(bits(C), want.view(np.uint32))
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        execute_batched(work)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        execute_batched(work)
    for C in Cs:
        C.zero_()
    g.replay()
    torch.cuda.synchronize()
    for C, want in zip(Cs, wants):
        assert np.array_equal(bits(C), want.view(np.uint32))
    assert device_status() == 0


TORCH16 = {_lib.BF16: torch.bfloat16, _lib.F16: torch.float16}


@pytest.mark.parametrize("vd", [_lib.BF16, _lib.F16])
@pytest.mark.parametrize("mr,n", [(2, 512), (4, 512), (4, 600), (4, 264)])
def test_16bit_gather_strips(cuda, vd, mr, n):
    """16-bit B on the gather kernel (untiled packs): nr = 256 runs 256-column strips (8 contiguous
    columns a lane), nr = 512 512-column strips (8 a lane in each 256-column half) when n reaches
    512, both with the mixed-precision FMA; bit-exact with the oracle."""
    m = Mapping.identity(mr)
    A = synth.row_skew(777, 512, 0.97, seed=mr + n, sigma=0.5, std=1.0)
    Bf = synth.dense(512, n, seed=5)
    B = torch.from_numpy(Bf).cuda().to(TORCH16[vd])
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, value_dtype=vd)
    want = O.Packed(O.Tables.of(m), A, value_dtype=vd).execute(B.cpu().view(torch.int16).numpy().view(np.uint16))
    for nr in (256, 512):
        C = torch.empty((777, n), device="cuda")
        plan = pm.explain(B, C, nr=nr)
        width = 512 if (nr == 512 and n >= 512) else 256
        assert (plan["kernel"], plan["strip_columns"]) == ("exec_batch_kernel", width), plan
        pm.execute(B, C, nr=nr)
        assert np.array_equal(bits(C), want.view(np.uint32)), nr
    assert device_status() == 0


def test_16bit_gather_strips_load_c_bf16_out_and_mr8(cuda):
    m = Mapping.identity(4)
    A = synth.row_skew(500, 384, 0.95, seed=9, std=1.0)
    B = torch.from_numpy(synth.dense(384, 512, seed=2)).cuda().bfloat16()
    Bref = B.cpu().view(torch.int16).numpy().view(np.uint16)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, value_dtype=_lib.BF16)
    ref = O.Packed(O.Tables.of(m), A, value_dtype=_lib.BF16)
    C0 = synth.dense(500, 512, seed=3)
    want = ref.execute(Bref, C0.copy(), load_c=True, epilogue=_lib.EPILOGUE_RELU)
    for nr in (256, 512):
        C = torch.from_numpy(C0.copy()).cuda()
        pm.execute(B, C, load_c=True, epilogue=_lib.EPILOGUE_RELU, nr=nr)
        assert np.array_equal(bits(C), want.view(np.uint32)), nr
        # BF16 output: the FP32 result rounded once
        Cb = torch.empty((500, 512), device="cuda", dtype=torch.bfloat16)
        pm.execute(B, Cb, nr=nr)
        assert torch.equal(Cb.cpu(), torch.from_numpy(ref.execute(Bref)).bfloat16()), nr
    # M_r = 8 keeps 128-column strips for 16-bit B
    m8 = Mapping.load("747f9")
    p8 = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m8, value_dtype=_lib.BF16)
    assert p8.explain(B, torch.empty((500, 512), device="cuda"), nr=256)["strip_columns"] == 128


def test_nr_values_outside_the_set_are_refused(cuda):
    pm, _, B, _ = case(128, 128, 512, 0.9, seed=1, mr=2)
    with pytest.raises(_lib.SpregError, match="nr must be"):
        pm.execute(B, nr=384)
