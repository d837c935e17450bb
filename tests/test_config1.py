"""The minimum slice as the workload states it: A 512 x 512 at 80 % sparsity with Bernoulli-uniform
unstructured nonzeros (sbench/SOP/sop_bench.py:49-50 draws its masks the same way), values N(0, 1);
B dense 512 x 256 FP32 N(0, 1); fixed seed; packed with M_r = 4 and the identity mapping 61fee,
executed with N_r = 64.

It is packed by the GPU packer (arena and descriptors byte for byte the oracle's restatement of
SOPTile::pack_panel / pack_tile, sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:129-261),
executed bit-exact against the oracle's executor (template:265-305), and checked against FP64 with
rel err <= 1e-5 -- through the C ABI directly, through the reference's Python surface
(make_sop_module / execute_tile, sbench/SOP/sop_driver.py:38-129) and through MatMulSpecialized
(cpp_testbed/src/spmm/nano/SpMM_SOP.h:107-178) with host buffers."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.matmul import MatMulSpecialized, TileConfig
from spreg.packed import PackedMatrix, device_status
from spreg.sop_driver import Acc, make_sop_module

pytestmark = pytest.mark.gpu

M, K, N, SPARSITY, SEED = 512, 512, 256, 0.8, 0


def config1():
    A = synth.bernoulli(M, K, SPARSITY, seed=SEED, std=1.0)
    B = synth.dense(K, N, seed=SEED + 1, std=1.0)
    return A, B


def test_config1_inputs_are_the_stated_workload():
    A, B = config1()
    assert A.shape == (512, 512) and B.shape == (512, 256)
    assert abs(synth.sparsity_of(A) - 0.8) < 0.01
    assert abs(float(A[A != 0].std()) - 1.0) < 0.05 and abs(float(B.std()) - 1.0) < 0.05
    assert Mapping.identity(4).mapping_id == "61fee"


def test_config1_pack_execute_bit_exact_and_fp64(cuda):
    A, B = config1()
    m = Mapping.identity(4)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m)
    ref = O.Packed(O.Tables.of(m), A)
    arena, descs, _ = pm.to_host()
    assert np.array_equal(arena, ref.arena) and np.array_equal(descs, ref.descs)
    assert pm.info["padding"] == 0 and pm.info["num_values"] == int(np.count_nonzero(A))  # template:214
    C = pm.execute(torch.from_numpy(B).cuda(), nr=64).cpu().numpy()
    want = ref.execute(B)
    assert np.array_equal(C.view(np.uint32), want.view(np.uint32))
    assert O.rel_err(C, O.dense_fp64(A, B)) <= 1e-5
    assert device_status() == 0


def test_config1_reference_python_surface(cuda):
    """make_sop_module(Acc(4, N_r = 64 floats = 4 x 16), ...) / make_sop_tile / execute_tile."""
    A, B = config1()
    m = Mapping.identity(4)
    module = make_sop_module(Acc(4, 4), m.nanokernels, m)
    tile = module.make_sop_tile(torch.from_numpy(A))
    t, C = module.execute_tile(tile, torch.from_numpy(B), 4)
    assert t > 0 and tile.padding() == 0
    want = O.Packed(O.Tables.of(m), A).execute(B)
    assert np.array_equal(C.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_config1_matmul_specialized_host_buffers(cuda):
    A, B = config1()
    m = Mapping.identity(4)
    rp, ci, v = synth.to_csr(A)
    mm = MatMulSpecialized(M, K, N, v, rp, ci, TileConfig(nr=64), 1, "", m)
    C = torch.zeros((M, N), dtype=torch.float32)
    mm(C, torch.from_numpy(B))
    want = O.Packed(O.Tables.of(m), A).execute(B)
    assert np.array_equal(C.numpy().view(np.uint32), want.view(np.uint32))


def test_config1_cpu_baseline_matches(cuda):
    """The timed CPU baseline (SIMD restatement of the executor) gives the same bits on this config."""
    A, B = config1()
    pk = O.Packed(O.Tables.of(Mapping.identity(4)), A)
    assert np.array_equal(pk.execute_fast(B).view(np.uint32), pk.execute(B).view(np.uint32))
