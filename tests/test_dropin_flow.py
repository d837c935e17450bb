"""The reference benchmark's own call sequence (sbench/SOP/sop_bench.py:150-210) against this
package: a 48 x 256 tile at 70-95 % sparsity, B = ones(256, 128); the CSR baseline, then SOP
modules for M_r 4 / 6 / 8 with their nanokernel sets and mappings, each result checked with
torch.allclose against tile @ B, and the mapping saved under its file id."""
import pytest
import torch

from oracle import oracle as O

from spreg import synth
from spreg.mapping import Mapping
from spreg.sop_driver import Acc, csr, make_sop_module
from spreg.sop_utils import save_mapping

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sparsity", [0.7, 0.8, 0.9, 0.95])
def test_sop_bench_sequence(cuda, tmp_path, sparsity):
    # a 0/1 tile as the reference's random_sp_matrix (sop_bench.py:49-50): with B = ones, C = row nnz
    tile = (torch.from_numpy(synth.bernoulli(48, 256, sparsity, seed=int(sparsity * 100))) != 0).float()
    bcols = 128
    B = torch.ones((256, bcols))
    sol = tile @ B
    assert torch.equal(sol[:, 0], tile.sum(1))

    t, result = csr.executor(tile.to_sparse_csr(), B, 16, min(bcols, 64))
    assert t > 0 and torch.allclose(result, sol)

    strategies = [(4, Mapping.identity(4)), (6, Mapping.identity(6)), (8, Mapping.load("400fa")),
                  (8, Mapping.load("747f9"))]
    for mr, mapping in strategies:
        module = make_sop_module(Acc(mr, 2), mapping.nanokernels, mapping)
        sop_tile = module.make_sop_tile(tile)
        t, result = module.execute_tile(sop_tile, B, 16)
        assert t > 0 and torch.allclose(result, sol), (mr, mapping.mapping_id)
        want_pad = O.Packed(O.Tables.of(mapping), tile.numpy()).sizes["padding"]
        assert sop_tile.padding() == want_pad and (want_pad == 0 or mr == 8)
        mid = save_mapping(mr, mapping, subdir="m", root=str(tmp_path))
        assert mid == mapping.mapping_id
