"""The reference's CSR baseline (`csr.executor`, pytorch_csr_wrapper.cpp:314-353) as a CUDA kernel:
bit-exact with the restated baseline (row x N-tile FMAs in CSR order), its argument checks, and
the bounds guard on a malformed CSR."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.packed import device_status
from spreg.sop_driver import csr

pytestmark = pytest.mark.gpu


def _csr_tensor(A):
    return torch.from_numpy(A).to_sparse_csr()


@pytest.mark.parametrize("n_tile", [16, 32, 64, 128])
@pytest.mark.parametrize("shape,n,sp", [((70, 300), 96, 0.85), ((257, 129), 131, 0.9), ((33, 512), 1, 0.7),
                                        ((512, 512), 256, 0.8), ((5, 64), 37, 0.5)])
def test_csr_executor_bit_exact(cuda, n_tile, shape, n, sp):
    A = synth.row_skew(*shape, sp, seed=shape[0] + n, std=1.0)
    A[3] = 0.0  # an empty row
    B = synth.dense(shape[1], n, seed=n)
    t, Cg = csr.executor(_csr_tensor(A), torch.from_numpy(B).cuda(), num_runs=1, n_tile=n_tile)
    rp, ci, v = synth.to_csr(A)
    want = O.csr_spmm(rp, ci, v, B)
    assert Cg.is_cuda and t > 0
    assert np.array_equal(Cg.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert O.rel_err(Cg.cpu().numpy(), O.dense_fp64(A, B)) <= 1e-5


def test_csr_executor_cpu_b_and_empty_matrix(cuda):
    A = np.zeros((40, 64), np.float32)
    B = synth.dense(64, 48, seed=1)
    t, Cc = csr.executor(_csr_tensor(A), torch.from_numpy(B), num_runs=2, n_tile=32)
    assert not Cc.is_cuda and torch.count_nonzero(Cc) == 0
    A[7, 5] = 2.0
    _, Cc = csr.executor(_csr_tensor(A), torch.from_numpy(B), num_runs=1, n_tile=64)
    assert np.array_equal(Cc[7].numpy(), 2.0 * B[5]) and torch.count_nonzero(Cc[:7]) == 0


def test_csr_executor_argument_errors(cuda):
    A = synth.row_skew(16, 32, 0.8, seed=2, std=1.0)
    B = torch.ones((32, 8), device="cuda")
    with pytest.raises(_lib.SpregError, match="n_tile"):
        csr.executor(_csr_tensor(A), B, num_runs=1, n_tile=48)
    with pytest.raises(RuntimeError, match="size mismatch"):
        csr.executor(_csr_tensor(A), torch.ones((31, 8), device="cuda"), num_runs=1)
    with pytest.raises(RuntimeError, match="sparse CSR"):
        csr.executor(torch.from_numpy(A), B, num_runs=1)


def test_csr_bad_column_index_is_guarded(cuda):
    """A column index past B's rows contributes nothing and sets the device status word; the
    other entries are still summed in order."""
    device_status(reset=True)
    rp = torch.tensor([0, 2, 3], dtype=torch.int32, device="cuda")
    ci = torch.tensor([1, 9, 0], dtype=torch.int32, device="cuda")  # 9 >= cols = 4
    v = torch.tensor([2.0, 5.0, 3.0], device="cuda")
    B = torch.arange(16, dtype=torch.float32, device="cuda").reshape(4, 4)
    Cd = torch.full((2, 4), -1.0, device="cuda")
    _lib.check(_lib.lib().spreg_csr_spmm(2, 4, 4, 3, rp.data_ptr(), ci.data_ptr(), v.data_ptr(), B.data_ptr(), 4,
                                         Cd.data_ptr(), 4, 64, _lib.stream_handle(None)))
    torch.cuda.synchronize()
    assert torch.equal(Cd[0], 2.0 * B[1]) and torch.equal(Cd[1], 3.0 * B[0])
    assert device_status(reset=True) == 20
    assert device_status() == 0
