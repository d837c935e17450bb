"""Executor with B tiles staged in shared memory (b_staging = 1): bit-exact with the oracle.

The tile kernel runs K-tiled packs: per job it copies each K tile's B rows for one strip into
shared memory and gathers from there.  Every output element is the same FMA chain as the other
executors, so results are compared bit for bit against the oracle's tiled execution.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.packed import PackedMatrix, device_status, execute_batched

pytestmark = pytest.mark.gpu

TORCH = {_lib.F32: torch.float32, _lib.BF16: torch.bfloat16, _lib.F16: torch.float16}


def padded(B: np.ndarray, dt, ld: int):
    """Device copy of B (K x n) in a K x ld buffer (ld >= n), as a K x n view."""
    K, n = B.shape
    buf = torch.zeros((K, ld), dtype=dt, device="cuda")
    buf[:, :n] = torch.from_numpy(B).to(dt)
    return buf[:, :n]


def run_pair(A, m, B, *, k_tile, m_tile=0, value_dtype=_lib.F32, c_dtype=_lib.F32, nr=0, ld=None, load_c=False,
             epilogue=0, col_offset=0, C0=None):
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, m_tile=m_tile, k_tile=k_tile,
                                 col_offset=col_offset, value_dtype=value_dtype)
    ref = O.Packed(O.Tables.of(m), A, m_tile=m_tile, k_tile=k_tile, col_offset=col_offset, value_dtype=value_dtype)
    n = B.shape[1]
    tb = padded(B, TORCH[value_dtype], ld or n)
    Bref = B if value_dtype == _lib.F32 else tb.cpu().contiguous().view(torch.int16).numpy().view(np.uint16)
    out_t = torch.float32 if c_dtype == _lib.F32 else torch.bfloat16
    Cg = torch.zeros((A.shape[0], n), dtype=out_t, device="cuda")
    Cr = np.zeros((A.shape[0], n), dtype=np.float32 if c_dtype == _lib.F32 else np.uint16)
    if C0 is not None:
        Cg.copy_(torch.from_numpy(C0).to(out_t))
        Cr[...] = C0 if c_dtype == _lib.F32 else Cg.cpu().view(torch.int16).numpy().view(np.uint16)
    pm.execute(tb, Cg, nr=nr, load_c=load_c, epilogue=epilogue, staging=1)
    ref.execute(Bref, Cr, load_c=load_c, epilogue=epilogue, c_dtype=c_dtype)
    got = Cg.cpu()
    got = got.numpy() if c_dtype == _lib.F32 else got.view(torch.int16).numpy().view(np.uint16)
    return got, Cr


def same_bits(a, b):
    if a.dtype == np.float32:
        return np.array_equal(a.view(np.uint32), b.view(np.uint32))
    return np.array_equal(a, b)


@pytest.mark.parametrize("mr,mp", [(2, None), (4, None), (6, None), (8, None), (8, "400fa"), (8, "747f9")])
@pytest.mark.parametrize("k_tile", [64, 128, 200])
def test_tile_kernel_fp32_bit_exact(cuda, mr, mp, k_tile):
    m = Mapping.load(mp) if mp else Mapping.identity(mr)
    A = synth.row_skew(150, 520, 0.88, seed=mr * 7 + k_tile, std=1.0)
    B = synth.dense(520, 96, seed=3)
    got, want = run_pair(A, m, B, k_tile=k_tile)
    assert same_bits(got, want)
    assert device_status() == 0


@pytest.mark.parametrize("nr", [32, 64, 128])
@pytest.mark.parametrize("n,ld", [(512, 512), (100, 100), (37, 40), (1, 4), (130, 136)])
def test_tile_kernel_widths_and_ragged_columns(cuda, nr, n, ld):
    m = Mapping.identity(4)
    A = synth.row_skew(257, 384, 0.9, seed=n, std=1.0)
    B = synth.dense(384, n, seed=n + 1)
    got, want = run_pair(A, m, B, k_tile=128, nr=nr, ld=ld)
    assert same_bits(got, want)


@pytest.mark.parametrize("vd,cd", [(_lib.BF16, _lib.F32), (_lib.BF16, _lib.BF16), (_lib.F16, _lib.F32)])
@pytest.mark.parametrize("load_c,epi", [(False, 0), (True, 1)])
def test_tile_kernel_dtypes_load_c_epilogue(cuda, vd, cd, load_c, epi):
    m = Mapping.identity(4)
    A = synth.row_skew(203, 1000, 0.9, seed=5, std=0.5)
    B = synth.dense(1000, 72, seed=6)
    C0 = synth.dense(203, 72, seed=7) if load_c else None
    got, want = run_pair(A, m, B, k_tile=256, value_dtype=vd, c_dtype=cd, load_c=load_c, epilogue=epi, C0=C0,
                         ld=80)
    assert same_bits(got, want)


def test_tile_kernel_row_tiles_and_col_offset(cuda):
    m = Mapping.load("400fa")
    A = synth.row_skew(300, 260, 0.85, seed=9, std=1.0)
    off = 12
    Bfull = synth.dense(260 + off + 5, 64, seed=10)
    got, want = run_pair(A, m, Bfull, k_tile=96, m_tile=48, col_offset=off)
    assert same_bits(got, want)


def test_tile_kernel_full_size_ffn(cuda):
    """A 2048 x 512 @ 90 % (row skew), N = 512, K tiles of 128: bit-exact, and rel err vs FP64."""
    m = Mapping.identity(4)
    A = synth.row_skew(2048, 512, 0.9, seed=11, std=0.02)
    B = synth.dense(512, 512, seed=12)
    got, want = run_pair(A, m, B, k_tile=128)
    assert same_bits(got, want)
    assert O.rel_err(got, O.dense_fp64(A, B)) <= 1e-5


def test_tile_kernel_batched_mixed_with_gather_kernel(cuda):
    """One work list: tile-kernel problems of several packs and shapes beside gather-kernel ones."""
    m4, m8 = Mapping.identity(4), Mapping.load("747f9")
    work, refs = [], []
    g = np.random.default_rng(0)
    for i in range(40):
        mm = m4 if i % 3 else m8
        M, K = int(g.integers(8, 400)), int(g.integers(16, 700))
        n = int(g.integers(1, 300))
        ld = (n + 3) // 4 * 4
        kt = [64, 128, 160][i % 3]  # a 160-row tile of 128 FP32 columns (80 KB) still fits a stage
        A = synth.row_skew(M, K, 0.9, seed=100 + i, std=1.0)
        B = synth.dense(K, n, seed=200 + i)
        pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), mm, k_tile=kt)
        tb = padded(B, torch.float32, ld)
        C = torch.zeros((M, n), device="cuda")
        work.append((pm, tb, C, dict(staging=1 if i % 4 else 0, nr=[0, 32, 64, 128][i % 4])))
        refs.append(O.Packed(O.Tables.of(mm), A, k_tile=kt).execute(B))
    execute_batched(work)
    for (pm, tb, C, kw), want in zip(work, refs):
        assert same_bits(C.cpu().numpy(), want)
    assert device_status() == 0


def test_tile_kernel_refusals(cuda):
    m = Mapping.identity(4)
    A = synth.row_skew(64, 512, 0.9, seed=1, std=1.0)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m)  # one K tile of 512 rows
    B = torch.ones((512, 128), device="cuda")
    with pytest.raises(_lib.SpregError, match="exceeds a stage"):
        pm.execute(B, nr=128, staging=1)
    pt = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=128)
    with pytest.raises(_lib.SpregError, match="16-byte aligned"):
        pt.execute(torch.ones((512, 37), device="cuda"), staging=1)  # rows of 148 bytes
    with pytest.raises(_lib.SpregError, match="16-byte aligned"):
        pt.execute(torch.ones((512, 65), device="cuda")[:, 1:], staging=1)  # B base not 16-byte aligned
    assert device_status() == 0


@pytest.mark.parametrize("vd,cd", [(_lib.BF16, _lib.F32), (_lib.BF16, _lib.BF16), (_lib.F16, _lib.F32)])
@pytest.mark.parametrize("n,ld", [(512, 512), (300, 304), (256, 264)])
@pytest.mark.parametrize("mr,mp", [(2, None), (4, None), (4, "75a1b")])
def test_tile_kernel_256_column_strips(cuda, vd, cd, n, ld, mr, mp):
    """nr = 256 with 16-bit B: 256-column strips (two half steps of 2 entries), ragged columns on
    the 32-column kernel, load_c and the ReLU epilogue; bit-exact with the oracle."""
    m = Mapping.load(mp) if mp else Mapping.identity(mr)
    A = synth.row_skew(203, 384, 0.9, seed=n + mr, std=0.5)
    B = synth.dense(384, n, seed=n + 1)
    C0 = synth.dense(203, n, seed=7)
    got, want = run_pair(A, m, B, k_tile=128, value_dtype=vd, c_dtype=cd, nr=256, ld=ld, load_c=True, epilogue=1,
                         C0=C0)
    assert same_bits(got, want)
    assert device_status() == 0


def test_tile_kernel_256_column_strips_in_a_batch(cuda):
    """Automatic strip width: BF16 SpMMs of several shapes in one launch take 256-column strips where
    the launch has the items for them; every result equals its own call and the oracle."""
    m = Mapping.identity(4)
    work, refs = [], []
    for i in range(24):
        M, K, n = (512, 256, 512) if i % 2 else (256, 512, 384)
        A = synth.row_skew(M, K, 0.9, seed=300 + i, std=1.0)
        B = synth.dense(K, n, seed=400 + i)
        pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=128, value_dtype=_lib.BF16)
        tb = torch.from_numpy(B).to(torch.bfloat16).cuda()
        C = torch.zeros((M, n), device="cuda")
        work.append((pm, tb, C, {}))
        Bq = tb.cpu().view(torch.int16).numpy().view(np.uint16)
        refs.append(O.Packed(O.Tables.of(m), A, k_tile=128, value_dtype=_lib.BF16).execute(Bq))
    execute_batched(work)
    for (pm, tb, C, kw), want in zip(work, refs):
        assert same_bits(C.cpu().numpy(), want)
    pm, tb, C, _ = work[1]
    C1 = pm.execute(tb, staging=1, nr=128)
    assert same_bits(C1.cpu().numpy(), C.cpu().numpy())
    assert device_status() == 0


def test_nr_256_with_fp32_b_runs_128_column_strips(cuda):
    m = Mapping.identity(4)
    A = synth.row_skew(64, 256, 0.9, seed=3, std=1.0)
    B = synth.dense(256, 512, seed=4)
    got, want = run_pair(A, m, B, k_tile=128, nr=256)
    assert same_bits(got, want)


@pytest.mark.parametrize("vd", [_lib.BF16, _lib.F16])
def test_tile_kernel_256_column_strips_ragged_k_and_row_tiles(cuda, vd):
    """256-column strips on a ragged last K tile (K = 400, K_c = 128), row tiles (m_tile 48) and a
    column offset into B."""
    m = Mapping.identity(4)
    A = synth.row_skew(301, 400, 0.92, seed=21, std=0.5)
    off = 8
    B = synth.dense(400 + off, 512, seed=22)
    got, want = run_pair(A, m, B, k_tile=128, m_tile=48, col_offset=off, value_dtype=vd, nr=256)
    assert same_bits(got, want)


def test_work_order_single_panel_and_empty_rows(cuda):
    """Work-ordered execution blocks with one panel, and with all-zero panels between dense ones."""
    m = Mapping.identity(4)
    A1 = synth.row_skew(3, 256, 0.5, seed=1, std=1.0)
    B1 = synth.dense(256, 128, seed=2)
    got, want = run_pair(A1, m, B1, k_tile=64)
    assert same_bits(got, want)
    A2 = synth.row_skew(96, 256, 0.8, seed=3, std=1.0)
    A2[8:40] = 0.0
    A2[60:64] = 0.0
    B2 = synth.dense(256, 256, seed=4)
    got, want = run_pair(A2, m, B2, k_tile=128)
    assert same_bits(got, want)


def test_large_matrix_bit_exact(cuda):
    """16384 x 4096 at 95 % (3.4 M nonzeros, 32 K tiles of 128), N = 96 with a ragged strip: the packed
    arena, the work order and both executors (B tiles and L1/L2 gathers) at a larger scale."""
    m = Mapping.load("75a1b")
    A = synth.row_skew(16384, 4096, 0.95, seed=77, std=1.0)
    B = synth.dense(4096, 96, seed=78)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=128)
    ref = O.Packed(O.Tables.of(m), A, k_tile=128)
    assert pm.info["arena_bytes"] == ref.sizes["arena_bytes"] and pm.info["nnz"] == ref.sizes["nnz"]
    want = ref.execute(B)
    tb = torch.from_numpy(B).cuda()
    for staging in (1, 2):
        got = pm.execute(tb, staging=staging).cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), staging
    assert O.rel_err(want, O.dense_fp64(A, B)) <= 1e-5
    assert device_status() == 0
