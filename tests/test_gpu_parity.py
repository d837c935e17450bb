"""GPU parity: libspreg.so's packer and executor against the CPU oracle.

Packing is integer work: the arena bytes and descriptors must be identical.  The executor
chains fmaf in the packed-entry order of the reference executor, so FP32 results must be
bit-identical to the oracle's; they are also checked against the reference's own spmm_naive
(golden fixtures, rel err <= 1e-5) and the FP64 dense product (rel err <= 1e-5).  BF16 / FP16
storage is bit-identical to the oracle's 16-bit path and within rel err 1e-2 of FP64."""
import glob
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.matmul import MatMulSpecialized, TileConfig
from spreg.packed import PackedMatrix, device_status, execute_batched
from spreg.sop_driver import Acc, make_sop_module, sort_and_encode_patterns

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

MAPPINGS = {
    "id2": lambda: Mapping.identity(2), "id4": lambda: Mapping.identity(4), "id6": lambda: Mapping.identity(6),
    "id8": lambda: Mapping.identity(8), "400fa": lambda: Mapping.load("400fa"), "747f9": lambda: Mapping.load("747f9"),
    "33960": lambda: Mapping.load("33960"), "75f82": lambda: Mapping.load("75f82"), "dcfff": lambda: Mapping.load("dcfff"),
}
SHAPES = [(64, 96, 0.8), (130, 200, 0.9), (7, 300, 0.5), (5, 1000, 0.97), (1, 1, 0.0), (33, 513, 0.7)]


def gpu_pack(A, m, **kw):
    return PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, **kw)


def assert_same_pack(pm: PackedMatrix, ref: O.Packed):
    arena, descs, scales = pm.to_host()
    assert pm.info["num_units"] == ref.num_units
    assert pm.info["arena_bytes"] == ref.sizes["arena_bytes"]
    for k in ("num_values", "padding", "nnz", "required_storage", "empty_units"):
        assert pm.info[k] == ref.sizes[k], k
    assert pm.info["num_col_indices"] == ref.sizes["num_col_indices"]
    assert np.array_equal(descs, ref.descs)
    assert np.array_equal(arena, ref.arena)
    if ref.scales is not None:
        assert np.array_equal(scales, ref.scales)


@pytest.mark.parametrize("mkey", list(MAPPINGS))
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: f"{s[0]}x{s[1]}@{s[2]}")
def test_pack_dense_bit_exact(cuda, mkey, shape):
    m = MAPPINGS[mkey]()
    A = synth.row_skew(shape[0], shape[1], shape[2], seed=hash(shape) % 1000, std=1.0)
    assert_same_pack(gpu_pack(A, m), O.Packed(O.Tables.of(m), A))


@pytest.mark.parametrize("vd", [_lib.F32, _lib.BF16, _lib.F16])
@pytest.mark.parametrize("tiles", [(0, 0), (8, 64), (16, 256), (4, 7)])
def test_pack_csr_tiled_dtypes_bit_exact(cuda, vd, tiles):
    m = Mapping.load("400fa") if tiles[0] % 8 == 0 else Mapping.identity(4)
    A = synth.row_skew(83, 260, 0.85, seed=3, std=0.5)
    A[:, 64:128] = 0.0
    rp, ci, v = synth.to_csr(A)
    # CSR with rows in a shuffled column order: the packer must not depend on it
    g = np.random.default_rng(0)
    for i in range(A.shape[0]):
        s, e = rp[i], rp[i + 1]
        p = g.permutation(e - s)
        ci[s:e], v[s:e] = ci[s:e][p], v[s:e][p]
    pm = PackedMatrix.from_csr(torch.from_numpy(rp).cuda(), torch.from_numpy(ci).cuda(), torch.from_numpy(v).cuda(),
                               A.shape, m, m_tile=tiles[0], k_tile=tiles[1], value_dtype=vd, col_offset=5)
    ref = O.Packed(O.Tables.of(m), A, m_tile=tiles[0], k_tile=tiles[1], col_offset=5, value_dtype=vd)
    assert_same_pack(pm, ref)


def test_pack_rejects_duplicate_csr_entries(cuda):
    rp = torch.tensor([0, 2], dtype=torch.int32, device="cuda")
    ci = torch.tensor([3, 3], dtype=torch.int32, device="cuda")
    v = torch.tensor([1.0, 2.0], device="cuda")
    with pytest.raises(_lib.SpregError, match="duplicate"):
        PackedMatrix.from_csr(rp, ci, v, (1, 8), Mapping.identity(4))


def test_pack_rejects_uncovering_mapping(cuda):
    bad = Mapping(4, {p: [p & 3] if p & 3 else [] for p in range(16)})
    A = np.ones((4, 4), np.float32)
    with pytest.raises(_lib.SpregError, match="invariant"):
        gpu_pack(A, bad)


def _exec_both(pm, ref, B, n=None, nr=0, load_c=False, C0=None, epilogue=0, c_dtype=_lib.F32, meta=0):
    torch_b = {_lib.F32: torch.float32, _lib.BF16: torch.bfloat16, _lib.F16: torch.float16}[pm.value_dtype]
    tb = torch.from_numpy(B).to(torch_b).cuda()
    Bref = B if pm.value_dtype == _lib.F32 else tb.cpu().view(torch.int16).numpy().view(np.uint16)
    out_t = torch.float32 if c_dtype == _lib.F32 else torch.bfloat16
    Cg = torch.zeros((pm.info["rows"], B.shape[1]), dtype=out_t, device="cuda")
    Cr = np.zeros((pm.info["rows"], B.shape[1]), dtype=np.float32 if c_dtype == _lib.F32 else np.uint16)
    if C0 is not None:
        Cg.copy_(torch.from_numpy(C0).to(out_t))
        Cr[...] = C0 if c_dtype == _lib.F32 else Cg.cpu().view(torch.int16).numpy().view(np.uint16)
    pm.execute(tb, Cg, n=n, nr=nr, load_c=load_c, epilogue=epilogue, meta=meta)
    ref.execute(Bref, Cr, n=n, load_c=load_c, epilogue=epilogue, c_dtype=c_dtype)
    got = Cg.cpu()
    got = got.numpy() if c_dtype == _lib.F32 else got.view(torch.int16).numpy().view(np.uint16)
    return got, Cr


@pytest.mark.parametrize("mkey", ["id2", "id4", "id6", "id8", "400fa", "747f9", "33960", "75f82"])
@pytest.mark.parametrize("n,nr", [(1, 0), (31, 32), (64, 64), (100, 0), (256, 128), (257, 128), (512, 0), (96, 64)])
@pytest.mark.parametrize("meta", [1, 2])
def test_execute_fp32_bit_exact(cuda, mkey, n, nr, meta):
    """Both executor kernels (execution-layout blocks staged per warp / arena streamed through
    registers) against the oracle."""
    m = MAPPINGS[mkey]()
    A = synth.row_skew(70, 300, 0.85, seed=n, std=1.0)
    B = synth.dense(300, n, seed=n + 1)
    pm, ref = gpu_pack(A, m), O.Packed(O.Tables.of(m), A)
    got, want = _exec_both(pm, ref, B, nr=nr, meta=meta)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert O.rel_err(got, O.dense_fp64(A, B)) <= 1e-5


@pytest.mark.parametrize("vd", [_lib.F32, _lib.BF16, _lib.F16])
@pytest.mark.parametrize("load_c,epi", [(False, 0), (True, 0), (True, 1), (False, 1)])
@pytest.mark.parametrize("meta", [1, 2])
def test_execute_dtypes_load_c_epilogue(cuda, vd, load_c, epi, meta):
    m = Mapping.identity(4) if meta == 1 else Mapping.load("400fa")
    A = synth.row_skew(66, 200, 0.8, seed=2, std=0.02)
    B = synth.dense(200, 130, seed=3)
    C0 = synth.dense(66, 130, seed=4)
    pm = gpu_pack(A, m, value_dtype=vd)
    ref = O.Packed(O.Tables.of(m), A, value_dtype=vd)
    got, want = _exec_both(pm, ref, B, load_c=load_c, C0=C0 if load_c else None, epilogue=epi, meta=meta)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    exact = O.dense_fp64(A, B) + (C0 if load_c else 0)
    if epi:
        exact = np.maximum(exact, 0)
    assert O.rel_err(got, exact) <= (1e-5 if vd == _lib.F32 else 1e-2)


def test_execute_bf16_output(cuda):
    m = Mapping.load("747f9")
    A = synth.row_skew(64, 512, 0.9, seed=5, std=0.02)
    B = synth.dense(512, 192, seed=6)
    pm = gpu_pack(A, m, value_dtype=_lib.BF16)
    ref = O.Packed(O.Tables.of(m), A, value_dtype=_lib.BF16)
    got, want = _exec_both(pm, ref, B, c_dtype=_lib.BF16, epilogue=1)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("tiles", [(8, 64), (16, 256), (4, 7)])
def test_execute_tiled_bit_exact_auto(cuda, tiles):
    m = Mapping.identity(4)
    A = synth.row_skew(90, 333, 0.9, seed=7, std=1.0)
    A[:, 64:128] = 0
    B = synth.dense(333, 160, seed=8)
    pm = gpu_pack(A, m, m_tile=tiles[0], k_tile=tiles[1])
    ref = O.Packed(O.Tables.of(m), A, m_tile=tiles[0], k_tile=tiles[1])
    got, want = _exec_both(pm, ref, B)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_execute_partial_n_leaves_rest(cuda):
    m = Mapping.identity(4)
    A = synth.bernoulli(40, 50, 0.7, seed=1)
    B = synth.dense(50, 100, seed=2)
    pm = gpu_pack(A, m)
    C = torch.full((40, 100), 7.0, device="cuda")
    pm.execute(torch.from_numpy(B).cuda(), C, n=37)
    C = C.cpu().numpy()
    assert np.all(C[:, 37:] == 7.0)
    assert O.rel_err(C[:, :37], O.dense_fp64(A, B[:, :37])) <= 1e-5


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))), ids=lambda p: os.path.basename(p)[:-4])
def test_golden_reference_spmm_naive(cuda, path):
    z = np.load(path)
    M, K = (int(x) for x in z["shape"])
    A = np.zeros((M, K), np.float32)
    A[np.repeat(np.arange(M), np.diff(z["row_ptrs"])), z["col_inds"]] = z["values"]
    for m in (Mapping.identity(4), Mapping.load("400fa")):
        pm = PackedMatrix.from_csr(*(torch.from_numpy(z[k]).cuda() for k in ("row_ptrs", "col_inds", "values")),
                                   (M, K), m)
        C = pm.execute(torch.from_numpy(z["B"]).cuda()).cpu().numpy()
        assert O.rel_err(C, z["C_ref_naive"]) <= 1e-5


@pytest.mark.parametrize("mkey", ["id4", "400fa"])
def test_known_answer_ones_gpu(cuda, mkey):
    m = MAPPINGS[mkey]()
    A = (synth.bernoulli(2048, 512, 0.9, seed=1) != 0).astype(np.float32)
    pm = gpu_pack(A, m)
    C = pm.execute(torch.ones((512, 512), device="cuda")).cpu().numpy()
    assert np.array_equal(C, np.repeat(A.sum(1, keepdims=True), 512, 1))


@pytest.mark.parametrize("shape", [(2048, 512), (512, 2048)])
@pytest.mark.parametrize("sparsity", [0.7, 0.9, 0.98])
def test_ffn_shapes_full_size(cuda, shape, sparsity):
    """Full FFN-shaped sizes: bit-exact with the oracle, plus linearity A(B1 + B2) = AB1 + AB2."""
    m = Mapping.identity(4)
    A = synth.row_skew(shape[0], shape[1], sparsity, seed=11, std=0.02)
    B = synth.dense(shape[1], 512, seed=12)
    pm, ref = gpu_pack(A, m), O.Packed(O.Tables.of(m), A)
    assert_same_pack(pm, ref)
    got, want = _exec_both(pm, ref, B)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    B2 = synth.dense(shape[1], 512, seed=13)
    tb1, tb2 = torch.from_numpy(B).cuda(), torch.from_numpy(B2).cuda()
    s = pm.execute(tb1 + tb2)
    assert torch.allclose(s, pm.execute(tb1) + pm.execute(tb2), rtol=1e-4, atol=1e-5)


def test_sort_and_encode_gpu_matches_oracle(cuda):
    g = np.random.default_rng(1)
    m = Mapping.load("400fa")
    t = O.Tables.of(m)
    allowed = [0] + m.nanokernels
    for n in (1, 255, 256, 257, 5000):
        codes = np.asarray(g.choice(allowed, size=n), np.int32)
        enc, order = sort_and_encode_patterns(m, torch.from_numpy(codes))
        e2, o2 = O.sort_and_encode(t, codes)
        assert np.array_equal(enc.numpy(), e2) and np.array_equal(order.numpy(), o2)


def test_sop_module_surface(cuda):
    """make_sop_module / make_sop_tile / execute_tile as sbench/SOP/sop_bench.py drives them."""
    acc = Acc(4, 4)
    m = Mapping.identity(4)
    mod = make_sop_module(acc, m.nanokernels, m)
    tile = (synth.bernoulli(48, 256, 0.8, seed=2) != 0).astype(np.float32)
    sop_tile = mod.make_sop_tile(torch.from_numpy(tile))
    assert sop_tile.padding() == 0
    B = torch.ones((256, 128))
    t, result = mod.execute_tile(sop_tile, B, num_runs=2)
    assert t > 0
    assert torch.allclose(result, torch.from_numpy(tile) @ B)
    ref = O.Packed(O.Tables.of(m), tile)
    assert_same_pack(sop_tile.packed, ref)
    # non-identity mapping with padding (SOPOrig-style callable)
    m8 = Mapping.load("400fa")
    mod8 = make_sop_module(Acc(8, 2), m8.nanokernels, lambda p: m8(p))
    t8 = mod8.make_sop_tile(torch.from_numpy(tile), col_offset=0)
    assert t8.padding() == O.Packed(O.Tables.of(m8), tile).sizes["padding"] > 0
    _, r8 = mod8.execute_tile(t8, B, num_runs=1, N_c=64)
    assert torch.allclose(r8[:, :64], (torch.from_numpy(tile) @ B)[:, :64]) and torch.all(r8[:, 64:] == 0)


def test_matmul_specialized_host_and_device(cuda):
    A = synth.row_skew(256, 384, 0.9, seed=21, std=1.0)
    B = synth.dense(384, 96, seed=22)
    rp, ci, v = synth.to_csr(A)
    mm = MatMulSpecialized(256, 384, 96, v, rp, ci, TileConfig(), 1, "AVX512_512_4", "61fee")
    cfg = mm.get_config()
    assert cfg.nr == 64 and cfg.M_c == 256 and cfg.K_c == 384
    C = np.zeros((256, 96), np.float32)
    mm(C, B)
    ref = O.Packed(O.Tables.of(Mapping.identity(4)), A).execute(B)
    assert np.array_equal(C, ref)
    Cd = torch.zeros((256, 96), device="cuda")
    mm(Cd, torch.from_numpy(B).cuda())
    assert np.array_equal(Cd.cpu().numpy(), ref)
    assert mm.require_storage == O.Packed(O.Tables.of(Mapping.identity(4)), A).sizes["required_storage"]
    # reference SOPConfig tiles (m_tile 16, k_tile 256)
    mm2 = MatMulSpecialized(256, 384, 96, v, rp, ci, TileConfig.from_sop_config({"m_tile": 16, "k_tile": 256}),
                            mapping_id="61fee")
    C2 = np.zeros((256, 96), np.float32)
    mm2(C2, B)
    ref2 = O.Packed(O.Tables.of(Mapping.identity(4)), A, m_tile=16, k_tile=256).execute(B)
    assert np.array_equal(C2, ref2)


def test_matmul_specialized_async_host_calls_overlap_and_match(cuda):
    """Host-buffer calls enqueued on several matmuls' streams, then synced: each C equals the oracle,
    also when one matmul runs two calls back to back before its sync."""
    mms, Bs, Cs, refs = [], [], [], []
    for i in range(6):
        A = synth.row_skew(200 + 8 * i, 256, 0.9, seed=40 + i, std=1.0)
        B = synth.dense(256, 160, seed=50 + i)
        rp, ci, v = synth.to_csr(A)
        mms.append(MatMulSpecialized(A.shape[0], 256, 160, v, rp, ci, TileConfig(K_c=128), 1, "", "61fee"))
        Bs.append(torch.from_numpy(B).pin_memory())
        Cs.append(torch.zeros((A.shape[0], 160)).pin_memory())
        refs.append(O.Packed(O.Tables.of(Mapping.identity(4)), A, k_tile=128).execute(B))
    C0b = torch.zeros_like(Cs[0]).pin_memory()
    for mm, B, C in zip(mms, Bs, Cs):
        mm.run_async(C, B)
    mms[0].run_async(C0b, Bs[0])  # second call on the same stream: runs after the first
    for mm in mms:
        mm.sync()
    for C, ref in zip(Cs, refs):
        assert np.array_equal(C.numpy(), ref)
    assert np.array_equal(C0b.numpy(), refs[0])
    with pytest.raises(ValueError, match="no conversion copy"):
        mms[1].run_async(Cs[1], Bs[1].double())  # a converted B would be freed before its copy runs
    assert device_status() == 0


def test_matmul_direct_host_output_matches_the_copy_path(cuda):
    """C stored by the kernel straight into pinned host memory (the default), C through device memory
    and a copy (direct output off), and a pageable C (always the copy path): the same bits."""
    A = synth.row_skew(300, 384, 0.9, seed=61, std=1.0)
    B = torch.from_numpy(synth.dense(384, 200, seed=62)).pin_memory()
    rp, ci, v = synth.to_csr(A)
    mm = MatMulSpecialized(300, 384, 200, v, rp, ci, TileConfig(K_c=128), 1, "", "61fee")
    want = O.Packed(O.Tables.of(Mapping.identity(4)), A, k_tile=128).execute(B.numpy())
    C_direct = torch.full((300, 200), -1.0).pin_memory()
    mm(C_direct, B)
    mm.set_direct_output(False)
    C_copy = torch.full((300, 200), -1.0).pin_memory()
    mm(C_copy, B)
    mm.set_direct_output(True)
    C_pageable = np.full((300, 200), -1.0, dtype=np.float32)
    mm(C_pageable, B)
    for C in (C_direct.numpy(), C_copy.numpy(), C_pageable):
        assert np.array_equal(C.view(np.uint32), want.view(np.uint32))
    assert device_status() == 0


def test_execute_batched_equals_individual(cuda):
    """Uneven SpMMs (mappings, M_r, dtypes, N with tails, K tiles) in one call: each result is the
    same as its own call and as the oracle."""
    cases = [(64, 128, 32, "id4", _lib.F32, 0), (100, 77, 257, "400fa", _lib.F32, 0), (8, 512, 1, "id4", _lib.F32, 0),
             (256, 64, 128, "id4", _lib.BF16, 0), (300, 200, 96, "747f9", _lib.BF16, 0),
             (90, 333, 200, "id4", _lib.F32, 64), (512, 512, 512, "id4", _lib.F32, 0)]
    items, want, refs = [], [], []
    for i, (M, K, N, mk, vd, kt) in enumerate(cases):
        m = MAPPINGS[mk]()
        A = synth.row_skew(M, K, 0.8, seed=i, std=1.0)
        Bn = synth.dense(K, N, seed=100 + i)
        tdt = torch.float32 if vd == _lib.F32 else torch.bfloat16
        B = torch.from_numpy(Bn).to(tdt).cuda()
        pm = gpu_pack(A, m, value_dtype=vd, k_tile=kt)
        Cb = torch.zeros((M, N), device="cuda")
        items.append((pm, B, Cb, {}))
        want.append(pm.execute(B))
        ref = O.Packed(O.Tables.of(m), A, value_dtype=vd, k_tile=kt)
        refs.append(ref.execute(Bn if vd == _lib.F32 else B.cpu().view(torch.int16).numpy().view(np.uint16)))
    execute_batched(items)
    for (pm, B, Cb, _), w, r in zip(items, want, refs):
        assert torch.equal(Cb, w)
        assert np.array_equal(Cb.cpu().numpy().view(np.uint32), r.view(np.uint32))


def test_empty_and_degenerate(cuda):
    m = Mapping.identity(4)
    for shape in [(0, 5), (5, 0), (4, 4)]:
        A = np.zeros(shape, np.float32)
        pm = gpu_pack(A, m)
        C = pm.execute(torch.ones((shape[1], 9), device="cuda"))
        assert torch.all(C == 0) and C.shape == (shape[0], 9)


@pytest.mark.parametrize("mkey", ["id4", "id6", "id8", "400fa", "747f9"])
@pytest.mark.parametrize("meta", [1, 2])
@pytest.mark.parametrize("vd", [_lib.F32, _lib.BF16])
@pytest.mark.parametrize("n,nr", [(128, 64), (256, 128), (512, 0), (300, 64), (64, 32)])
def test_execute_kernels_bit_exact(cuda, mkey, meta, vd, n, nr):
    """Batched execution-layout kernel (meta 1) and register-stream kernel (meta 2): identical bits."""
    m = MAPPINGS[mkey]()
    A = synth.row_skew(520, 384, 0.9, seed=n + nr, std=0.5)
    B = synth.dense(384, n, seed=n)
    pm, ref = gpu_pack(A, m, value_dtype=vd), O.Packed(O.Tables.of(m), A, value_dtype=vd)
    torch_b = torch.float32 if vd == _lib.F32 else torch.bfloat16
    tb = torch.from_numpy(B).to(torch_b).cuda()
    Cg = pm.execute(tb, nr=nr, meta=meta).cpu().numpy()
    Bref = B if vd == _lib.F32 else tb.cpu().view(torch.int16).numpy().view(np.uint16)
    want = ref.execute(Bref)
    assert np.array_equal(Cg.view(np.uint32), want.view(np.uint32))


def test_b_staging_panel_by_panel_pack_is_rejected(cuda):
    """Shared-memory B tiles need one column range per K tile; SOPTile packs have per-panel offsets."""
    module = make_sop_module(Acc(4, 64), list(range(1, 16)), lambda p: p)
    A = torch.from_numpy(synth.bernoulli(64, 64, 0.5, seed=1))
    tile = module.make_sop_tile(A)
    with pytest.raises(_lib.SpregError, match="dense/CSR pack"):
        tile.packed.execute(torch.ones((64, 64), device="cuda"), staging=1)


@pytest.mark.parametrize("meta", [1, 2])
def test_execute_with_col_offset(cuda, meta):
    """A tile packed with a column offset reads B rows [offset, offset + K)."""
    m = Mapping.identity(4)
    A = synth.row_skew(256, 200, 0.85, seed=3, std=1.0)
    off = 37
    B = synth.dense(200 + off + 11, 256, seed=4)
    pm = gpu_pack(A, m, col_offset=off)
    ref = O.Packed(O.Tables.of(m), A, col_offset=off)
    C = pm.execute(torch.from_numpy(B).cuda(), nr=64, meta=meta).cpu().numpy()
    assert np.array_equal(C.view(np.uint32), ref.execute(B).view(np.uint32))
    assert O.rel_err(C, O.dense_fp64(A, B[off:off + 200])) <= 1e-5


@pytest.mark.parametrize("tiles", [(8, 64), (16, 256), (4, 7)])
@pytest.mark.parametrize("meta", [1, 2])
def test_execute_tiled_kernels(cuda, tiles, meta):
    """K-tiled packs on both kernels: units of one row panel run in K-tile order."""
    m = Mapping.load("400fa") if tiles[0] % 8 == 0 else Mapping.identity(4)
    A = synth.row_skew(90, 333, 0.9, seed=7, std=1.0)
    A[:, 64:128] = 0
    B = synth.dense(333, 200, seed=8)
    pm = gpu_pack(A, m, m_tile=tiles[0], k_tile=tiles[1])
    ref = O.Packed(O.Tables.of(m), A, m_tile=tiles[0], k_tile=tiles[1])
    got, want = _exec_both(pm, ref, B, meta=meta)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_device_status_clear(cuda):
    from spreg.packed import device_status
    assert device_status(reset=True) == 0


def test_bounded_wait_gives_up_and_the_context_stays_usable(cuda):
    """A wait on an mbarrier that nothing arrives on (short limit) ends with status 30 instead of a
    hang; afterwards the status clears and an SpMM still runs bit-exact."""
    import time
    from spreg.packed import selftest_wait_timeout
    device_status(reset=True)
    t0 = time.perf_counter()
    status, polls = selftest_wait_timeout(1000)
    assert status == 30 and polls == 1000
    assert time.perf_counter() - t0 < 5.0
    assert device_status(reset=True) == 30 and device_status() == 0
    m = Mapping.identity(4)
    A = synth.row_skew(64, 256, 0.9, seed=5, std=1.0)
    B = synth.dense(256, 64, seed=6)
    got = gpu_pack(A, m, k_tile=128).execute(torch.from_numpy(B).cuda(), staging=1).cpu().numpy()
    assert np.array_equal(got.view(np.uint32), O.Packed(O.Tables.of(m), A, k_tile=128).execute(B).view(np.uint32))
    with pytest.raises(_lib.SpregError, match="limit"):
        selftest_wait_timeout(0)
