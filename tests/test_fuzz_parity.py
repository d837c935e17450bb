"""Seeded random sweep over the executor's configuration space, bit-exact against the oracle.

Each case draws a shape, sparsity, panel height and nanokernel set, storage type, row / K tiles,
column offset, N, strip width, B / C leading dimensions, load_c, epilogue and staging, runs it on
the GPU alone and in one batched launch with all the other cases, and compares both with the
oracle's execution of the same packing.
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
MAPS = [("id2", 2), ("id4", 4), ("id6", 6), ("id8", 8), ("400fa", 8), ("747f9", 8), ("75a1b", 4)]


def draw_case(g):
    name, mr = MAPS[int(g.integers(len(MAPS)))]
    m = Mapping.identity(mr) if name.startswith("id") else Mapping.load(name)
    M, K = int(g.integers(1, 300)), int(g.integers(1, 600))
    sp = float(g.choice([0.0, 0.5, 0.8, 0.9, 0.97, 1.0]))
    vd = [_lib.F32, _lib.BF16, _lib.F16][int(g.integers(3))]
    k_tile = int(g.choice([0, 0, 64, 128, 200]))
    m_tile = int(g.choice([0, 0, mr * 4, mr * 12]))
    col_offset = int(g.choice([0, 0, 3, 16]))
    n = int(g.choice([1, 7, 32, 64, 100, 128, 256, 300, 512]))
    nr = int(g.choice([0, 0, 32, 64, 128, 256]))
    ld_pad = int(g.choice([0, 0, 8]))
    load_c = bool(g.integers(2))
    epi = int(g.integers(2))
    staging = int(g.choice([0, 0, 2]))
    return dict(m=m, M=M, K=K, sp=sp, vd=vd, k_tile=k_tile, m_tile=m_tile, col_offset=col_offset, n=n, nr=nr,
                ld_pad=ld_pad, load_c=load_c, epi=epi, staging=staging)


def build(c, seed):
    A = synth.row_skew(c["M"], c["K"], c["sp"], seed=seed, std=1.0) if c["sp"] < 1.0 else \
        np.zeros((c["M"], c["K"]), np.float32)
    rows_b = c["K"] + c["col_offset"]
    B = synth.dense(rows_b, c["n"], seed=seed + 1)
    ld = c["n"] + c["ld_pad"]
    tb = torch.zeros((rows_b, ld), dtype=TORCH[c["vd"]], device="cuda")
    tb[:, :c["n"]] = torch.from_numpy(B).to(TORCH[c["vd"]])
    tb = tb[:, :c["n"]]
    C0 = synth.dense(c["M"], c["n"], seed=seed + 2)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), c["m"], m_tile=c["m_tile"], k_tile=c["k_tile"],
                                 col_offset=c["col_offset"], value_dtype=c["vd"])
    ref = O.Packed(O.Tables.of(c["m"]), A, m_tile=c["m_tile"], k_tile=c["k_tile"], col_offset=c["col_offset"],
                   value_dtype=c["vd"])
    Bref = B if c["vd"] == _lib.F32 else tb.cpu().contiguous().view(torch.int16).numpy().view(np.uint16)
    want = np.array(C0 if c["load_c"] else np.zeros_like(C0), dtype=np.float32)
    ref.execute(Bref, want, load_c=c["load_c"], epilogue=c["epi"])
    return pm, tb, C0, want


def kwargs_of(c):
    return dict(nr=c["nr"], load_c=c["load_c"], epilogue=c["epi"], staging=c["staging"])


@pytest.mark.parametrize("block", range(4))
def test_fuzz_alone_and_batched_bit_exact(cuda, block):
    g = np.random.default_rng(1000 + block)
    cases = [draw_case(g) for _ in range(40)]
    built = [build(c, 7000 + 100 * block + i) for i, c in enumerate(cases)]
    work, wants = [], []
    for i, (c, (pm, tb, C0, want)) in enumerate(zip(cases, built)):
        C = torch.from_numpy(C0).cuda() if c["load_c"] else torch.zeros((c["M"], c["n"]), device="cuda")
        pm.execute(tb, C, **kwargs_of(c))  # automatic (0) and L1/L2 (2) staging take every pack
        got = C.cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (i, c)
        Cb = torch.from_numpy(C0).cuda() if c["load_c"] else torch.zeros((c["M"], c["n"]), device="cuda")
        work.append((pm, tb, Cb, kwargs_of(c)))
        wants.append((i, c, want))
    execute_batched(work)
    for (pm, tb, Cb, kw), (i, c, want) in zip(work, wants):
        assert np.array_equal(Cb.cpu().numpy().view(np.uint32), want.view(np.uint32)), ("batched", i, c)
    assert device_status() == 0


def draw_wide(g):
    """A case for the wide strips (nr = 256 / 512): high sparsity, widths around the strip
    boundaries, B row strides that keep or lose 16-byte alignment, untiled and K-tiled packs
    (the latter through the gather kernel with staging 2, or the executor's own choice)."""
    c = draw_case(g)
    c.update(M=int(g.integers(1, 700)), sp=float(g.choice([0.9, 0.95, 0.98, 0.99])),
             nr=int(g.choice([256, 512])), n=int(g.choice([256, 264, 300, 512, 520, 600, 1024])),
             k_tile=int(g.choice([0, 0, 128])), staging=int(g.choice([0, 2])), ld_pad=int(g.choice([0, 4, 8, 3])))
    return c


@pytest.mark.parametrize("block", range(2))
def test_fuzz_wide_strips_bit_exact(cuda, block):
    g = np.random.default_rng(2000 + block)
    cases = [draw_wide(g) for _ in range(40)]
    built = [build(c, 9000 + 100 * block + i) for i, c in enumerate(cases)]
    work, wants = [], []
    for i, (c, (pm, tb, C0, want)) in enumerate(zip(cases, built)):
        C = torch.from_numpy(C0).cuda() if c["load_c"] else torch.zeros((c["M"], c["n"]), device="cuda")
        pm.execute(tb, C, **kwargs_of(c))
        assert np.array_equal(C.cpu().numpy().view(np.uint32), want.view(np.uint32)), (i, c)
        Cb = torch.from_numpy(C0).cuda() if c["load_c"] else torch.zeros((c["M"], c["n"]), device="cuda")
        work.append((pm, tb, Cb, kwargs_of(c)))
        wants.append((i, c, want))
    execute_batched(work)
    for (pm, tb, Cb, kw), (i, c, want) in zip(work, wants):
        assert np.array_equal(Cb.cpu().numpy().view(np.uint32), want.view(np.uint32)), ("batched", i, c)
    assert device_status() == 0
