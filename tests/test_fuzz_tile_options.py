"""Seeded random combinations of the B-tile executor's options, each bit for bit against the oracle
(sbench/SOP/_C/pytorch_wrapper_intrin.cpp.template:265-305; the load-balanced order where a call is
split, oracle.load_balanced_execute): shapes and ragged edges, K tiles, strip widths (masked tail
strips and 32-column tails), panel rounds, load-balanced splits, job orders, CTA tiling, storage
types, load_c and ReLU."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from spreg import _lib, synth
from spreg.mapping import Mapping
from spreg.packed import PackedMatrix, device_status

pytestmark = pytest.mark.gpu

TORCH = {_lib.F32: torch.float32, _lib.BF16: torch.bfloat16}


def draw(seed):
    r = np.random.default_rng(seed)
    vd = (_lib.F32, _lib.BF16)[r.integers(2)]
    mr = int(r.choice([2, 4, 8]))
    M = int(r.integers(40, 900))
    K = int(r.choice([128, 192, 256, 384, 512]))
    k_tile = int(r.choice([64, 128]))
    nr = int(r.choice([32, 64, 128]))
    n = int(r.integers(1, 80)) * 4  # whole lane columns for every width up to 4 (16-byte rows for 16-bit B)
    if vd == _lib.BF16:
        n = max(8, n // 8 * 8)
    rounds = int(r.choice([0, 0, 2, 5]))
    balance = int(r.integers(2))
    if rounds and K * 32 * (nr // 32) * (4 if vd == _lib.F32 else 2) > 190 * 1024:
        nr = 32  # the whole-K strip of panel rounds must fit shared memory
    return dict(vd=vd, mr=mr, M=M, K=K, k_tile=k_tile, nr=nr, n=n, rounds=rounds, balance=balance,
                order=int(r.integers(2)), warps=int(r.choice([0, 0, 4, 8])), load_c=bool(r.integers(2)),
                epilogue=int(r.integers(2)), sparsity=float(r.choice([0.8, 0.9, 0.97])),
                sigma=float(r.choice([0.5, 1.2])), seed=seed)


@pytest.mark.parametrize("seed", range(40))
def test_tile_options_match_the_oracle(cuda, seed):
    c = draw(seed)
    m = Mapping.identity(c["mr"])
    A = synth.row_skew(c["M"], c["K"], c["sparsity"], seed=seed, sigma=c["sigma"], std=1.0)
    B = synth.dense(c["K"], c["n"], seed=seed + 1000)
    C0 = synth.dense(c["M"], c["n"], seed=seed + 2000)
    vd = c["vd"]
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, k_tile=c["k_tile"], value_dtype=vd)
    Bt = torch.from_numpy(B).cuda().to(TORCH[vd])
    Bref = B if vd == _lib.F32 else Bt.cpu().view(torch.int16).numpy().view(np.uint16)
    Cg = torch.from_numpy(C0.copy()).cuda()
    kw = dict(nr=c["nr"], rounds=c["rounds"], order=c["order"], warps=c["warps"], staging=1)
    H, split, heavy = pm.load_balance_plan(Bt, Cg, nr=c["nr"], warps=c["warps"], staging=1, rounds=c["rounds"])
    pm.execute(Bt, Cg, load_c=c["load_c"], epilogue=c["epilogue"], balance=c["balance"], **kw)
    out = C0.copy() if c["load_c"] else None
    if c["balance"] and H > 0:
        want = O.load_balanced_execute(O.Tables.of(m), A, Bref, heavy, split, c["k_tile"], value_dtype=vd, out=out,
                                       load_c=c["load_c"], epilogue=c["epilogue"])
    else:
        want = O.Packed(O.Tables.of(m), A, k_tile=c["k_tile"], value_dtype=vd).execute(
            Bref, out, load_c=c["load_c"], epilogue=c["epilogue"])
    got = Cg.cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), c
    assert device_status() == 0
