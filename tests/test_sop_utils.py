"""The reference's Python helpers (sop_utils.py, distribution.py, mapping.py) under their names:
each against a direct restatement of the reference's loop."""
import hashlib

import numpy as np
import pytest
import torch

from spreg import synth
from spreg.mapping import Mapping
from spreg.sop_utils import (Codelet, compute_histogram, get_codelets_from_panel, pattern_code, popcount,
                             save_mapping, tile_matrix)


def test_codelets_match_the_reference_loop():
    panel = torch.from_numpy(synth.bernoulli(4, 200, 0.7, seed=1))
    want = {}
    for row in panel.t():  # sop_utils.py:33-40
        nnz = popcount(pattern_code(row))
        if nnz == 0:
            continue
        want.setdefault(nnz, Codelet(nnz=nnz, cols=0)).cols += 1
    assert get_codelets_from_panel(panel) == list(want.values())


def test_tile_matrix_splits_like_torch():
    m = torch.arange(35 * 22, dtype=torch.float32).reshape(35, 22)
    tiles = tile_matrix(m, (16, 8))
    assert [(i, j) for i, j, _ in tiles] == [(i, j) for i in range(3) for j in range(3)]
    assert tiles[-1][2].shape == (3, 6) and torch.equal(tiles[4][2], m[16:32, 8:16])


@pytest.mark.parametrize("mr", [2, 4, 8])
def test_compute_histogram_matches_the_reference_loop(mr):
    A = synth.row_skew(37, 50, 0.8, seed=mr, std=1.0)
    count = [0] * 2 ** mr  # distribution.py:18-26
    for i in range(0, A.shape[0], mr):
        for row in torch.from_numpy(A[i:i + mr]).t():
            count[pattern_code(row)] += 1
    want = np.array(count) / (A.shape[1] * A.shape[0] // mr)
    np.testing.assert_allclose(compute_histogram(mr, torch.from_numpy(A)), want, rtol=0, atol=0)


def test_save_mapping_names_files_like_the_reference(tmp_path):
    fn = lambda p: [p | 1] if p & 1 == 0 and p != 0 else [p]  # noqa: E731
    mid = save_mapping(4, fn, subdir="m", root=str(tmp_path))
    assert mid == hashlib.md5(str({i: fn(i) for i in range(1, 16)}).encode("utf-8")).hexdigest()[-5:]
    text = (tmp_path / "m" / f"mapping_{mid}.txt").read_text()
    assert text.splitlines()[0] == "4" and text.splitlines()[2] == "2: [3]"
    assert Mapping.from_text(text).mapping_id == mid
    with pytest.raises(TypeError):
        save_mapping(2, lambda p: p, subdir="m", root=str(tmp_path))  # list(int) fails as in the reference
