"""Matrix files (.smtx / .mtx) and the on-disk packed-weight format."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from spreg import io, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_MTX = os.path.join(O.REFERENCE_ROOT, "bundled_datasets/random/random_90_768_768.mtx") if O.REFERENCE_ROOT else ""


def _csr(A):
    rp, ci, v = synth.to_csr(A)
    return A.shape[0], A.shape[1], rp, ci, v


# ---------------------------------------------------------------------------- .smtx
def test_smtx_round_trip(tmp_path):
    A = synth.bernoulli(37, 53, 0.8, seed=1)
    rows, cols, rp, ci, _ = _csr(A)
    p = tmp_path / "a.smtx"
    io.write_smtx(str(p), rows, cols, rp, ci)
    r, c, rp2, ci2 = io.load_smtx(str(p))
    assert (r, c) == (rows, cols) and np.array_equal(rp2, rp) and np.array_equal(ci2, ci)
    assert rp2.dtype == np.int32 and ci2.dtype == np.int32
    _, _, _, _, v = io.read_smtx(str(p))
    assert v.dtype == np.float32 and np.all(v == 1.0)  # ParseSMTX.h:52


def test_smtx_multiline_and_trailing_tokens(tmp_path):
    p = tmp_path / "b.smtx"
    p.write_text("3,4,3\n0 1\n2 3 99\n1 3 0\n")  # row pointers over two lines; 99 ends the pointer line
    r, c, rp, ci = io.load_smtx(str(p))
    assert (r, c) == (3, 4) and list(rp) == [0, 1, 2, 3] and list(ci) == [1, 3, 0]


@pytest.mark.parametrize("text", ["3, 4\n", "2,2,1\n0 1\n", "2,2,1\n0 1 1\n5\n", "2,2,2\n0 1 1\n0 1\n"])
def test_smtx_malformed(tmp_path, text):
    p = tmp_path / "bad.smtx"
    p.write_text(text)
    with pytest.raises(ValueError):
        io.load_smtx(str(p))


def test_missing_files_raise():
    with pytest.raises(FileNotFoundError):
        io.load_smtx("/nonexistent/x.smtx")
    with pytest.raises(FileNotFoundError):
        io.read_mtx("/nonexistent/x.mtx")


# ---------------------------------------------------------------------------- .mtx
def test_mtx_round_trip_general(tmp_path):
    A = synth.row_skew(41, 29, 0.7, seed=2, std=1.0)
    rows, cols, rp, ci, v = _csr(A)
    p = tmp_path / "g.mtx"
    io.write_mtx(str(p), rows, cols, rp, ci, v)
    r, c, rp2, ci2, v2 = io.read_mtx(str(p))
    assert (r, c) == (rows, cols)
    np.testing.assert_array_equal(io.csr_to_dense(r, c, rp2, ci2, v2), A)


def test_mtx_symmetric_pattern_comments(tmp_path):
    p = tmp_path / "s.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n% a comment\n%\n3 3 3\n1 1\n3 1\n2 2\n")
    r, c, rp, ci, v = io.read_mtx(str(p))
    D = io.csr_to_dense(r, c, rp, ci, v)
    np.testing.assert_array_equal(D, np.array([[1, 0, 1], [0, 1, 0], [1, 0, 0]], dtype=np.float32))


@pytest.mark.parametrize("body,err", [
    ("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n", "coordinate"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n1 1 2.0\n", "repeated"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n", "outside"),
    ("%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1.0\n", "entries expected"),
    ("not a header\n", "Matrix Market"),
])
def test_mtx_errors(tmp_path, body, err):
    p = tmp_path / "e.mtx"
    p.write_text(body)
    with pytest.raises(ValueError, match=err):
        io.read_mtx(str(p))


@pytest.mark.skipif(not (REF_MTX and os.path.exists(REF_MTX)), reason="reference checkout absent")
def test_mtx_reads_reference_bundled_matrix():
    """The reference's bundled random_90_768_768.mtx: the first 96 rows equal the golden fixture."""
    r, c, rp, ci, v = io.read_mtx(REF_MTX)
    assert (r, c) == (768, 768) and rp[-1] == 58982
    g = np.load(os.path.join(GOLDEN, "mtx_random90_rows0_96_n16.npz"))
    A = io.csr_to_dense(r, c, rp, ci, v)[:96]
    G = io.csr_to_dense(96, 768, g["row_ptrs"], g["col_inds"], g["values"])
    np.testing.assert_array_equal(A, G)


def test_packed_header_rejects_other_files(tmp_path):
    p = tmp_path / "x.bin"
    p.write_bytes(b"NOTAPACK" + b"\0" * 32)
    with pytest.raises(ValueError, match="not a packed-weight file"):
        io.read_packed_header(str(p))


# ---------------------------------------------------------------------------- packed format (GPU)
@pytest.mark.gpu
@pytest.mark.parametrize("case", ["f32_identity_tiled", "bf16_400fa", "f16_scaled", "f32_coloffset_mtile"])
def test_packed_file_round_trip(cuda, tmp_path, case):
    import torch
    from spreg import _lib
    from spreg.mapping import Mapping
    from spreg.packed import PackedMatrix
    A = synth.row_skew(133, 300, 0.9, seed=5, std=1.0)
    kw = dict(f32_identity_tiled=dict(m=Mapping.identity(4), k_tile=128),
              bf16_400fa=dict(m=Mapping.load("400fa"), value_dtype=_lib.BF16),
              f16_scaled=dict(m=Mapping.identity(2), value_dtype=_lib.F16, k_tile=64),
              f32_coloffset_mtile=dict(m=Mapping.identity(4), m_tile=16, col_offset=7))[case]
    m = kw.pop("m")
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), m, **kw)
    p = str(tmp_path / "w.spk")
    io.save_packed(pm, p, nr=64)
    h = io.read_packed_header(p)
    assert h["version"] == io.FORMAT_VERSION and h["mapping_id"] == m.mapping_id and h["nr"] == 64
    q = io.load_packed(p)
    a1, d1, s1 = pm.to_host()
    a2, d2, s2 = q.to_host()
    assert np.array_equal(a1, a2) and np.array_equal(d1, d2)
    assert (s1 is None and s2 is None) or np.array_equal(s1, s2)
    for k in ("nnz", "padding", "num_values", "num_col_indices", "arena_bytes", "required_storage", "empty_units"):
        assert q.info[k] == pm.info[k], k
    off = kw.get("col_offset", 0)
    dt = {_lib.F32: torch.float32, _lib.BF16: torch.bfloat16, _lib.F16: torch.float16}[pm.value_dtype]
    B = torch.from_numpy(synth.dense(300 + off, 64, seed=6)).to(dt).cuda()
    c1, c2 = pm.execute(B).cpu().numpy(), q.execute(B).cpu().numpy()
    assert np.array_equal(c1.view(np.uint32), c2.view(np.uint32))


@pytest.mark.gpu
def test_packed_file_corruption_is_caught(cuda, tmp_path):
    import json
    import struct
    import zlib

    import torch
    from spreg import _lib
    from spreg.mapping import Mapping
    from spreg.packed import PackedMatrix
    A = synth.row_skew(64, 256, 0.9, seed=8, std=1.0)
    pm = PackedMatrix.from_dense(torch.from_numpy(A).cuda(), Mapping.identity(4), k_tile=128)
    p = str(tmp_path / "w.spk")
    io.save_packed(pm, p)
    raw = bytearray(open(p, "rb").read())
    hlen = struct.unpack("<II", raw[8:16])[1]
    h = json.loads(raw[16:16 + hlen])
    body = 16 + hlen
    # 1. a flipped payload byte fails the CRC
    bad = bytearray(raw)
    bad[body + 3] ^= 0xFF
    open(p, "wb").write(bad)
    with pytest.raises(ValueError, match="corrupt"):
        io.load_packed(p)

    # 2. a column index moved out of its K tile, with the CRC recomputed: the device check refuses it
    arena = bytearray(raw[body: body + h["arena_bytes"]])
    descs = np.frombuffer(bytes(raw[body + h["arena_bytes"]: body + h["arena_bytes"] + h["descs_bytes"]]),
                          dtype=np.dtype([("values_off", "<i8"), ("cols_off", "<i8"), ("counts_off", "<i8"),
                                          ("num_values", "<i4"), ("num_cols", "<i4")]))
    u = int(np.argmax(descs["num_cols"] > 0))
    co = int(descs[u]["cols_off"])
    arena[co: co + 4] = struct.pack("<i", 255)  # unit u lies in K tile 0 (columns 0 .. 127)
    h2 = dict(h)
    h2["crc32"] = [zlib.crc32(bytes(arena))] + h["crc32"][1:]
    hb = json.dumps(h2, sort_keys=True).encode()
    out = raw[:8] + struct.pack("<II", 1, len(hb)) + hb + bytes(arena) + raw[body + h["arena_bytes"]:]
    open(p, "wb").write(out)
    with pytest.raises(_lib.SpregError, match="K tile"):
        io.load_packed(p)

    # 3. a descriptor pointing past the arena
    d2 = descs.copy()
    d2[0]["values_off"] = h["arena_bytes"] + 64
    db = d2.tobytes()
    h3 = dict(h)
    h3["crc32"] = [h["crc32"][0], zlib.crc32(db), h["crc32"][2]]
    hb = json.dumps(h3, sort_keys=True).encode()
    out = (raw[:8] + struct.pack("<II", 1, len(hb)) + hb + raw[body: body + h["arena_bytes"]] + db
           + raw[body + h["arena_bytes"] + h["descs_bytes"]:])
    open(p, "wb").write(out)
    with pytest.raises(_lib.SpregError, match="outside the arena"):
        io.load_packed(p)


@pytest.mark.gpu
def test_mtx_to_packed_execute(cuda, tmp_path):
    import torch
    from spreg.mapping import Mapping
    from spreg.packed import PackedMatrix
    A = synth.row_skew(90, 120, 0.85, seed=9, std=1.0)
    rows, cols, rp, ci, v = _csr(A)
    p = str(tmp_path / "a.mtx")
    io.write_mtx(p, rows, cols, rp, ci, v)
    r, c, rp2, ci2, v2 = io.read_mtx(p)
    m = Mapping.identity(4)
    pm = PackedMatrix.from_csr(torch.from_numpy(rp2).cuda(), torch.from_numpy(ci2).cuda(),
                               torch.from_numpy(v2).cuda(), (r, c), m)
    B = synth.dense(120, 40, seed=10)
    got = pm.execute(torch.from_numpy(B).cuda()).cpu().numpy()
    want = O.Packed(O.Tables.of(m), io.csr_to_dense(r, c, rp2, ci2, v2)).execute(B)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
