"""The C ABI library loads, exports every function include/spreg.h declares, and its host-only
entry points (mapping tables, argument checks) behave as the reference interface does.  No
compute calls: these run without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from spreg import _lib
from spreg.mapping import Mapping
from spreg.sop_driver import Acc, make_sop_module

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "spreg.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(spreg_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_expected_surface():
    names = header_functions()
    for n in ("spreg_pack_csr", "spreg_execute", "spreg_execute_batched", "spreg_tile_pack_panel",
              "spreg_matmul_run", "spreg_last_error", "spreg_sort_and_encode_patterns"):
        assert n in names


def test_library_exports_every_declared_function():
    L = ctypes.CDLL(_lib.LIB_PATH)
    names = header_functions()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(_lib.PROTOTYPES), set(names) ^ set(_lib.PROTOTYPES)
    assert _lib.lib().spreg_version() >= 100


@pytest.mark.parametrize("mr", [2, 4, 6, 8])
def test_mapping_ids_match_oracle(mr):
    m = Mapping.identity(mr)
    assert m.nkern_patterns() == [int(x) for x in O.Tables.of(m).id_to_pattern[: 2 ** mr - 1]]
    assert m.encode(0) == _lib.ZERO_PATTERN_ID
    assert m.encode(1) == 0


def test_named_mapping_tables_match_oracle():
    for mid in ("400fa", "747f9", "33960", "75f82"):
        m = Mapping.load(mid)
        t = O.Tables.of(m)
        assert m.num_nkern() == t.num_nkern
        assert m.nkern_patterns() == [int(x) for x in t.id_to_pattern[: t.num_nkern]]
        for c in range(2 ** m.mr):
            assert m.encode(c) == (int(t.code_to_id[c]) if t.code_to_id[c] != -1 else -1)


def test_mapping_argument_errors():
    with pytest.raises(ValueError):
        Mapping(3, {1: [1]})
    offs = np.zeros(9, np.int32)
    h = ctypes.c_void_p()
    st = _lib.lib().spreg_mapping_create(3, offs.ctypes.data, offs.ctypes.data, None, 0, ctypes.byref(h))
    assert st == _lib.SPREG_ERR_INVALID_ARG and "M_r" in _lib.last_error()
    bad = Mapping(4, {p: [p] for p in range(1, 16)}, nanokernels=[1, 2, 4, 8])
    with pytest.raises(_lib.SpregError) as e:
        bad.handle
    assert "not a nanokernel" in str(e.value)
    assert e.value.status == _lib.SPREG_ERR_INVALID_ARG


def test_make_sop_module_without_gpu():
    m = Mapping.load("400fa")
    mod = make_sop_module(Acc(8, 2), m.nanokernels, m)
    assert mod.mapping.num_nkern() == 19
    assert mod.kernel_id.startswith("spreg_GB300_M8_N2_19k")
    with pytest.raises(AssertionError):
        make_sop_module(Acc(4, 4), [0, 1], lambda p: [p])


def test_error_status_and_message_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("checks the no-GPU failure path")
    m = Mapping.identity(4)
    rp = np.zeros(2, np.int32)
    csr = _lib.Csr(1, 1, 0, rp.ctypes.data, None, None)
    h = ctypes.c_void_p()
    st = _lib.lib().spreg_pack_csr(m.handle, ctypes.byref(csr), None, ctypes.byref(h), None)
    assert st != _lib.SPREG_OK and h.value is None
    assert _lib.last_error()
