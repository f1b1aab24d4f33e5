"""The C ABI library without a GPU: it loads, exports every symbol that
include/byo_gpu.h declares, the ctypes table matches the header, and device
calls report errors instead of crashing."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "byo_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(byo_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def L():
    from byo_gb300 import build as nb
    nb.build()
    from byo_gb300 import _abi
    return _abi.lib()


def test_exports_every_declared_symbol(L):
    names = _declared()
    assert len(names) >= 40
    for n in names:
        assert hasattr(L, n), n


def test_ctypes_table_matches_header():
    from byo_gb300 import _abi
    assert sorted(_abi.SIGNATURES) == _declared()


def test_version(L):
    assert L.byo_version().startswith(b"byo_gpu")


def test_null_arguments_are_rejected(L):
    from byo_gb300 import _abi
    assert L.byo_gpu_init(0, None) == _abi.BYO_EINVAL
    assert L.byo_bfs(None, 0, None, None, 0, None) == _abi.BYO_EINVAL
    assert L.byo_graph_num_vertices(None) == 0
    assert L.byo_cc(None, None) == _abi.BYO_EINVAL


def test_init_without_gpu_fails_cleanly(L):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from byo_gb300 import _abi
    h = ctypes.c_void_p()
    assert L.byo_gpu_init(0, ctypes.byref(h)) == _abi.BYO_EDEVICE
    assert not h.value
