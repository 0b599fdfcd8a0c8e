"""C ABI checks that need no GPU: the library builds, loads and exports every
entry point declared in include/messi_gb300.h; host-side argument handling."""
import ctypes
import os
import re

import pytest

from messi_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "messi_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(messi_[a-z0-9_]+)\s*\(", text)))


def test_header_declarations_are_bound():
    names = _declared()
    assert "messi_felsenstein_pairs" in names and "messi_inside" in names
    assert set(names) <= set(_lib.EXPORTED), set(names) - set(_lib.EXPORTED)


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in _declared():
        assert hasattr(lib, name), name


def test_strerror_and_version():
    lib = _lib.load()
    assert lib.messi_strerror(_lib.MESSI_EINVAL).decode() == "invalid argument"
    assert lib.messi_strerror(0).decode() == "ok"
    assert lib.messi_version() >= 100


def test_null_arguments_are_rejected_without_a_gpu():
    lib = _lib.load()
    assert lib.messi_ctx_create(0, None) == _lib.MESSI_EINVAL
    assert lib.messi_ctx_destroy(None) == _lib.MESSI_EINVAL
    assert lib.messi_dataset_destroy(None) == _lib.MESSI_EINVAL
    assert lib.messi_ctx_last_launches(None, None) == _lib.MESSI_EINVAL


def test_ctx_create_reports_missing_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.messi_ctx_create(0, ctypes.byref(h)) == _lib.MESSI_ECUDA
    assert not h.value


def test_error_type_carries_status():
    with pytest.raises(_lib.MessiError) as e:
        _lib.check(_lib.MESSI_EINVAL, "probe")
    assert e.value.status == _lib.MESSI_EINVAL
