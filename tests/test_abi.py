"""The C ABI library: builds, loads, exports every symbol of include/pjg.h,
and fails loudly (no CPU fallback) when no GPU is visible."""

import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "pjg.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pjg_[a-z_]+)\s*\(", text)))


def test_header_symbols_exported():
    from pyjess_gb300 import _build, _native

    _build.build()
    lib = ctypes.CDLL(str(_build.LIB))
    syms = declared_symbols()
    assert len(syms) >= 14
    for name in syms:
        assert hasattr(lib, name), name
    assert sorted(_native.EXPORTED) == syms


def test_no_device_fails_loudly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from pyjess_gb300 import _native

    with pytest.raises(RuntimeError, match="no CUDA device"):
        _native.init(0)


def test_query_without_device_raises(t133, amy):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from pyjess_gb300 import Jess

    q = Jess([t133]).query(amy, 2, 2, 2)
    with pytest.raises(RuntimeError):
        next(q)
