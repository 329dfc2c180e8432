"""The drop-in boundary: libff.so builds, loads, and exports exactly what
include/ff.h declares.  No compute call is made here (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ff.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ff_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from tsl_array_n_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from tsl_array_n_gb300 import _lib
    assert set(declared_functions()) == set(_lib.PROTOTYPES)


def test_version_and_error_string(lib):
    assert lib.ff_version().startswith(b"ff ")
    assert isinstance(lib.ff_last_error(), bytes)


def test_null_arguments_are_errors_not_crashes(lib):
    assert lib.ff_ctx_create(0, None) == -1
    assert b"NULL" in lib.ff_last_error()
    assert lib.ff_field_upload(None, None, 0) == -1
    assert lib.ff_pressure3_project(None, None, None, None, None, None, None, None) == -1


def test_no_device_fails_loudly(lib):
    """Without a CUDA device the context cannot be created: FF_E_CUDA, never a
    CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert lib.ff_ctx_create(0, C.byref(h)) == -2
    assert not h.value


def test_package_refuses_without_library(tmp_path, monkeypatch):
    """A missing libff.so raises instead of falling back to anything."""
    from tsl_array_n_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(_lib.FFError):
        _lib.load(str(tmp_path / "missing.so"))
