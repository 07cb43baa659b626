"""The C ABI library loads and exports every function that include/*.h declares (no GPU call)."""
import glob
import os
import re

import pytest

from caroli_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(caroli_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ["caroli_ctx_create", "caroli_plan_upload", "caroli_sigma_upload", "caroli_solve_batch",
              "caroli_ctx_destroy"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    if not os.path.exists(_native.LIB_PATH):
        pytest.fail(f"{_native.LIB_PATH} not built (run __graft_entry__.build())")
    lib = _native.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_native, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_native, "_lib", None)
    with pytest.raises(_native.NativeError):
        _native.load()
