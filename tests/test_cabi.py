"""The C ABI library loads and exports every entry point include/rdp_cuda.h declares
(no compute call is made: this runs without a GPU)."""
import ctypes
import os
import re

from rdp_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rdp\w*)\s*\(", src)) - {"rdp_validation_cb"})


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(native.library_path())
    names = _declared("rdp_cuda.h")
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(native.EXPORTED_SYMBOLS) <= set(names)


def test_cmdgen_exports():
    from rdp_gb300 import cmdgen
    lib = cmdgen._load()
    for n in _declared("rdp_cmdgen.h"):
        assert hasattr(lib, n), n


def test_no_cpu_fallback_when_library_missing(monkeypatch, tmp_path):
    monkeypatch.setattr(native, "_lib", None)
    monkeypatch.setattr(native, "library_path", lambda: str(tmp_path / "missing.so"))
    try:
        native.lib()
    except RuntimeError as e:
        assert "not built" in str(e)
    else:
        raise AssertionError("loading a missing library must fail")
