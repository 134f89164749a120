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


def test_enqueue_many_rejects_a_handle_given_twice():
    """Two host threads on one instance's recorder would race: a handle that appears twice is
    rejected before any handle is dereferenced or any thread starts (the handles here are
    stand-in addresses, never valid processors)."""
    lib = ctypes.CDLL(native.library_path())
    f = lib.rdp_batch_enqueue_many
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p),
                  ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint32), ctypes.c_void_p, ctypes.c_uint32]
    words = (ctypes.c_uint32 * 2)(0x29 << 24, 0)
    for handles in ([0x1000, 0x2000, 0x1000], [0x3000, 0x3000]):
        n = len(handles)
        insts = (ctypes.c_void_p * n)(*handles)
        wptrs = (ctypes.c_void_p * n)(*([ctypes.addressof(words)] * n))
        counts = (ctypes.c_uint32 * n)(*([2] * n))
        assert f(ctypes.c_void_p(0x10), n, insts, wptrs, counts, None, 2) == native.RDP_ERR_INVALID


def test_cpp_facade_header_compiles():
    """include/rdp_cuda.hpp (RDP::CommandProcessor over the C ABI) and the C++ program that the GPU
    test drives through it compile as C++17 (no GPU needed)."""
    import shutil
    import subprocess
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if not shutil.which("g++"):
        import pytest
        pytest.skip("no g++")
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "facade_test.cpp")],
                   check=True)


def test_create_rejects_inconsistent_upscaling_flags():
    """rdp_cp_create checks its flags before touching a device: super-sampled readback needs an
    upscaling factor (Renderer::init_renderer, rdp_renderer.cpp:59-60), and upscaling needs hidden
    RDRAM of half the RDRAM size (the multisampled slices are addressed that way)."""
    lib = native.lib()
    rd = (ctypes.c_uint8 * (1 << 20))()
    cases = [(native.CREATE_SUPER_SAMPLED_READ_BACK, 1 << 19),
             (native.CREATE_UPSCALING_2X, 1 << 18),
             (native.CREATE_UPSCALING_4X | native.CREATE_SUPER_SAMPLED_READ_BACK, 1 << 20),
             (1 << 9, 1 << 19)]
    for flags, hidden in cases:
        info = native._CreateInfo(ctypes.addressof(rd), 0, 1 << 20, hidden, flags, 0)
        h = ctypes.c_void_p()
        assert lib.rdp_cp_create(ctypes.byref(info), ctypes.byref(h)) == native.RDP_ERR_INVALID, hex(flags)
        assert not h.value
