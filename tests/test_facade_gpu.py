"""The header-only C++ face of the library (include/rdp_cuda.hpp: RDP::CommandProcessor with the
reference's constructor and method names, rdp_device.hpp:111-197), driven by a compiled C++
program (tests/cpp/facade_test.cpp) the way an emulator drives the reference: commands in uneven
chunks, timeline signal / wait, the command-thread mode with the in-band meta ops (MetaFlush,
MetaSignalTimeline) in the stream, scanout_sync, scanout() returning the device image and
scanout_async_buffer().  Both renderings must equal the oracle's RDRAM, and every scanout the
oracle's VI output (exact: integer data)."""
import os
import subprocess

import numpy as np
import pytest

from rdp_gb300 import VIRegister, cmdgen, native
from rdp_testutil import run_oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _start(a, b):
    return ((a & 0x3ff) << 16) | (b & 0x3ff)


def _vi_regs():
    """320x240 RGBA5551 colour image scanned out at 640x240: AA filter with resampling, divot and
    dither filter, no gamma dither (so that two scanouts of one frame are the same image)."""
    return {VIRegister.Control: 2 | (1 << 4) | (1 << 16), VIRegister.Origin: cmdgen.color_addr(),
            VIRegister.Width: 320, VIRegister.VSync: 525, VIRegister.VStart: _start(34, 34 + 480),
            VIRegister.HStart: _start(108, 108 + 640), VIRegister.XScale: 512, VIRegister.YScale: 1024}


def _build(tmp_path):
    exe = tmp_path / "facade_test"
    lib_dir = os.path.dirname(native.library_path())
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", "facade_test.cpp"), "-o",
                    str(exe), "-L", lib_dir, "-lrdp_cuda", "-Wl,-rpath," + lib_dir, "-L",
                    os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(CUDA, "lib64")],
                   check=True)
    return exe


def _image(path):
    a = np.fromfile(path, dtype=np.uint32)
    return int(a[0]), int(a[1]), a[2:]


def test_cpp_facade_matches_oracle(tmp_path):
    exe = _build(tmp_path)
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=21, num_prims=1500)
    words, rdram, _ = cmdgen.generate_stream(p)
    words.astype(np.uint32).tofile(tmp_path / "words.bin")
    rdram.tofile(tmp_path / "rdram.bin")
    regs = _vi_regs()
    np.array([[int(r), v] for r, v in regs.items()], dtype=np.uint32).tofile(tmp_path / "vi.bin")
    out = subprocess.run([str(exe), str(tmp_path / "words.bin"), str(tmp_path / "rdram.bin"),
                          str(tmp_path / "vi.bin"), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "facade_test ok" in out.stdout

    o_rd, _, _, _ = run_oracle(words, rdram)
    for name in ("sync_rdram.bin", "threaded_rdram.bin"):
        got = np.fromfile(tmp_path / name, dtype=np.uint8)
        assert np.array_equal(got, o_rd), name

    from oracle import Oracle
    from rdp_gb300 import ScanoutOptions
    o = Oracle(8 << 20)
    o.write_rdram(o_rd)
    _, o_hid, _, _ = run_oracle(words, rdram)
    o.write_hidden(o_hid)
    for r, v in regs.items():
        o.set_vi_register(r, v)
    img = o.scanout(ScanoutOptions(blend_previous_frame=0, upscale_deinterlacing=0).as_words())
    assert img is not None
    for name in ("sync_vi.bin", "threaded_vi_device.bin", "threaded_vi_async.bin"):
        w, h, px = _image(tmp_path / name)
        assert (w, h) == (img.shape[1], img.shape[0]), name
        assert np.array_equal(px, img.reshape(-1)), name
