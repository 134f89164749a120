"""The allocation-free TMEM update (rdp_tmem_update_noalloc) against the processor's own TMEM path.

Some callers cannot allocate device memory -- an emulator frame loop recorded inside a CUDA stream
capture, where cudaMalloc is not allowed, or an application that owns every device buffer itself.
For them the library offers one entry point whose scratch lives in a fixed device array.  This test
feeds the same texture loads through the normal C ABI (rdp_cp_enqueue + rdp_cp_get_tmem) and through
the allocation-free entry point with caller-owned torch buffers, twice in a row (the second call
starts from the first call's TMEM and reuses the shared scratch), and requires identical TMEM words.
TMEM is integer data: the tolerance is exact equality.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RDP_OK, RDP_ERR_TOO_LARGE = 0, 6
MAX_UPLOADS = 1024

UPLOAD = np.dtype([("width", "<i4"), ("height", "<i4"), ("min_t_mod", "<f4"), ("max_t_mod", "<f4"),
                   ("vram_addr", "<i4"), ("vram_width", "<i4"), ("vram_size", "<i4"),
                   ("vram_effective_width", "<i4"), ("tmem_offset", "<i4"), ("tmem_stride_words", "<i4"),
                   ("tmem_size", "<i4"), ("tmem_fmt", "<i4"), ("mode", "<i4"), ("inv_tmem_stride_words", "<f4"),
                   ("dxt", "<i4"), ("padding", "<i4")])
assert UPLOAD.itemsize == 64


def _load_commands(addr, width, height, stride_bytes, tmem_bytes):
    """RDP words loading an RGBA16 width x height texture at `addr` into TMEM via LoadTile (tile 7)."""
    line_qw, tmem_qw = stride_bytes // 8, tmem_bytes // 8
    return [
        (0x3d << 24) | (0 << 21) | (2 << 19) | (width - 1), addr,
        (0x35 << 24) | (0 << 21) | (2 << 19) | (line_qw << 9) | tmem_qw, 7 << 24,
        (0x34 << 24), (7 << 24) | (((width - 1) << 2) << 12) | ((height - 1) << 2),
    ]


def _upload_plan(addr, width, height, stride_bytes, tmem_bytes):
    """The upload plan the processor derives for that LoadTile (16-bit texels, 16-bit tile)."""
    u = np.zeros(1, UPLOAD)
    eff = (width + 3) & ~3
    u["width"], u["height"] = eff, height
    u["vram_addr"], u["vram_width"], u["vram_size"], u["vram_effective_width"] = addr, width, 2, eff
    u["tmem_offset"], u["tmem_stride_words"] = tmem_bytes & 0xfff, stride_bytes // 2
    u["tmem_size"], u["tmem_fmt"], u["mode"] = 2, 0, 0
    u["inv_tmem_stride_words"] = np.float32(1.0) / np.float32(stride_bytes // 2)
    return u


LOADS_FIRST = [(0x600000, 32, 32, 64, 0), (0x601000, 16, 16, 32, 2048)]
LOADS_SECOND = [(0x602000, 16, 32, 32, 512), (0x603000, 8, 8, 16, 3584)]


def test_noalloc_tmem_update_matches_processor():
    torch = pytest.importorskip("torch")
    from rdp_gb300 import CommandProcessor
    from rdp_gb300.native import lib

    L = lib()
    fn = L.rdp_tmem_update_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int

    rdram_size = 8 << 20
    rng = np.random.default_rng(1234)
    rdram = np.zeros(rdram_size, np.uint8)
    rdram[0x600000:0x604000] = rng.integers(0, 256, 0x4000, dtype=np.uint8)

    dev = torch.device("cuda:0")
    rdram_dev = torch.from_numpy(rdram.copy()).to(dev)
    tmem_dev = torch.zeros(2048, dtype=torch.int16, device=dev)
    stream = torch.cuda.current_stream(dev)

    with CommandProcessor(rdram.copy(), rdram_size=rdram_size) as cp:
        for loads in (LOADS_FIRST, LOADS_SECOND):
            words = sum((_load_commands(*l) for l in loads), [])
            cp.enqueue_command(np.array(words, np.uint32))
            expected = cp.get_tmem()

            plans = np.concatenate([_upload_plan(*l) for l in loads])
            uploads_dev = torch.from_numpy(plans.view(np.uint8).copy()).to(dev)
            snaps_dev = torch.zeros((len(loads) + 1) * 2048, dtype=torch.int16, device=dev)
            before = tmem_dev.clone()
            rc = fn(uploads_dev.data_ptr(), len(loads), rdram_dev.data_ptr(), rdram_size, tmem_dev.data_ptr(),
                    snaps_dev.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
            assert rc == RDP_OK
            torch.cuda.synchronize(dev)
            got = tmem_dev.cpu().numpy().view(np.uint16)
            assert np.array_equal(got, expected), "TMEM differs in %d words" % int((got != expected).sum())
            snaps = snaps_dev.cpu().numpy().view(np.uint16).reshape(len(loads) + 1, 2048)
            assert np.array_equal(snaps[0], before.cpu().numpy().view(np.uint16))
            assert np.array_equal(snaps[-1], expected)


def test_noalloc_rejects_too_many_uploads():
    from rdp_gb300.native import lib
    fn = lib().rdp_tmem_update_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    # Checked before any pointer is touched or any work is queued.
    assert fn(1, MAX_UPLOADS + 1, 1, 8 << 20, 1, 1, None) == RDP_ERR_TOO_LARGE
