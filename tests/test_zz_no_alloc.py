"""The allocation-free TMEM update (rdp_tmem_update_noalloc) against the processor's own TMEM path.

Some callers cannot allocate device memory -- an emulator frame loop recorded inside a CUDA stream
capture, where cudaMalloc is not allowed, or an application that owns every device buffer itself.
For them the library offers one entry point whose scratch lives in a fixed device array.  This test
feeds the same texture loads through the normal C ABI (rdp_cp_enqueue + rdp_cp_get_tmem) and through
the allocation-free entry point with caller-owned torch buffers, twice in a row (the second call
starts from the first call's TMEM and reuses the shared scratch), and requires identical TMEM words.
The loads cover all three upload modes -- LoadTile, LoadTLUT and LoadBlock (its fp32 line
stepping) -- with plans checked against the oracle's planning on the CPU (tests/test_tmem_plans.py).
TMEM is integer data: the tolerance is exact equality.
"""
import ctypes

import numpy as np
import pytest

from tmem_plans import GROUP_FIRST, GROUP_SECOND, TEXTURE_BYTES, commands, plan

pytestmark = pytest.mark.gpu

RDP_OK, RDP_ERR_TOO_LARGE = 0, 6
MAX_UPLOADS = 1024


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
    lo, hi = TEXTURE_BYTES
    rdram[lo:hi] = rng.integers(0, 256, hi - lo, dtype=np.uint8)

    dev = torch.device("cuda:0")
    rdram_dev = torch.from_numpy(rdram.copy()).to(dev)
    tmem_dev = torch.zeros(2048, dtype=torch.int16, device=dev)
    stream = torch.cuda.current_stream(dev)

    with CommandProcessor(rdram.copy(), rdram_size=rdram_size) as cp:
        for loads in (GROUP_FIRST, GROUP_SECOND):
            words = sum((commands(l) for l in loads), [])
            cp.enqueue_command(np.array(words, np.uint32))
            expected = cp.get_tmem()

            plans = np.concatenate([plan(l) for l in loads])
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
