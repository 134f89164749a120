"""Internal upscaling (2x / 4x / 8x) and super-sampled readback through the C ABI against the CPU
oracle (rdp_renderer.cpp:545-601, 1937-2085, 2223-2342; update_upscaled_domain_*.comp).

Compared bit for bit after each stream: RDRAM, hidden RDRAM and TMEM (the 1x rendering, or the
resolve with super-sampled readback), and the multisampled RDRAM / hidden RDRAM the upscaled passes
render into (factor^2 slices).  Upscaled scanout (the fetch from the multisampled copy, the VI at
the scaled resolution, downscale_steps) is compared image for image."""
import numpy as np
import pytest

from rdp_gb300 import CommandProcessor, ScanoutOptions, VIRegister, cmdgen
from rdp_testutil import diff_report

pytestmark = pytest.mark.gpu

F = cmdgen.FLAGS
RDRAM = 8 << 20


def _stream(config, **kw):
    p = cmdgen.default_params(config, **kw)
    words, rdram, _ = cmdgen.generate_stream(p)
    return words, rdram


def _compare(cp, o):
    errs = [diff_report("rdram", cp.begin_read_rdram().copy(), o.rdram()),
            diff_report("hidden", cp.begin_read_hidden_rdram().copy(), o.hidden()),
            diff_report("tmem", cp.get_tmem().view(np.uint8), o.tmem().view(np.uint8)),
            diff_report("upscaled rdram", cp.upscaled_rdram(), o.upscaled_rdram()),
            diff_report("upscaled hidden", cp.upscaled_hidden_rdram(), o.upscaled_hidden())]
    errs = [e for e in errs if e]
    assert not errs, "; ".join(errs)


def _run(segments, rdram, factor, ssaa=False, dither=False):
    """segments: command word arrays, or (offset, bytes) CPU writes to RDRAM between them."""
    from oracle import Oracle
    o = Oracle(RDRAM)
    o.set_upscaling(factor, ssaa, dither)
    o.write_rdram(rdram)
    rd = np.array(rdram, dtype=np.uint8, copy=True)
    with CommandProcessor(rd, rdram_size=RDRAM, upscaling=factor, super_sampled_readback=ssaa,
                          super_sampled_dither=dither) as cp:
        assert cp.get_scaling_factor() == factor
        for seg in segments:
            if isinstance(seg, tuple):
                off, data = seg
                host = cp.begin_read_rdram()
                host[off:off + len(data)] = data
                cp.end_write_rdram()
                o.rdram()  # begin_read_rdram idles: the oracle's pass ends there too
                o.write_rdram(data, off)
            else:
                cp.enqueue_command(seg)
                assert o.enqueue(seg) == len(seg)
        cp.wait_for_timeline(cp.signal_timeline())
        _compare(cp, o)
        ms = cp.upscaled_rdram()
    return ms


@pytest.mark.parametrize("factor", [2, 4])
def test_textured_depth_frame_upscaled(factor):
    # 320x240 RGBA5551 + Z16, 2-cycle textured triangles: rendered at 1x and again at the factor.
    words, rdram = _stream(cmdgen.CONFIG_TEXTURED, seed=0, num_prims=1200)
    ms = _run([words], rdram, factor)
    # The upscaled passes wrote every slice (not only a replicated 1x image).
    slices = ms.reshape(factor * factor, RDRAM)
    assert all(np.count_nonzero(slices[i] != slices[0]) for i in range(1, factor * factor))


def test_plain_frame_upscaled_8x():
    words, rdram = _stream(cmdgen.CONFIG_PLAIN, seed=1, num_prims=500)
    _run([words], rdram, 8)


def test_mixed_frame_upscaled():
    # 640x480 RGBA8888 with copy-mode rectangles (native resolution quirk), TLUT triangles, fill
    # rectangles, LOD: the copy-mode image is 16-bit and narrower, so it goes through the "pre"
    # updates only.
    words, rdram = _stream(cmdgen.CONFIG_MIXED, seed=0, num_prims=1500, num_frames=1)
    _run([words], rdram, 2)


def test_cpu_writes_between_passes_reach_the_upscaled_domain():
    # RDRAM the CPU writes after a pass (inside and outside the image) is propagated to every sample
    # by the next pass's "pre" update; what the 1x passes draw is not (the upscaled pass draws it).
    words, rdram = _stream(cmdgen.CONFIG_TEXTURED, seed=2, num_prims=800)
    from rdp_gb300.dump import split_commands
    half = len(words) // 2
    cut = 0
    for _, w in split_commands(words):  # a command boundary near the middle
        if cut >= half:
            break
        cut += len(w)
    rng = np.random.default_rng(5)
    patch = rng.integers(0, 256, 64 * 1024, dtype=np.uint8)
    _run([words[:cut], (cmdgen.color_addr() + 4096, patch), words[cut:]], rdram, 2)


@pytest.mark.parametrize("fb_format", [cmdgen.FB_RGBA5551, cmdgen.FB_RGBA8888, cmdgen.FB_I8, cmdgen.FB_IA88,
                                       cmdgen.FB_I4])
def test_fuzz_streams_upscaled(fb_format):
    # Every framebuffer format: 16/32-bit images at least 256 wide render upscaled, the others only
    # feed the upscaled domain through the "pre" updates.
    p = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=7, num_prims=300, fb_format=fb_format,
                              flags=F["FUZZ"] | F["CLEAR"])
    words, rdram, _ = cmdgen.generate_stream(p)
    _run([words], rdram, 2)


@pytest.mark.parametrize("fb_format", [cmdgen.FB_RGBA5551, cmdgen.FB_RGBA8888, cmdgen.FB_I8, cmdgen.FB_IA88])
def test_super_sampled_readback(fb_format):
    # Every pass renders only upscaled and is resolved into RDRAM.
    p = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=11, num_prims=300, fb_format=fb_format,
                              flags=F["FUZZ"] | F["CLEAR"])
    words, rdram, _ = cmdgen.generate_stream(p)
    _run([words], rdram, 2, ssaa=True)


@pytest.mark.parametrize("dither", [False, True])
def test_super_sampled_readback_textured_4x(dither):
    words, rdram = _stream(cmdgen.CONFIG_TEXTURED, seed=3, num_prims=600)
    _run([words], rdram, 4, ssaa=True, dither=dither)


def _start(a, b):
    return ((a & 0x3ff) << 16) | (b & 0x3ff)


def _vi_regs(frame):
    # The mixed frame's 640x480 RGBA8888 image: AA + resampling, divot, dither filter, interlaced.
    return {VIRegister.Control: 3 | (1 << 4) | (1 << 16) | (1 << 6), VIRegister.Origin: cmdgen.color_addr(),
            VIRegister.Width: 640, VIRegister.VSync: 525, VIRegister.VStart: _start(34, 34 + 480),
            VIRegister.HStart: _start(108, 108 + 640), VIRegister.XScale: 1024, VIRegister.YScale: 2048,
            VIRegister.VCurrentLine: frame & 1}


@pytest.mark.parametrize("factor,downscale", [(2, 0), (2, 1), (4, 1)])
def test_upscaled_scanout(factor, downscale):
    from oracle import Oracle
    words, rdram = _stream(cmdgen.CONFIG_MIXED, seed=4, num_prims=600, num_frames=1)
    o = Oracle(RDRAM)
    o.set_upscaling(factor)
    o.write_rdram(rdram)
    rd = np.array(rdram, dtype=np.uint8, copy=True)
    opts = ScanoutOptions()
    opts.downscale_steps = downscale
    opts.blend_previous_frame = 1
    opts.upscale_deinterlacing = 0
    ow = opts.as_words()
    with CommandProcessor(rd, rdram_size=RDRAM, upscaling=factor) as cp:
        cp.enqueue_command(words)
        o.enqueue(words)
        for frame in range(2):
            for r, v in _vi_regs(frame).items():
                cp.set_vi_register(r, v)
                o.set_vi_register(r, v)
            img = cp.scanout_sync(opts)
            ref = o.scanout(ow)
            assert img is not None and ref is not None
            assert img.shape == ref.shape == (480 * factor >> downscale, 640 * factor >> downscale)
            assert np.array_equal(img, ref), "frame %d: %d pixels differ" % (frame, np.count_nonzero(img != ref))


def test_upscaling_limits():
    # An upscaling processor cannot record sync-point captures, and batch instances cannot upscale
    # (rdp_cp_capture_begin / rdp_batch_add_instance return RDP_ERR_INVALID).
    import ctypes
    from rdp_gb300 import native
    with CommandProcessor(rdram_size=RDRAM, upscaling=2) as cp:
        assert native.lib().rdp_cp_capture_begin(cp._h) == native.RDP_ERR_INVALID
        # Still usable afterwards.
        cp.enqueue_command(np.array([0x29000000, 0], dtype=np.uint32))
        cp.wait_for_timeline(cp.signal_timeline())
    b = native.Batch()
    try:
        rd = np.zeros(RDRAM, dtype=np.uint8)
        info = native._CreateInfo(rd.ctypes.data, 0, RDRAM, RDRAM // 2, native.CREATE_UPSCALING_2X, 0)
        h = ctypes.c_void_p()
        assert native.lib().rdp_batch_add_instance(b._h, ctypes.byref(info), ctypes.byref(h)) == native.RDP_ERR_INVALID
    finally:
        b.close()


def test_upscaling_with_command_thread():
    # Decoding on the processor's command thread drives the same upscaled passes.
    from oracle import Oracle
    words, rdram = _stream(cmdgen.CONFIG_TEXTURED, seed=5, num_prims=400)
    o = Oracle(RDRAM)
    o.set_upscaling(2)
    o.write_rdram(rdram)
    o.enqueue(words)
    rd = np.array(rdram, dtype=np.uint8, copy=True)
    with CommandProcessor(rd, rdram_size=RDRAM, upscaling=2, command_thread=True) as cp:
        for chunk in np.array_split(words, 5):
            cp.enqueue_command(chunk)
        cp.wait_for_timeline(cp.signal_timeline())
        _compare(cp, o)
