"""VI scanout parity: the CUDA VI kernels (through the C ABI) against the CPU oracle
on random RDRAM and random VI register states, following the reference's VI
conformance variants (vi_conformance.cpp:52-160): AA modes, RGBA5551/8888, divot,
dither filter, gamma, gamma dither, serrate, PAL, random scale/bias and random
H/V start.  The whole RGBA8 output is compared (the reference compares RGB)."""
import zlib

import numpy as np
import pytest

from rdp_gb300 import CommandProcessor, ScanoutOptions, VIRegister

pytestmark = pytest.mark.gpu

RDRAM = 8 << 20


def _start(a, b):
    return ((a & 0x3ff) << 16) | (b & 0x3ff)


def _scale(factor, bias):
    return ((bias & 0xfff) << 16) | (factor & 0xfff)


def _variant_regs(rng, v, iteration):
    ctrl = (v["aa"] << 8) | v["fmt"]
    ctrl |= (1 << 4) if v["divot"] else 0
    ctrl |= (1 << 16) if v["dither"] else 0
    ctrl |= (1 << 3) if v["gamma"] else 0
    ctrl |= (1 << 2) if v["gamma_dither"] else 0
    ctrl |= (1 << 6) if v["serrate"] else 0
    pal = v["pal"]
    regs = {
        VIRegister.Control: ctrl,
        VIRegister.Origin: 567123,
        VIRegister.Width: 100,
        VIRegister.VSync: 625 if pal else 525,
        VIRegister.VStart: _start(44 if pal else 34, (44 if pal else 34) + 224 * 2),
        VIRegister.XScale: _scale(v.get("x_scale", 1024), 0),
        VIRegister.YScale: _scale(v.get("y_scale", 1024), 0),
        VIRegister.HStart: _start(128 if pal else 108, (128 if pal else 108) + 640),
        VIRegister.VCurrentLine: int(v["serrate"]) & (iteration & 1),
    }
    if v.get("random_scale"):
        regs[VIRegister.XScale] = _scale(int(rng.integers(0, 1 << 32)), int(rng.integers(0, 1 << 32)))
        regs[VIRegister.YScale] = _scale(int(rng.integers(0, 1 << 32)), int(rng.integers(0, 1 << 32)))
    if v.get("random_start"):
        regs[VIRegister.HStart] = _start(int(rng.integers(0, 1 << 32)), int(rng.integers(0, 1 << 32)))
        regs[VIRegister.VStart] = _start(int(rng.integers(0, 1 << 32)), int(rng.integers(0, 1 << 32)))
    return regs


VARIANTS = {
    "5551_replicate": dict(aa=3, fmt=2, divot=False, dither=False, gamma=False, gamma_dither=False, serrate=False, pal=False),
    "5551_aa_divot_dither_gamma": dict(aa=1, fmt=2, divot=True, dither=True, gamma=True, gamma_dither=False, serrate=False, pal=False),
    "5551_aa_always_gamma_dither": dict(aa=0, fmt=2, divot=True, dither=True, gamma=True, gamma_dither=True, serrate=False, pal=False),
    "8888_resamp_only": dict(aa=2, fmt=3, divot=False, dither=False, gamma=False, gamma_dither=True, serrate=False, pal=False),
    "8888_aa_divot": dict(aa=0, fmt=3, divot=True, dither=True, gamma=True, gamma_dither=True, serrate=False, pal=False),
    "5551_serrate_pal": dict(aa=0, fmt=2, divot=True, dither=True, gamma=True, gamma_dither=True, serrate=True, pal=True),
    "5551_scale_bias": dict(aa=0, fmt=2, divot=True, dither=True, gamma=True, gamma_dither=False, serrate=False, pal=False, random_scale=True),
    "8888_start": dict(aa=1, fmt=3, divot=True, dither=False, gamma=True, gamma_dither=True, serrate=True, pal=False, random_start=True),
    "5551_upscaled_fetch_bug": dict(aa=0, fmt=2, divot=True, dither=True, gamma=False, gamma_dither=False, serrate=False, pal=False, y_scale=512, x_scale=512),
    "blank_and_reserved": dict(aa=0, fmt=1, divot=True, dither=True, gamma=True, gamma_dither=False, serrate=False, pal=False),
}


@pytest.mark.parametrize("name", sorted(VARIANTS))
def test_vi_variant(name):
    from oracle import Oracle
    v = VARIANTS[name]
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    opts = ScanoutOptions(blend_previous_frame=1, upscale_deinterlacing=0)
    o = Oracle(RDRAM)
    with CommandProcessor(np.zeros(RDRAM, np.uint8), rdram_size=RDRAM) as cp:
        for it in range(6):
            rd = rng.integers(0, 256, RDRAM, dtype=np.uint8)
            hid = rng.integers(0, 4, RDRAM // 2, dtype=np.uint8)
            cp.write_rdram(rd)
            cp.write_hidden_rdram(hid)
            o.write_rdram(rd)
            o.write_hidden(hid)
            regs = _variant_regs(rng, v, it)
            if name == "blank_and_reserved":
                regs[VIRegister.Control] = (regs[VIRegister.Control] & ~3) | (it % 3)
            for r, val in regs.items():
                cp.set_vi_register(r, val)
                o.set_vi_register(r, val)
            got = cp.scanout_sync(opts)
            exp = o.scanout(opts.as_words())
            assert (got is None) == (exp is None), (it, got is None, exp is None)
            if got is not None:
                assert got.shape == exp.shape, (it, got.shape, exp.shape)
                diff = np.nonzero(got != exp)
                assert diff[0].size == 0, "iteration %d: %d pixels differ, first at %s (gpu %08x oracle %08x)" % (
                    it, diff[0].size, (diff[0][0], diff[1][0]), got[diff[0][0], diff[1][0]], exp[diff[0][0], diff[1][0]])


def test_vi_per_scanline_hstart_xscale():
    from oracle import Oracle
    rng = np.random.default_rng(7)
    opts = ScanoutOptions(blend_previous_frame=1, upscale_deinterlacing=0)
    o = Oracle(RDRAM)
    rd = rng.integers(0, 256, RDRAM, dtype=np.uint8)
    hid = rng.integers(0, 4, RDRAM // 2, dtype=np.uint8)
    with CommandProcessor(np.zeros(RDRAM, np.uint8), rdram_size=RDRAM) as cp:
        cp.write_rdram(rd)
        cp.write_hidden_rdram(hid)
        o.write_rdram(rd)
        o.write_hidden(hid)
        v = dict(aa=0, fmt=2, divot=True, dither=True, gamma=True, gamma_dither=False, serrate=False, pal=False)
        for r, val in _variant_regs(rng, v, 0).items():
            cp.set_vi_register(r, val)
            o.set_vi_register(r, val)
        for t in (cp, o):
            t.begin_vi_register_per_scanline(3)
        line = 40
        for _ in range(20):
            hs = _start(100 + int(rng.integers(0, 40)), 700 + int(rng.integers(0, 60)))
            xs = _scale(400 + int(rng.integers(0, 800)), int(rng.integers(0, 512)))
            line += int(rng.integers(5, 20))
            for t in (cp, o):
                t.set_vi_register_for_scanline(1, hs)
                t.set_vi_register_for_scanline(2, xs)
                t.latch_vi_register_for_scanline(line)
        for t in (cp, o):
            t.end_vi_register_per_scanline()
        got = cp.scanout_sync(opts)
        exp = o.scanout(opts.as_words())
        assert got is not None and np.array_equal(got, exp)


def test_vi_crop_persist_and_downscale_options():
    """ScanoutOptions beyond the filters (video_interface.cpp:1215-1310): the crop rectangle and the
    aspect-preserving overscan crop (doubled when interlaced), persist_frame_on_invalid_input (an
    invalid VI state within four frames of a valid one repeats the last image, later ones give no
    image) and downscale_steps (no effect at 1x scale), against the oracle frame by frame."""
    from oracle import Oracle
    rng = np.random.default_rng(11)
    rd = rng.integers(0, 256, RDRAM, dtype=np.uint8)
    hid = rng.integers(0, 4, RDRAM // 2, dtype=np.uint8)
    o = Oracle(RDRAM)
    o.write_rdram(rd)
    o.write_hidden(hid)
    base = dict(aa=0, fmt=2, divot=True, dither=True, gamma=True, gamma_dither=False, serrate=False, pal=False)
    serr = dict(base, serrate=True)
    cases = [
        (base, ScanoutOptions(crop_rect_enable=1, crop_left=13, crop_right=7, crop_top=5, crop_bottom=9), False),
        (serr, ScanoutOptions(crop_rect_enable=1, crop_left=3, crop_right=21, crop_top=4, crop_bottom=2,
                              upscale_deinterlacing=0), False),
        (base, ScanoutOptions(crop_overscan_pixels=8), False),
        (serr, ScanoutOptions(crop_overscan_pixels=6, upscale_deinterlacing=0), False),
        (base, ScanoutOptions(downscale_steps=3), False),
        # valid, then invalid states (h_start beyond the line): repeated within four frames, then none
        (base, ScanoutOptions(persist_frame_on_invalid_input=1), False),
    ] + [(base, ScanoutOptions(persist_frame_on_invalid_input=1), True)] * 6
    with CommandProcessor(np.zeros(RDRAM, np.uint8), rdram_size=RDRAM) as cp:
        cp.write_rdram(rd)
        cp.write_hidden_rdram(hid)
        none_seen = repeat_seen = 0
        for it, (v, opts, invalid) in enumerate(cases):
            regs = _variant_regs(rng, v, it)
            if invalid:
                regs[VIRegister.HStart] = _start(760, 900)  # h_start past the 640-pixel line
            for r, val in regs.items():
                cp.set_vi_register(r, val)
                o.set_vi_register(r, val)
            got = cp.scanout_sync(opts)
            exp = o.scanout(opts.as_words())
            assert (got is None) == (exp is None), it
            if got is not None:
                assert got.shape == exp.shape and np.array_equal(got, exp), it
            if invalid:
                none_seen += got is None
                repeat_seen += got is not None
        assert repeat_seen >= 1 and none_seen >= 1  # both sides of the four-frame window
    cropped = ScanoutOptions(crop_rect_enable=1, crop_left=13, crop_right=7, crop_top=5, crop_bottom=9)
    assert cropped.crop_left == 13
