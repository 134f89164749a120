"""Properties of the oracle's internal upscaling (rdp_renderer.cpp:545-601, 2223-2342;
update_upscaled_domain_*.comp), checked on the CPU: the 1x rendering is unchanged by it, CPU
writes reach every sample through the "pre" update, native-resolution primitives fill whole sample
blocks, and the super-sampled resolve is the mean of the samples."""
import numpy as np
import pytest

from rdp_gb300 import cmdgen

RDRAM = 8 << 20


def _oracle(factor, ssaa=False, dither=False):
    from oracle import Oracle
    o = Oracle(RDRAM)
    o.set_upscaling(factor, ssaa, dither)
    return o


def _stream(config, **kw):
    p = cmdgen.default_params(config, **kw)
    words, rdram, _ = cmdgen.generate_stream(p)
    return words, rdram


def test_set_upscaling_rules():
    from oracle import Oracle
    o = Oracle(RDRAM)
    for bad in (0, 3, 16):
        with pytest.raises(ValueError):
            o.set_upscaling(bad)
    with pytest.raises(ValueError):
        Oracle(RDRAM, RDRAM // 4).set_upscaling(2)  # hidden RDRAM must be half of RDRAM
    o.set_upscaling(4)
    assert o.upscaling_factor() == 4 and o.upscaled_rdram().size == 16 * RDRAM


@pytest.mark.parametrize("factor", [2, 4])
def test_native_rendering_unchanged(factor):
    words, rdram = _stream(cmdgen.CONFIG_TEXTURED, seed=0, num_prims=300)
    from oracle import Oracle
    ref = Oracle(RDRAM)
    ref.write_rdram(rdram)
    ref.enqueue(words)
    o = _oracle(factor)
    o.write_rdram(rdram)
    o.enqueue(words)
    assert np.array_equal(o.rdram(), ref.rdram()) and np.array_equal(o.hidden(), ref.hidden())
    assert np.array_equal(o.tmem(), ref.tmem())


def test_cpu_write_reaches_every_sample():
    # A pass over a 320-wide RGBA5551 image, then a CPU write inside the image, then another pass:
    # its "pre" update copies the written bytes (which differ from the reference copy) to all slices.
    words, rdram = _stream(cmdgen.CONFIG_PLAIN, seed=0, num_prims=50)
    o = _oracle(2)
    o.write_rdram(rdram)
    o.enqueue(words)
    o.rdram()
    addr = cmdgen.color_addr() + 320 * 2 * 200  # row 200, below most of the scene
    patch = np.arange(256, dtype=np.uint8)
    o.write_rdram(patch, addr)
    o.enqueue(words)  # same image, same rows: the pass's range covers the patch
    ms = o.upscaled_rdram().reshape(4, RDRAM)
    rd = o.rdram()
    # Bytes the second pass did not overwrite keep the CPU's value in every slice.
    keep = rd[addr:addr + 256] == patch
    assert keep.any()
    for s in range(4):
        assert np.array_equal(ms[s, addr:addr + 256][keep], patch[keep])


def test_fill_rectangle_fills_whole_sample_blocks():
    # FillRectangle draws at native resolution (TRIANGLE_SETUP_DISABLE_UPSCALING_BIT): every sample
    # of a native pixel takes the fill colour, so all slices match the 1x image over the rectangle.
    words, rdram = _stream(cmdgen.CONFIG_PLAIN, seed=0, num_prims=0)  # just the full-screen clear
    o = _oracle(4)
    o.write_rdram(rdram)
    o.enqueue(words)
    rd = o.rdram()
    ms = o.upscaled_rdram().reshape(16, RDRAM)
    base, size = cmdgen.color_addr(), 320 * 240 * 2
    for s in range(16):
        assert np.array_equal(ms[s, base:base + size], rd[base:base + size])


def test_ssaa_resolve_is_the_mean_of_the_samples():
    words, rdram = _stream(cmdgen.CONFIG_PLAIN, seed=3, num_prims=200, fb_format=cmdgen.FB_RGBA8888)
    o = _oracle(2, ssaa=True)
    o.write_rdram(rdram)
    o.enqueue(words)
    rd = o.rdram()
    ms = o.upscaled_rdram().reshape(4, RDRAM)
    base, n = cmdgen.color_addr(), 320 * 240
    native = rd[base:base + 4 * n].view(np.uint32).astype(np.int64)
    samples = [ms[s, base:base + 4 * n].view(np.uint32).astype(np.int64) for s in range(4)]
    written = native != rdram[base:base + 4 * n].view(np.uint32)
    assert written.mean() > 0.5
    for shift in (24, 16, 8, 0):
        mean = (sum((v >> shift) & 0xff for v in samples) + 2) // 4
        assert np.array_equal(((native >> shift) & 0xff)[written], mean[written])


def test_upscaled_fill_picks_the_native_pixels_half_of_the_fill_colour():
    # Fill mode into a 320-wide RGBA5551 image: each native pixel takes the half of the 32-bit fill
    # colour its own address selects (memory_interfacing.h:440-470), in every sample.
    addr = 0x100000
    words = np.array([0x3f100000 | 319, addr,                 # SetColorImage RGBA5551, 320 wide
                      0x2d000000, (320 << 14) | (240 << 2),   # SetScissor 0,0 - 320,240
                      0x2f300000, 0,                          # SetOtherModes: fill cycle
                      0x37000000, 0x12345678,                 # SetFillColor: two different halves
                      0x36000000 | (63 << 14) | (15 << 2), (8 << 14) | (4 << 2),  # FillRectangle 8,4 - 63,15
                      0x29000000, 0], dtype=np.uint32)
    o = _oracle(2)
    o.enqueue(words)
    rd = o.rdram()
    ms = o.upscaled_rdram().reshape(4, RDRAM)
    row = rd[addr + 320 * 2 * 5:addr + 320 * 2 * 6].view(np.uint16)
    assert row[8] != row[9] and {int(row[8]), int(row[9])} == {0x1234, 0x5678}
    for sl in range(4):
        assert np.array_equal(ms[sl, addr:addr + 320 * 2 * 16], rd[addr:addr + 320 * 2 * 16])
