"""Bit-exact parity of the CUDA path (through the C ABI) against the CPU oracle
on seeded command streams.  Compare = RDRAM + hidden RDRAM + TMEM bytes, as the
reference's conformance suites do (conformance_utils.hpp:282-304)."""
import pytest

from rdp_gb300 import cmdgen
from rdp_testutil import assert_parity

pytestmark = pytest.mark.gpu

F = cmdgen.FLAGS


def _stream(config, **kw):
    p = cmdgen.default_params(config, **kw)
    words, rdram, _ = cmdgen.generate_stream(p)
    return words, rdram


def test_plain_frame_full_size():
    # The plain frame: 320x240 RGBA5551, FillRect clear + 2,000 Gouraud triangles, seed 0.
    words, rdram = _stream(cmdgen.CONFIG_PLAIN, seed=0)
    assert_parity(words, rdram)


@pytest.mark.parametrize("seed", [1, 2])
def test_plain_frame_seeds(seed):
    words, rdram = _stream(cmdgen.CONFIG_PLAIN, seed=seed, num_prims=600)
    assert_parity(words, rdram, chunks=7)


def test_textured_depth_frame():
    # The textured, depth-tested 2-cycle frame at reduced primitive count.
    words, rdram = _stream(cmdgen.CONFIG_TEXTURED, seed=0, num_prims=1500)
    assert_parity(words, rdram)


def test_mixed_frame():
    # The mixed 640x480 RGBA8888 frame at reduced primitive count.  Its copy-mode rectangles
    # go to a second (16-bit) image, so the reference ends a pass at every image switch;
    # this path keeps both images in one pass and must still match bit for bit.
    words, rdram = _stream(cmdgen.CONFIG_MIXED, seed=0, num_prims=3000, num_frames=1)
    stats = assert_parity(words, rdram)
    assert stats["passes"] < stats["reference_passes"], stats


def test_mixed_two_frames():
    words, rdram = _stream(cmdgen.CONFIG_MIXED, seed=3, num_prims=800, num_frames=2)
    assert_parity(words, rdram)


@pytest.mark.parametrize("fb_format", [cmdgen.FB_RGBA5551, cmdgen.FB_RGBA8888, cmdgen.FB_I8, cmdgen.FB_IA88,
                                       cmdgen.FB_I4])
@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_fuzz_streams(fb_format, seed):
    # Random other-modes, combiner/blender selectors, texture formats, loads, scissor/interlace,
    # fill/copy/1-cycle/2-cycle triangles and rectangles on every framebuffer format.
    p = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=seed, num_prims=400, fb_format=fb_format,
                              flags=F["FUZZ"] | F["CLEAR"])
    words, rdram, _ = cmdgen.generate_stream(p)
    assert_parity(words, rdram)


@pytest.mark.parametrize("fb_format", [cmdgen.FB_RGBA5551, cmdgen.FB_I8, cmdgen.FB_RGBA8888])
@pytest.mark.parametrize("seed", [101, 102])
def test_fuzz_long_streams(fb_format, seed):
    # Longer fuzz streams: many colour-image switches (several images per pass, I8 among
    # them), loads from rendered images (read-after-write hazards), scissor/interlace.
    p = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=seed, num_prims=2500, fb_format=fb_format,
                              flags=F["FUZZ"] | F["CLEAR"])
    words, rdram, _ = cmdgen.generate_stream(p)
    assert_parity(words, rdram, chunks=3)
