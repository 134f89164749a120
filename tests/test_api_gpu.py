"""CommandProcessor API behaviour (rdp_device.hpp:111-197): validation reports, timeline
semantics, creation errors, quirks and frame contexts."""
import numpy as np
import pytest

from rdp_gb300 import CommandProcessor, RdpError, cmdgen
from rdp_testutil import assert_parity

pytestmark = pytest.mark.gpu


def _color_image(size, fmt, width, addr=0x100000):
    return [(0x3f << 24) | (fmt << 21) | (size << 19) | (width - 1), addr]


def _other_modes(cycle):
    return [(0x2f << 24) | (cycle << 20), 0]


SCISSOR = [(0x2d << 24), ((320 << 2) << 12) | (240 << 2)]


def _fill_rect(x0, y0, x1, y1):
    return [(0x36 << 24) | ((x1 << 2) << 12) | (y1 << 2), ((x0 << 2) << 12) | (y0 << 2)]


def test_validation_reports_fill_on_4bpp_and_copy_on_32bpp():
    seen = []
    with CommandProcessor() as cp:
        cp.set_validation_interface(lambda err, msg: seen.append((err, msg)))
        words = _color_image(0, 0, 320) + SCISSOR + _other_modes(3) + _fill_rect(0, 0, 15, 15)
        cp.enqueue_command(np.array(words, np.uint32))
        words = (_color_image(3, 0, 320) + _other_modes(2) +
                 [(0x24 << 24) | ((16 << 2) << 12) | (16 << 2), 0, 0, (4 << 10 << 16) | (1 << 10)])
        cp.enqueue_command(np.array(words, np.uint32))
        cp.idle()
    codes = [e for e, _ in seen]
    assert 0 in codes, seen  # RDP_VALIDATION_FILL_4BPP
    assert 4 in codes, seen  # RDP_VALIDATION_COPY_32BPP


def test_timeline_values_increase_and_unsignalled_values_are_rejected():
    p = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=2, num_prims=300)
    words, rdram, _ = cmdgen.generate_stream(p)
    with CommandProcessor(rdram.copy()) as cp:
        cp.enqueue_command(words)
        v1 = cp.signal_timeline()
        cp.enqueue_command(words)
        v2 = cp.signal_timeline()
        assert v2 > v1
        cp.wait_for_timeline(v2)
        cp.wait_for_timeline(v1)  # already complete
        with pytest.raises(RdpError):
            cp.wait_for_timeline(v2 + 5)


def test_create_rejects_bad_sizes():
    with pytest.raises(RdpError):
        CommandProcessor(rdram_size=3 << 20)
    with pytest.raises(RdpError):
        CommandProcessor(rdram_size=8 << 20, hidden_rdram_size=3 << 20)


def test_quirks_and_frame_contexts_match_the_oracle():
    # Non-native texture rectangles (quirks 0) on the textured / copy-rectangle mix, with the
    # quirk word sent in-band as the reference's MetaSetQuirks does.
    p = cmdgen.default_params(cmdgen.CONFIG_MIXED, seed=12, num_prims=800, num_frames=1)
    words, rdram, _ = cmdgen.generate_stream(p)
    stream = np.concatenate([np.array([0x04 << 24, 0], np.uint32), words])
    assert_parity(stream, rdram)
    p2 = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=13, num_prims=200)
    w2, rd2, _ = cmdgen.generate_stream(p2)
    with CommandProcessor(rd2.copy()) as cp:
        cp.enqueue_command(w2[: len(w2) // 2])
        cp.begin_frame_context()
        cp.enqueue_command(w2[len(w2) // 2:])
        cp.idle()
        from rdp_testutil import run_oracle
        o_rd = run_oracle(w2, rd2)[0]
        assert np.array_equal(cp.begin_read_rdram(), o_rd)
