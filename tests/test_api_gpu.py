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


def _split_commands(words):
    """Word offsets where each RDP command starts (the RDP's command lengths)."""
    lengths = {0x08: 8, 0x09: 12, 0x0a: 24, 0x0b: 28, 0x0c: 24, 0x0d: 28, 0x0e: 40, 0x0f: 44, 0x24: 4, 0x25: 4}
    out, i = [], 0
    while i < len(words):
        out.append(i)
        i += lengths.get((int(words[i]) >> 24) & 63, 2)
    return out


def test_in_band_meta_ops_and_command_thread_match_the_oracle():
    """The reference's in-band meta ops in the command stream (rdp_device.cpp:926-952): MetaFlush
    and MetaIdle between commands and MetaSignalTimeline with its 64-bit value, decoded on the
    calling thread and on the command thread (command ring, command_ring.cpp:71-134).  The image
    equals the oracle's rendering of the same stream without the meta ops; a value signalled in band
    completes with everything before it."""
    from rdp_testutil import run_oracle
    p = cmdgen.default_params(cmdgen.CONFIG_MIXED, seed=31, num_prims=2500, num_frames=1)
    words, rdram, _ = cmdgen.generate_stream(p)
    starts = _split_commands(words)
    pieces = []
    for k, (a, b) in enumerate(zip(starts, starts[1:] + [len(words)])):
        pieces.append(words[a:b])
        if k % 500 == 499:
            pieces.append(np.array([0x02 << 24], np.uint32))  # MetaFlush
        if k % 700 == 699:
            pieces.append(np.array([0x03 << 24], np.uint32))  # MetaIdle
    stream = np.concatenate(pieces + [np.array([0x01 << 24, 41, 0], np.uint32)])  # MetaSignalTimeline 41
    o_rd, o_hid, _, _ = run_oracle(words, rdram)
    for threaded in (False, True):
        with CommandProcessor(rdram.copy(), command_thread=threaded) as cp:
            cuts = np.linspace(0, len(stream), 37).astype(int)  # uneven chunks cut through commands
            for a, b in zip(cuts[:-1], cuts[1:]):
                cp.enqueue_command(stream[a:b])
            cp.wait_for_timeline(41)
            v = cp.signal_timeline()
            assert v >= 1
            cp.wait_for_timeline(v)
            assert np.array_equal(cp.begin_read_rdram(), o_rd), "threaded=%s" % threaded
            assert np.array_equal(cp.begin_read_hidden_rdram(), o_hid), "threaded=%s" % threaded
