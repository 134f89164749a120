"""Stand-alone sync-point captures (rdp_cp_capture_begin / _end, rdp_graph_replay) against the CPU
oracle.  A capture records its launches first and builds the CUDA graph at the end, so a buffer
the executor grows while recording must stay allocated for the launches recorded before it: here
the first pass fills (a one-group bitmask per tile) and a later one draws 3,000 primitives on a
640x480 image (96 bitmask words per tile), so the bitmask buffer grows in the middle of the
recording.  Each replay renders the stream again against device RDRAM; the oracle enqueues it again."""
import numpy as np
import pytest

from rdp_gb300 import CommandProcessor, cmdgen
from rdp_testutil import diff_report

pytestmark = pytest.mark.gpu

RDRAM = 8 << 20


def _fill_pass():
    # 320x240 RGBA5551 image at 4 MiB (clear of the generator's images and textures), one fill.
    return np.array([(0x3f << 24) | (0 << 21) | (2 << 19) | 319, 0x400000,
                     (0x2d << 24), ((320 << 2) << 12) | (240 << 2),
                     (0x2f << 24) | (3 << 20), 0,
                     0x37 << 24, 0x12345679,
                     (0x36 << 24) | ((319 << 2) << 12) | (239 << 2), 0,
                     0x29 << 24, 0], dtype=np.uint32)


def test_capture_keeps_buffers_grown_while_recording():
    from oracle import Oracle
    p = cmdgen.default_params(cmdgen.CONFIG_MIXED, seed=6, num_prims=3000, num_frames=1)
    geo, rdram, _ = cmdgen.generate_stream(p)
    words = np.concatenate([_fill_pass(), geo])
    o = Oracle(RDRAM)
    o.write_rdram(rdram)
    rd = np.array(rdram, dtype=np.uint8, copy=True)
    with CommandProcessor(rd, rdram_size=RDRAM) as cp:
        g = cp.capture(words)
        try:
            for replay in range(2):
                g.replay(1)
                assert o.enqueue(words) == len(words)
                errs = [diff_report("rdram", cp.begin_read_rdram().copy(), o.rdram()),
                        diff_report("hidden", cp.begin_read_hidden_rdram().copy(), o.hidden())]
                errs = [e for e in errs if e]
                assert not errs, "replay %d: %s" % (replay, "; ".join(errs))
        finally:
            g.close()
