"""The dump validator (rdp_gb300/validate.py, the reference's rdp_validate_dump.cpp) on the CPU: two
oracles agree draw by draw; an oracle given one planted wrong command is caught at that draw, with
the differing memory, address and framebuffer coordinate reported."""
import os
import sys

import numpy as np

from rdp_gb300 import cmdgen
from rdp_gb300.dump import DumpWriter, split_commands
from rdp_gb300.validate import validate_dump

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
from validate_dump import OracleTarget  # noqa: E402


def _dump(path, words, rdram):
    with DumpWriter(path) as d:
        d.flush_dram(rdram)
        d.flush_hidden_dram(np.full(4 << 20, 3, np.uint8))
        d.commands(words)
        d.commands(np.array([0x29 << 24, 0], np.uint32))
        d.signal_complete()
        d.end_frame()


class PlantedMistake(OracleTarget):
    """An oracle whose shade triangle number `k` (a draw) gets a different first vertex colour."""

    def __init__(self, k):
        super().__init__()
        self.k, self.seen = k, 0

    def enqueue(self, words):
        w = np.array(words, np.uint32)
        if ((int(w[0]) >> 24) & 63) == 0x0c:
            if self.seen == self.k:
                w[8] ^= 0x00ff0000  # shade coefficients: the red start value
            self.seen += 1
        super().enqueue(w)


def test_validator_passes_identical_renderers_and_catches_a_planted_mistake(tmp_path):
    p = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=9, num_prims=60)
    words, rdram, _ = cmdgen.generate_stream(p)
    path = tmp_path / "v.rdpdump"
    _dump(path, words, rdram)
    draws = sum(1 for op, _ in split_commands(words) if op in (0x08, 0x09, 0x0a, 0x0b, 0x0c, 0x0d, 0x0e, 0x0f, 0x24,
                                                                  0x25, 0x36))
    a, b = OracleTarget(), OracleTarget()
    r = validate_dump(path, a, b)
    assert r["passed"] and r["checks"] == draws and r["frames"] == 1
    syncs = sum(1 for op, _ in split_commands(words) if op == 0x29) + 1  # the stream's own, and the dump's
    r = validate_dump(path, OracleTarget(), OracleTarget(), sync_only=True)
    assert r["passed"] and r["checks"] == syncs
    bad = PlantedMistake(20)
    r = validate_dump(path, OracleTarget(), bad)
    assert not r["passed"]
    f = r["failure"]
    assert f["memory"] in ("RDRAM", "hidden RDRAM") and f["frame"] == 0
    # Caught at the draw of the planted triangle (the clear is draw 1, triangles follow).
    assert f["draw"] == bad_draw_number(words, 20)
    assert f["coordinate"]["image"] == "color" and 0 <= f["coordinate"]["x"] < 320 and 0 <= f["coordinate"]["y"] < 240


def bad_draw_number(words, k):
    n = seen = 0
    for op, _ in split_commands(words):
        if op in (0x08, 0x09, 0x0a, 0x0b, 0x0c, 0x0d, 0x0e, 0x0f, 0x24, 0x25, 0x36):
            n += 1
        if op == 0x0c:
            if seen == k:
                return n
            seen += 1
    raise AssertionError("no such triangle")
