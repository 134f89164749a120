"""Seeded command-stream generator: determinism and stream structure."""
import numpy as np

from rdp_gb300 import cmdgen

LEN = {0x08: 8, 0x09: 12, 0x0a: 24, 0x0b: 28, 0x0c: 24, 0x0d: 28, 0x0e: 40, 0x0f: 44, 0x24: 4, 0x25: 4}


def _walk(words):
    i, ops = 0, []
    while i < len(words):
        op = (int(words[i]) >> 24) & 63
        ops.append(op)
        i += LEN.get(op, 2)
    assert i == len(words)
    return ops


def test_same_seed_same_words():
    a = cmdgen.generate_stream(cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=5, num_prims=100))
    b = cmdgen.generate_stream(cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=5, num_prims=100))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_plain_config_structure():
    words, rdram, prims = cmdgen.generate_stream(cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=0))
    ops = _walk(words)
    assert ops.count(0x0c) == 2000          # Gouraud triangles
    assert ops.count(0x36) == 1             # FillRect clear
    assert ops[-1] == 0x29                  # SyncFull ends the frame
    assert prims == 2001


def test_mixed_config_contains_each_kind():
    words, _, _ = cmdgen.generate_stream(cmdgen.default_params(cmdgen.CONFIG_MIXED, seed=1, num_prims=2000,
                                                               num_frames=1))
    ops = set(_walk(words))
    for op in (0x0e, 0x0f, 0x24, 0x36, 0x30, 0x33, 0x34):
        assert op in ops, hex(op)
