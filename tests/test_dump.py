"""RDPDUMP2 files: the Python writer and reader round-trip a generated stream; the native
replayer renders a dump exactly like direct enqueueing, with scanout images equal to the
oracle's replay of the same file."""
import numpy as np
import pytest

from rdp_gb300 import cmdgen
from rdp_gb300.dump import DumpWriter, read_dump, split_commands

VI_REGS = {0: (1 << 8) | (1 << 4) | (1 << 16) | (1 << 3) | 2, 1: 0x100000, 2: 320, 6: 525,
           10: (34 << 16) | (34 + 480), 12: 512, 13: 1024, 9: (108 << 16) | (108 + 640)}


def _write(path, words, rdram, frames=1):
    with DumpWriter(path) as d:
        d.flush_dram(rdram)
        d.flush_hidden_dram(np.full(4 << 20, 3, np.uint8))
        for _ in range(frames):
            for r, v in VI_REGS.items():
                d.set_vi_register(r, v)
            d.commands(words)
            d.signal_complete()
            d.end_frame()


def _stream():
    p = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=8, num_prims=400)
    words, rdram, _ = cmdgen.generate_stream(p)
    return words, rdram


def test_round_trip(tmp_path):
    words, rdram = _stream()
    path = tmp_path / "s.rdpdump"
    _write(path, words, rdram, frames=2)
    ev = list(read_dump(path))
    kinds = [k for k, _ in ev]
    assert kinds.count("end_frame") == 2 and kinds[0] == "rdram" and kinds[1] == "hidden"
    assert np.array_equal(ev[0][1], rdram)
    cmds = np.concatenate([w for k, (op, w) in [(k, p) for k, p in ev if k == "command"]])
    assert np.array_equal(cmds, np.concatenate([words, words]))
    assert [op for op, _ in split_commands(words)] == [int(w[0] >> 24) & 63 for _, w in split_commands(words)]


def _oracle_replay(path):
    from oracle import Oracle
    from rdp_gb300 import ScanoutOptions
    o = Oracle(8 << 20)
    opts = ScanoutOptions(blend_previous_frame=1, upscale_deinterlacing=0).as_words()
    frames = []
    for kind, payload in read_dump(path):
        if kind == "rdram":
            o.write_rdram(payload)
        elif kind == "hidden":
            o.write_hidden(payload)
        elif kind == "command":
            o.enqueue(payload[1])
        elif kind == "vi":
            o.set_vi_register(*payload)
        elif kind == "end_frame":
            frames.append(o.scanout(opts))
    return o, frames


@pytest.mark.gpu
def test_native_replay_matches_direct_and_oracle(tmp_path):
    from rdp_gb300 import CommandProcessor
    from rdp_gb300.dump import replay
    from rdp_testutil import run_gpu
    words, rdram = _stream()
    path = tmp_path / "s.rdpdump"
    _write(path, words, rdram, frames=2)
    with CommandProcessor(np.zeros(8 << 20, np.uint8)) as cp:
        frames = replay(cp, path)
        got = cp.begin_read_rdram().copy()
    direct, _, _, _ = run_gpu(np.concatenate([words, words]), rdram)
    assert np.array_equal(got, direct)
    o, oframes = _oracle_replay(path)
    assert len(frames) == len(oframes) == 2
    for a, b in zip(frames, oframes):
        assert a is not None and b is not None and np.array_equal(a, b)
    assert np.array_equal(got, o.rdram())
