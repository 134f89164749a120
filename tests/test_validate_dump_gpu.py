"""The dump validator with the GPU path as the candidate and the CPU oracle as the reference (the
reference project's rdp-validate-dump run): a textured, depth-tested capture compared after every
draw, and a mixed-primitive capture (copy / fill rectangles, TLUT, LOD) after every SyncFull --
TMEM, RDRAM and hidden RDRAM identical at each point; also through the command-line tool."""
import os
import subprocess
import sys

import numpy as np
import pytest

from rdp_gb300 import CommandProcessor, cmdgen
from rdp_gb300.dump import DumpWriter
from rdp_gb300.validate import GpuTarget, validate_dump

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from validate_dump import OracleTarget  # noqa: E402


def _dump(path, frames):
    with DumpWriter(path) as d:
        first = True
        for words, rdram in frames:
            if first:
                d.flush_dram(rdram)
                d.flush_hidden_dram(np.full(4 << 20, 3, np.uint8))
                first = False
            d.commands(words)
            d.commands(np.array([0x29 << 24, 0], np.uint32))
            d.signal_complete()
            d.end_frame()


def test_gpu_matches_oracle_draw_by_draw(tmp_path):
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=51, num_prims=250)
    words, rdram, _ = cmdgen.generate_stream(p)
    path = tmp_path / "textured.rdpdump"
    _dump(path, [(words, rdram)])
    ref = OracleTarget()
    with CommandProcessor(np.zeros(8 << 20, np.uint8)) as cp:
        r = validate_dump(path, ref, GpuTarget(cp))
    ref.close()
    assert r["passed"], r
    assert r["checks"] >= 250


def test_gpu_matches_oracle_sync_by_sync_and_cli(tmp_path):
    frames = []
    for seed in (52, 53):
        p = cmdgen.default_params(cmdgen.CONFIG_MIXED, seed=seed, num_prims=1500, num_frames=1)
        words, rdram, _ = cmdgen.generate_stream(p)
        frames.append((words, rdram))
    path = tmp_path / "mixed.rdpdump"
    _dump(path, frames)
    ref = OracleTarget()
    with CommandProcessor(np.zeros(8 << 20, np.uint8)) as cp:
        r = validate_dump(path, ref, GpuTarget(cp), sync_only=True)
    ref.close()
    assert r["passed"], r
    assert r["frames"] == 2 and r["checks"] >= 2
    out = subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "validate_dump.py"), str(path), "--sync-only",
                          "--begin-frame", "1"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert '"passed": true' in out.stdout
