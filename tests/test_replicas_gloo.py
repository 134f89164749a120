"""bench.py with N > 1 ranks is replicas only: every rank renders its own instances, and the ranks
meet only in the barrier around the timed region and in two reductions -- the maximum of their
timed seconds and the sum of their units.  These run here as two gloo ranks on CPU (127.0.0.1),
with no GPU and no kernel launched; the reference arm's non-zero ranks exit without work."""
import json
import os
import socket
import subprocess
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RANK = r"""
import json, sys
sys.path.insert(0, {root!r})
import bench
dist, rank, world, local = bench._dist()
bench._barrier(dist)
out = dict(rank=rank, world=world, local=local,
           max=bench._max_over_ranks(dist, 1.5 + rank),
           sum=bench._sum_over_ranks(dist, 10 * (rank + 1)))
bench._barrier(dist)
dist.destroy_process_group()
print(json.dumps(out))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_reduce_time_and_units():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(r),
                   LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        so, se = p.communicate(timeout=240)
        assert p.returncode == 0, se[-2000:]
        outs.append(json.loads(so.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["world"] == 2 and o["local"] == o["rank"]
        assert o["max"] == 2.5          # the slower rank's seconds
        assert o["sum"] == 30.0         # units of both ranks


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    args = types.SimpleNamespace(instances=64, steps=1, warmup=0, workload="batched")
    assert bench.run_reference_batched(args) is None
    assert capsys.readouterr().out == ""
