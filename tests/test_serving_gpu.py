"""Serving loop (rdp_serve_run): continuous batching of Poisson-arriving frame requests from many
instances; every instance ends with exactly what rendering its own requests alone produces, and
a sample of instances matches the CPU oracle."""
import numpy as np
import pytest

from rdp_gb300 import Batch, cmdgen
from rdp_gb300.serving import latency_summary, poisson_trace
from rdp_testutil import run_oracle

pytestmark = pytest.mark.gpu


def _frames(n, per_instance):
    frames, inits = [], []
    for i in range(n):
        seq = []
        for k in range(per_instance):
            p = cmdgen.batched_instance_params(i, min_prims=200, max_prims=2500, seed_base=1000 + 97 * k)
            w, rd, _ = cmdgen.generate_stream(p)
            seq.append(w)
            if k == 0:
                inits.append(rd)
        frames.append(seq)
    return frames, inits


def test_serving_same_alone_and_in_the_mix():
    n = 12
    frames, inits = _frames(n, 3)
    trace = poisson_trace(n, rate_fps=4000.0, duration_s=0.02, frames=frames, seed=5)
    assert len(trace) > 40
    with Batch() as b:
        insts = [b.add_instance(rd.copy()) for rd in inits]
        res, stats = b.serve(insts, trace, hbm_budget_bytes=2 << 30)
        assert stats["max_in_flight"] > 1 and stats["submits"] > 1  # frames overlapped on the device
        assert np.all(res["latency_s"] > 0)
        summary = latency_summary(res["latency_s"])
        assert summary["requests"] == len(trace)
        mixed = [cp.begin_read_rdram().copy() for cp in insts]
        mixed_hidden = [cp.begin_read_hidden_rdram() for cp in insts]
    # Alone: each instance's requests, in arrival order, through its own processor.
    for i in range(n):
        words = [w for (k, w, _) in trace if k == i]
        if not words:
            continue
        with Batch() as b:
            cp = b.add_instance(inits[i].copy())
            for w in words:
                cp.enqueue_command(w)
                cp.wait_for_timeline(cp.signal_timeline())
            assert np.array_equal(cp.begin_read_rdram(), mixed[i]), i
            assert np.array_equal(cp.begin_read_hidden_rdram(), mixed_hidden[i]), i
        if i < 2:  # a sample against the CPU oracle
            rd, hid, _, _ = run_oracle(np.concatenate(words), inits[i])
            assert np.array_equal(rd, mixed[i]) and np.array_equal(hid, mixed_hidden[i])


def test_serving_admission_respects_budget():
    n = 6
    frames, inits = _frames(n, 1)
    trace = poisson_trace(n, rate_fps=20000.0, duration_s=0.003, frames=[f[0] for f in frames], seed=9)
    with Batch() as b:
        insts = [b.add_instance(rd.copy()) for rd in inits]
        res, stats = b.serve(insts, trace, hbm_budget_bytes=1, max_in_flight=2)
        assert stats["max_in_flight"] <= 2
        assert np.all(res["done_s"] >= res["admit_s"])
