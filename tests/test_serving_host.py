"""Host side of the serving configuration (no GPU): the Poisson request traces the serving loop
runs and the latency summary it reports."""
import numpy as np

from rdp_gb300.serving import latency_summary, poisson_trace


def test_poisson_trace_rate_order_and_instances():
    frames = [np.full(4, i, dtype=np.uint32) for i in range(16)]
    trace = poisson_trace(16, rate_fps=20000.0, duration_s=0.5, frames=frames, seed=3)
    n = len(trace)
    # 10,000 expected arrivals; a Poisson count stays within 5 sigma (500).
    assert abs(n - 10000) < 500, n
    t = np.array([r[2] for r in trace])
    assert np.all(np.diff(t) >= 0) and t[0] >= 0 and t[-1] < 0.5
    inst = np.array([r[0] for r in trace])
    counts = np.bincount(inst, minlength=16)
    assert counts.min() > 0.8 * n / 16 and counts.max() < 1.2 * n / 16, counts
    for i, w, _ in trace:
        assert w[0] == i  # each request carries its own instance's frame
    # Same seed, same trace.
    again = poisson_trace(16, rate_fps=20000.0, duration_s=0.5, frames=frames, seed=3)
    assert [(r[0], r[2]) for r in again] == [(r[0], r[2]) for r in trace]


def test_poisson_trace_takes_an_instances_frames_in_turn():
    frames = [[np.array([10 * i + k], dtype=np.uint32) for k in range(3)] for i in range(4)]
    trace = poisson_trace(4, rate_fps=5000.0, duration_s=0.2, frames=frames, seed=1)
    seen = {i: [] for i in range(4)}
    for i, w, _ in trace:
        seen[i].append(int(w[0]))
    for i, ws in seen.items():
        assert ws == [10 * i + (k % 3) for k in range(len(ws))], (i, ws[:6])


def test_latency_summary_in_milliseconds():
    lat = np.arange(1, 101) * 1e-3  # 1 .. 100 ms
    s = latency_summary(lat)
    assert s["requests"] == 100
    assert abs(s["p50_ms"] - 50.5) < 1e-9 and abs(s["p99_ms"] - 99.01) < 1e-9
    assert abs(s["mean_ms"] - 50.5) < 1e-9 and abs(s["max_ms"] - 100.0) < 1e-9
