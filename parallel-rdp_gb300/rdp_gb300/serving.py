"""Request traces for the serving loop (rdp_serve_run): instances submit frames as a Poisson
process; latency percentiles of a run."""
import numpy as np


def poisson_trace(num_instances, rate_fps, duration_s, frames, seed=0):
    """Arrivals of a Poisson process at `rate_fps` (aggregate) over `duration_s`; each request
    picks an instance uniformly and uses frames[instance] (a words array or a list of them,
    taken in turn).  Returns [(instance, words, arrival_s)] sorted by arrival."""
    rng = np.random.default_rng(seed)
    t, out, turn = 0.0, [], [0] * num_instances
    while True:
        t += rng.exponential(1.0 / rate_fps)
        if t >= duration_s:
            break
        i = int(rng.integers(0, num_instances))
        f = frames[i]
        if isinstance(f, (list, tuple)):
            w = f[turn[i] % len(f)]
            turn[i] += 1
        else:
            w = f
        out.append((i, w, t))
    return out


def latency_summary(latency_s):
    lat = np.asarray(latency_s) * 1e3
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "requests": int(lat.size)}
