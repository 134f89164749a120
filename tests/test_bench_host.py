"""Host side of bench.py (no GPU): the clock sampler that records SM clocks and throttle reasons
during the timed region, driven by a stand-in `nvidia-smi` that prints CSV samples."""
import os
import stat
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Prints one sample every 20 ms, like `nvidia-smi --query-gpu=... --format=csv,noheader,nounits -lms N`:
# index, clocks.sm, clocks.max.sm, power.draw, reasons.active, hw_slowdown, hw_thermal_slowdown,
# sw_thermal_slowdown, sw_power_cap.
_FAKE = """#!{python}
import sys, time
rows = ["0, 2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1965, 2070, 1390.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1100.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"]
k = 0
while True:
    print(rows[k % len(rows)], flush=True)
    k += 1
    time.sleep(0.02)
"""


def test_clock_sampler_parses_samples_and_reasons(tmp_path, monkeypatch):
    fake = tmp_path / "nvidia-smi"
    fake.write_text(_FAKE.format(python=sys.executable))
    fake.chmod(fake.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ.get("PATH", ""))
    sys.path.insert(0, ROOT)
    import bench
    c = bench.ClockSampler(0)
    c.start()
    assert os.path.getsize(c.path) > 0  # sampling is live when start() returns
    time.sleep(0.2)
    out = c.stop()
    assert out["samples"] >= 3
    assert out["sm_max_mhz"] == 2070.0
    assert out["sm_mhz"] in (1965.0, 2070.0)
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))
    sys.path.insert(0, ROOT)
    import bench
    c = bench.ClockSampler(0)
    c.start()
    assert c.stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_reference_arm_prints_its_contract_line():
    # The reference arm (the CPU restatement of the reference's algorithm on the host cores),
    # on two instances: one JSON line with the base metric, the reference marker, the CPU
    # baseline it measured and an end-to-end entry without device copies.
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--instances", "2",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "passes/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "passes/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_int_alu_roofline_reads_the_op_table_and_uses_the_issue_peak():
    """roofline.int_alu: ops per step from oracle/op_table.json over the step time, against SMs x
    128 lanes x the sampled clock; the shading kernel's figure uses the shading stages' ops."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    table = json.load(open(os.path.join(ROOT, "oracle", "op_table.json")))["workloads"]["batched64"]
    r = bench._int_alu_roofline("batched64", 20.0, 10.0, 152, 2000.0)
    peak = 152 * 128 * 2000e6 / 1e12
    assert abs(r["peak"] - peak) < 1e-9
    assert abs(r["achieved"] - table["ops_total"] / 0.020 / 1e12) < 1e-6
    assert abs(r["k_shade"]["achieved"] - table["ops_shading_stages"] / 0.010 / 1e12) < 1e-6
    assert abs(r["frac"] - r["achieved"] / peak) < 1e-12
    assert 0 < table["ops_shading_stages"] < table["ops_total"]
    assert bench._int_alu_roofline("no such workload", 20.0, 10.0, 152, 2000.0) is None


def test_step_hbm_roofline_counts_commands_tiles_and_texture_sources():
    sys.path.insert(0, ROOT)
    import bench
    r = bench._step_hbm_roofline(1000, 10, 64 * 2 * 9, 3, 1.0, 8000.0, "fallback")
    assert r["algorithmic_bytes_per_step"] == 1000 + 10 * 64 * 2 * 9 + 3 * 4096
    assert abs(r["achieved"] - r["algorithmic_bytes_per_step"] / 1e-3 / 1e9) < 1e-9
    assert abs(r["frac"] - r["achieved"] / 8000.0) < 1e-12


def test_serving_parity_check_renders_each_sampled_instance_as_often_as_it_was_served():
    """The serving bench's 1 % output sample: digests and render counts recorded on the GPU side are
    checked by rendering the same instance's frame that many times through the oracle."""
    import hashlib
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    from oracle import Oracle
    from rdp_gb300 import cmdgen
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()  # noqa: E731
    words, rdram, _ = cmdgen.generate_stream(cmdgen.batched_instance_params(5))
    o = Oracle(8 << 20)
    o.write_rdram(rdram)
    for _ in range(3):
        o.enqueue(words)
    good = {"renders": 3, "rdram_sha256": sha(o.rdram()), "hidden_sha256": sha(o.hidden())}
    o.close()
    r = bench._check_serving_parity({"requests_sampled": 2, "of_requests": 200, "instances": {5: good}}, threads=2)
    assert r["passed"] and r["instances_checked"] == 1 and r["renders_checked"] == 3
    # Instance 5's frame is not idempotent: one render gives another image than three.
    wrong = dict(good, renders=1)
    r = bench._check_serving_parity({"requests_sampled": 2, "of_requests": 200, "instances": {5: wrong}}, threads=2)
    assert not r["passed"] and r["mismatches"] == [5]
