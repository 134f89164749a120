"""Committed golden fixtures (tests/golden/golden.json, made by
tests/golden/make_golden.py from the CPU oracle).

CPU: the generator still produces the same command words and the oracle still
produces the same RDRAM / hidden RDRAM / TMEM / fragment counts and VI images.
GPU: the CUDA path (through the C ABI) produces the committed digests without
running the oracle."""
import json
import os

import numpy as np
import pytest

from rdp_gb300 import cmdgen

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "golden.json")) as f:
    GOLDEN = json.load(f)

import golden.make_golden as mg  # noqa: E402


def _stream(case):
    p = cmdgen.default_params(case["config"], **case["params"])
    words, rdram, _ = cmdgen.generate_stream(p)
    assert mg.sha(words) == case["words_sha256"], "generator output changed"
    return words, rdram


@pytest.mark.parametrize("name", sorted(GOLDEN["render"]))
def test_oracle_render_golden(name):
    case = GOLDEN["render"][name]
    got = mg.oracle_render(case["config"], case["params"])
    for k in ("words_sha256", "rdram_sha256", "hidden_sha256", "tmem_sha256", "fragments"):
        assert got[k] == case[k], k


@pytest.mark.parametrize("name", sorted(GOLDEN["vi"]))
def test_oracle_vi_golden(name):
    case = GOLDEN["vi"][name]
    assert mg.vi_frames(case["variant"], len(case["frames"]), "oracle") == case["frames"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GOLDEN["render"]))
def test_gpu_render_golden(name):
    from rdp_testutil import run_gpu
    case = GOLDEN["render"][name]
    words, rdram = _stream(case)
    rd, hid, tmem, stats = run_gpu(words, rdram)
    assert mg.sha(rd) == case["rdram_sha256"]
    assert mg.sha(hid) == case["hidden_sha256"]
    assert mg.sha(tmem) == case["tmem_sha256"]
    assert stats["fragments"] == case["fragments"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GOLDEN["vi"]))
def test_gpu_vi_golden(name):
    from rdp_gb300 import CommandProcessor
    case = GOLDEN["vi"][name]
    with CommandProcessor(np.zeros(8 << 20, np.uint8)) as cp:
        assert mg.vi_frames(case["variant"], len(case["frames"]), cp) == case["frames"]


CONFIGS = json.load(open(os.path.join(HERE, "golden", "configs.json")))


def test_configs_golden_generator_and_oracle_still_agree():
    """CPU side of tests/golden/configs.json: the generator still produces the committed command
    words of the benchmark-size configurations, and the oracle still renders the smallest batched
    instance to the committed digests."""
    from oracle import Oracle
    b = CONFIGS["instances"][:64]
    for g in b[:4]:
        words, _, prims = cmdgen.generate_stream(cmdgen.batched_instance_params(g["instance"]))
        assert mg.sha(words) == g["words_sha256"] and prims == g["primitives"]
    small = min(b, key=lambda g: g["primitives"])
    words, rdram, _ = cmdgen.generate_stream(cmdgen.batched_instance_params(small["instance"]))
    o = Oracle(8 << 20)
    o.write_rdram(rdram)
    o.enqueue(words)
    assert mg.sha(o.rdram()) == small["rdram_sha256"] and mg.sha(o.hidden()) == small["hidden_sha256"]
    assert o.fragments() == small["fragments"] and o.reference_passes() == small["reference_passes"]
    o.close()
    words, _, _, offsets = cmdgen.generate_frames(cmdgen.default_params(cmdgen.CONFIG_MIXED))
    assert mg.sha(words) == CONFIGS["mixed16"]["words_sha256"] and len(offsets) == 17
