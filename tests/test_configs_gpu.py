"""Parity at the benchmark's own sizes, against the oracle's committed answers
(tests/golden/configs.json, made by tests/golden/make_golden_configs.py).

* The batched-instances workload exactly as bench.py runs it: 64 instances (seeds 0-63, up to
  50,000 primitives, 320x240 / 640x240 / 640x480), one batch, every instance's frame parsed on
  the batch's host threads and submitted together -- the launches where the multi-CTA scans, the
  per-SM queues with stealing and primitive-major shading order engage -- then again with the
  learned tile order training online, then as a captured CUDA graph replayed twice.  After each,
  every instance's RDRAM and hidden RDRAM must equal the oracle's after as many renders of the
  frame on the same memory, and the fragment and reference-pass counts of a frame must match.
* The mixed 640x480 RGBA8888 sequence as configured (16 frames of 50,000 primitives): after every
  frame the RDRAM, hidden RDRAM and the VI scanout (AA, divot, dither filter, interlaced) must
  equal the oracle's.

All comparisons are exact (integer data)."""
import hashlib
import json
import os

import numpy as np
import pytest

from rdp_gb300 import Batch, CommandProcessor, cmdgen

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "configs.json")))


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def _check_instances(insts, golden, what, renders=1):
    """Every instance's RDRAM and hidden RDRAM against the oracle's after `renders` renders of the
    instance's frame on the same memory."""
    bad = []
    for cp, g in zip(insts, golden):
        want = g if renders == 1 else g["renders"][str(renders)]
        if _sha(cp.begin_read_rdram()) != want["rdram_sha256"] or _sha(cp.begin_read_hidden_rdram()) != want["hidden_sha256"]:
            bad.append(g["instance"])
    assert not bad, "%s: instances %s differ from the oracle" % (what, bad)


def test_batched_64_instance_sync_point_matches_oracle():
    golden = GOLDEN["instances"][:64]
    streams = []
    for g in golden:
        words, rdram, prims = cmdgen.generate_stream(cmdgen.batched_instance_params(g["instance"]))
        assert _sha(words) == g["words_sha256"], "generator output changed"
        streams.append((words, rdram))
    assert max(g["primitives"] for g in golden) > 40000
    with Batch() as b:
        insts = [b.add_instance(np.array(rd, copy=True)) for _, rd in streams]
        words = [w for w, _ in streams]

        def step():
            values = b.enqueue_many(insts, words)
            b.submit()
            for cp, v in zip(insts, values):
                cp.wait_for_timeline(v)

        s0 = [cp.stats() for cp in insts]
        step()
        s1 = [cp.stats() for cp in insts]
        for i, (a, c, g) in enumerate(zip(s0, s1, golden)):
            assert c["fragments"] - a["fragments"] == g["fragments"], "instance %d fragments" % i
            assert c["reference_passes"] - a["reference_passes"] == g["reference_passes"], "instance %d passes" % i
        _check_instances(insts, golden, "first sync point")
        assert b.stats()["rounds"] >= 3

        # The learned tile order, training online (as the benchmark's warm-up does).
        b.idle()
        b.set_schedule(learned_order=True, train=True, learning_rate=3e-3)
        for _ in range(2):
            step()
            b.idle()
        _check_instances(insts, golden, "learned order while training", renders=3)

        # The timed form: the sync point captured as one CUDA graph (recording renders nothing),
        # replayed twice.
        b.set_schedule(learned_order=True, train=False)
        graph = b.capture(words)
        graph.replay(2)
        graph.close()
        _check_instances(insts, golden, "graph replay", renders=5)


def test_mixed_16_frames_of_50000_primitives_with_vi_match_oracle():
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden_configs import mixed_scanout_options, mixed_vi_regs
    golden = GOLDEN["mixed16"]
    p = cmdgen.default_params(cmdgen.CONFIG_MIXED)
    assert p.num_frames == 16 and p.num_prims == 50000 and p.width == 640 and p.height == 480
    words, rdram, prims, offsets = cmdgen.generate_frames(p)
    assert _sha(words) == golden["words_sha256"]
    opts = mixed_scanout_options()
    with CommandProcessor(np.array(rdram, copy=True)) as cp:
        for f, g in enumerate(golden["frames"]):
            cp.enqueue_command(words[offsets[f]:offsets[f + 1]])
            for r, v in mixed_vi_regs(f).items():
                cp.set_vi_register(r, v)
            img = cp.scanout_sync(opts)
            vi = None if img is None else [int(img.shape[1]), int(img.shape[0]), _sha(img)]
            assert vi == g["vi"], "frame %d VI scanout" % f
            assert _sha(cp.begin_read_rdram()) == g["rdram_sha256"], "frame %d RDRAM" % f
            assert _sha(cp.begin_read_hidden_rdram()) == g["hidden_sha256"], "frame %d hidden RDRAM" % f
            assert cp.stats()["fragments"] == g["fragments"], "frame %d fragments" % f
        assert cp.stats()["reference_passes"] == golden["reference_passes"]
