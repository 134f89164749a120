"""Batched instances (rdp_batch_*): every instance of a batch renders exactly what a
stand-alone processor renders from the same command stream, bit for bit, while the
batch launches one kernel chain per round for all instances.  Instances follow the
batched-instances workload (mixed RGBA8888 primitive mix, resolutions from
320x240 / 640x240 / 640x480, log-uniform primitive counts), at reduced sizes."""
import numpy as np
import pytest

from rdp_gb300 import Batch, cmdgen
from rdp_testutil import run_gpu, run_oracle

pytestmark = pytest.mark.gpu


def _instance_streams(n, max_prims, seed_base=0):
    out = []
    for i in range(n):
        p = cmdgen.batched_instance_params(i, min_prims=100, max_prims=max_prims, seed_base=seed_base)
        words, rdram, _ = cmdgen.generate_stream(p)
        out.append((words, rdram))
    return out


def _read(cp):
    return cp.begin_read_rdram().copy(), cp.begin_read_hidden_rdram(), cp.get_tmem()


def test_batch_matches_standalone_and_oracle():
    streams = _instance_streams(6, 1500)
    with Batch() as b:
        insts = [b.add_instance(np.array(rd, copy=True)) for _, rd in streams]
        for cp, (w, _) in zip(insts, streams):
            cp.enqueue_command(w)
        values = [cp.signal_timeline() for cp in insts]
        b.submit()
        for cp, v in zip(insts, values):
            cp.wait_for_timeline(v)
        st = b.stats()
        assert st["instances"] == 6 and st["rounds"] >= 1
        # Rounds hold at most one pass per instance, so rounds < passes when >1 instance has work.
        assert st["rounds"] < st["passes"]
        for i, (cp, (w, rd)) in enumerate(zip(insts, streams)):
            g_rd, g_hid, g_tmem = _read(cp)
            s_rd, s_hid, s_tmem, s_stats = run_gpu(w, rd)
            assert np.array_equal(g_rd, s_rd), "instance %d rdram" % i
            assert np.array_equal(g_hid, s_hid), "instance %d hidden" % i
            assert np.array_equal(g_tmem, s_tmem), "instance %d tmem" % i
            assert cp.stats()["fragments"] == s_stats["fragments"]
            if i < 2:
                o_rd, o_hid, o_tmem, frags = run_oracle(w, rd)
                assert np.array_equal(g_rd, o_rd) and np.array_equal(g_hid, o_hid)
                assert np.array_equal(g_tmem.view(np.uint8), o_tmem.view(np.uint8))
                assert cp.stats()["fragments"] == frags


def test_batch_wait_submits_and_frames_stay_ordered():
    # Two frames per instance, the second enqueued after waiting on the first; waiting on an
    # unsubmitted timeline value submits the batch.
    a = _instance_streams(3, 600, seed_base=10)
    c = _instance_streams(3, 600, seed_base=20)
    with Batch() as b:
        insts = [b.add_instance(np.array(rd, copy=True)) for _, rd in a]
        for cp, (w, _) in zip(insts, a):
            cp.enqueue_command(w)
        v = [cp.signal_timeline() for cp in insts]
        insts[1].wait_for_timeline(v[1])  # submits every instance's deferred passes
        for cp, (w, _) in zip(insts, c):
            cp.enqueue_command(w)
        for cp in insts:
            cp.idle()
        for i, cp in enumerate(insts):
            words = np.concatenate([a[i][0], c[i][0]])
            s_rd, s_hid, s_tmem, _ = run_gpu(words, a[i][1])
            g_rd, g_hid, g_tmem = _read(cp)
            assert np.array_equal(g_rd, s_rd) and np.array_equal(g_hid, s_hid) and np.array_equal(g_tmem, s_tmem)


def test_batch_graph_replays_all_instances():
    streams = _instance_streams(4, 800, seed_base=30)
    with Batch() as b:
        insts = [b.add_instance(np.array(rd, copy=True)) for _, rd in streams]
        g = b.capture([w for w, _ in streams])
        assert g.kernels > 0
        ms = g.replay(3)
        assert ms > 0.0
        g.close()
        st = b.stats()
        assert st["passes"] >= 4


def test_batch_instance_destroy_keeps_others():
    streams = _instance_streams(3, 500, seed_base=40)
    with Batch() as b:
        insts = [b.add_instance(np.array(rd, copy=True)) for _, rd in streams]
        for cp, (w, _) in zip(insts, streams):
            cp.enqueue_command(w)
        insts[0].close()  # finishes its own work, leaves the batch
        for cp in insts[1:]:
            cp.idle()
        for cp, (w, rd) in zip(insts[1:], streams[1:]):
            s_rd, _, _, _ = run_gpu(w, rd)
            assert np.array_equal(cp.begin_read_rdram(), s_rd)


def test_enqueue_many_matches_sequential():
    streams = _instance_streams(8, 1200, seed_base=70)
    with Batch() as b:
        insts = [b.add_instance(np.array(rd, copy=True)) for _, rd in streams]
        values = b.enqueue_many(insts, [w for w, _ in streams])
        b.submit()
        for cp, v in zip(insts, values):
            cp.wait_for_timeline(v)
        for cp, (w, rd) in zip(insts, streams):
            s_rd, s_hid, _, stats = run_gpu(w, rd)
            assert np.array_equal(cp.begin_read_rdram(), s_rd)
            assert np.array_equal(cp.begin_read_hidden_rdram(), s_hid)
            assert cp.stats()["reference_passes"] == stats["reference_passes"]
