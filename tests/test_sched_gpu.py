"""Learned tile scheduling (sched.cu): the GPU training kernels agree with the CPU restatement,
the learned order never changes output, online training lowers the loss, and on a workload
whose heaviest tiles come last in tile order the trained order shortens the blend kernel."""
import numpy as np
import pytest

from rdp_gb300 import Batch, cmdgen, mlp_forward, mlp_gradients
from rdp_testutil import run_gpu
import mlp_oracle as mo

pytestmark = pytest.mark.gpu
F = cmdgen.FLAGS


def test_gradients_match_cpu_oracle():
    rng = np.random.default_rng(0)
    p = mo.fp16_round(mo.init_params(5)).astype(np.float32)
    x = rng.uniform(0, 1, (300, mo.IN)).astype(np.float32)
    y = rng.uniform(0, 2, 300).astype(np.float32)
    g, loss = mlp_gradients(p, x, y)
    gc, lc = mo.gradients(p.astype(np.float64), x.astype(np.float64), y.astype(np.float64))
    # FP32 accumulation on the GPU against float64: tolerance relative to the largest gradient.
    assert np.abs(g - gc).max() <= 1e-5 * max(1.0, np.abs(gc).max())
    assert abs(loss - lc) <= 1e-5 * max(1.0, lc)


def test_forward_matches_cpu_oracle():
    rng = np.random.default_rng(1)
    p = mo.fp16_round(mo.init_params(6)).astype(np.float32)
    x = rng.uniform(0, 1, (500, mo.IN)).astype(np.float32)
    out = mlp_forward(p, x)
    ref, _ = mo.forward(p.astype(np.float64), x.astype(np.float64))
    assert np.abs(out - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def _streams(n, seed_base):
    out = []
    for i in range(n):
        p = cmdgen.batched_instance_params(i, min_prims=300, max_prims=1500, seed_base=seed_base)
        w, rd, _ = cmdgen.generate_stream(p)
        out.append((w, rd))
    return out


def test_learned_order_and_training_are_bit_exact():
    streams = _streams(5, 60)
    with Batch(record_tile_cycles=True) as b:
        b.set_schedule(learned_order=True, train=True, learning_rate=3e-3)
        insts = [b.add_instance(rd.copy()) for _, rd in streams]
        for cp, (w, _) in zip(insts, streams):
            cp.enqueue_command(w)
        b.idle()
        for cp, (w, rd) in zip(insts, streams):
            s_rd, s_hid, s_tmem, _ = run_gpu(w, rd)
            assert np.array_equal(cp.begin_read_rdram(), s_rd)
            assert np.array_equal(cp.begin_read_hidden_rdram(), s_hid)
            assert np.array_equal(cp.get_tmem(), s_tmem)


def _hotspot_batch():
    # A busy sync point (24 instances of the batched-instances mix) followed, last in tile
    # order, by a textured, depth-tested frame whose 1,000 triangles all sit in the top-left
    # 16x16 pixels: a few tiles with ~1,000 pairs each, which in tile order start last.
    streams = []
    for i in range(24):
        p = cmdgen.batched_instance_params(i, min_prims=4000, max_prims=20000, seed_base=400)
        w, rd, _ = cmdgen.generate_stream(p)
        streams.append((w, rd))
    base = cmdgen.default_params(cmdgen.CONFIG_TEXTURED)
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=300, num_prims=1000, flags=base.flags | F["HOTSPOT"])
    w, rd, _ = cmdgen.generate_stream(p)
    streams.append((w, rd))
    return streams


def test_online_training_lowers_loss_and_trained_order_shortens_blend():
    streams = _hotspot_batch()
    with Batch(record_tile_cycles=True) as b:
        insts = [b.add_instance(rd.copy()) for _, rd in streams]

        def frame():
            for cp, (w, _) in zip(insts, streams):
                cp.enqueue_command(w)
            b.idle()

        frame()
        b.set_schedule(learned_order=True, train=True, learning_rate=3e-3)
        losses = []
        for _ in range(12):
            frame()
            losses.append(b.get_model()[1])
        assert np.mean(losses[-5:]) < 0.5 * losses[0], losses

        def blend_ms(learned):
            b.set_schedule(learned_order=learned, train=False)
            g = b.capture([w for w, _ in streams])
            g.replay(2)
            t = []
            for _ in range(7):
                g.replay(1)
                t.append(g.last_blend_ms())
            g.close()
            return float(np.median(t))

        static, learned = blend_ms(False), blend_ms(True)
        static2, learned2 = blend_ms(False), blend_ms(True)
        print("blend ms static %.3f %.3f learned %.3f %.3f" % (static, static2, learned, learned2))
        # Measured on a GB300: ~3.5 ms in tile order, ~2.9 ms longest-predicted-first.
        assert min(learned, learned2) < 0.95 * min(static, static2)
