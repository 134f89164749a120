"""Kernel specialisations: every compiled variant of the shading kernel -- the general shader and
the render-state-specialised shader (separate code for fill, copy, untextured, one-texel,
one-texel-through-TLUT, two-texel and LOD primitives), each at four register budgets -- produces
the same RDRAM / hidden RDRAM / TMEM bytes, and the autotuner settles on one of them."""
import numpy as np
import pytest

from rdp_gb300 import (SHADE_ORDERS, SHADE_VARIANTS, Batch, cmdgen, get_shade_order, get_shade_variant,
                       set_shade_order, set_shade_variant)
from rdp_testutil import assert_parity, run_gpu

pytestmark = pytest.mark.gpu
F = cmdgen.FLAGS


@pytest.fixture
def restore_tuning():
    yield
    set_shade_variant(-1)


def test_all_variants_bit_exact(restore_tuning):
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=3, num_prims=1200)
    words, rdram, _ = cmdgen.generate_stream(p)
    q = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=4, num_prims=800, fb_format=cmdgen.FB_RGBA8888,
                              flags=F["FUZZ"] | F["CLEAR"])
    fwords, frdram, _ = cmdgen.generate_stream(q)
    # Copy-mode rectangles, fill rectangles, CI8 + TLUT and LOD triangles (the mixed primitive mix),
    # and untextured Gouraud triangles: every render-state variant of the specialised shader runs.
    m = cmdgen.default_params(cmdgen.CONFIG_MIXED, seed=6, num_prims=3000, num_frames=1)
    mwords, mrdram, _ = cmdgen.generate_stream(m)
    g = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=7, num_prims=500)
    gwords, grdram, _ = cmdgen.generate_stream(g)
    results = []
    for v in range(SHADE_VARIANTS):
        set_shade_variant(v)
        assert get_shade_variant() == v
        if v in (0, SHADE_VARIANTS - 1):  # the general and a specialised variant against the oracle
            assert_parity(words, rdram)
            assert_parity(mwords, mrdram)
        results.append((run_gpu(words, rdram)[:3], run_gpu(fwords, frdram)[:3], run_gpu(mwords, mrdram)[:3],
                        run_gpu(gwords, grdram)[:3]))
    for r in results[1:]:
        for a, b in zip(r, results[0]):
            for x, y in zip(a, b):
                assert np.array_equal(x, y)


def test_autotuner_picks_a_variant(restore_tuning):
    set_shade_variant(-1)
    streams = []
    for i in range(8):
        p = cmdgen.batched_instance_params(i, min_prims=2000, max_prims=6000, seed_base=50)
        w, rd, _ = cmdgen.generate_stream(p)
        streams.append((w, rd))
    with Batch() as b:
        insts = [b.add_instance(rd.copy()) for _, rd in streams]
        for _ in range(12):
            for cp, (w, _) in zip(insts, streams):
                cp.enqueue_command(w)
            b.idle()
            if get_shade_variant() >= 0:
                break
    assert 0 <= get_shade_variant() < SHADE_VARIANTS


@pytest.fixture
def restore_order():
    before = get_shade_order()
    yield
    set_shade_order(before)


def _order_run(words, rdram, streams):
    single = run_gpu(words, rdram)[:3]
    with Batch() as b:
        insts = [b.add_instance(rd.copy()) for _, rd in streams]
        for cp, (w, _) in zip(insts, streams):
            cp.enqueue_command(w)
        b.idle()
        batched = [cp.begin_read_rdram().copy() for cp in insts]
        batched += [cp.begin_read_hidden_rdram().copy() for cp in insts]
    return single, batched


@pytest.mark.parametrize("variant", [1, 5], ids=["general", "specialised"])
def test_shade_orders_bit_exact(restore_order, restore_tuning, monkeypatch, variant):
    """Tile order with a fixed stride, per-SM work queues and primitive-major order shade the
    same pairs: identical bytes, on a single stream and on a batch of instances, with the general
    and the render-state-specialised shading kernels.  The size thresholds are
    set to 0 so that every launch, down to the smallest, takes the queues (and their stealing
    sweep) and the primitive-major order; one more run keeps the default thresholds.  The
    single stream's big pass (10,000 primitives, 1,200 tiles) takes the one-CTA scans, the
    batch's launches the multi-CTA ones."""
    set_shade_variant(variant)
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=5, num_prims=10000)
    words, rdram, _ = cmdgen.generate_stream(p)
    streams = []
    for i in range(8):
        q = cmdgen.batched_instance_params(i, min_prims=3000, max_prims=6000, seed_base=70)
        w, rd, _ = cmdgen.generate_stream(q)
        streams.append((w, rd))
    set_shade_order(SHADE_ORDERS["strided"])
    base = _order_run(words, rdram, streams)
    runs = []
    monkeypatch.setenv("RDP_SHADE_PERM_MIN_PRIMS", "0")
    monkeypatch.setenv("RDP_SHADE_QUEUE_MIN", "0")
    for order in (SHADE_ORDERS["sm_queues"], SHADE_ORDERS["primitive_major"]):
        set_shade_order(order)
        assert get_shade_order() == order
        if order == SHADE_ORDERS["primitive_major"]:
            assert_parity(words, rdram)
        runs.append(_order_run(words, rdram, streams))
    monkeypatch.delenv("RDP_SHADE_PERM_MIN_PRIMS")
    monkeypatch.delenv("RDP_SHADE_QUEUE_MIN")
    runs.append(_order_run(words, rdram, streams))
    for single, batched in runs:
        for x, y in zip(single, base[0]):
            assert np.array_equal(x, y)
        for x, y in zip(batched, base[1]):
            assert np.array_equal(x, y)


def test_shade_order_rejects_unknown():
    with pytest.raises(Exception):
        set_shade_order(3)


@pytest.mark.parametrize("kernel", ["0", "1"], ids=["lookahead", "staged"])
def test_blend_kernels_bit_exact(monkeypatch, kernel):
    """Both blend kernels -- per-pair inputs through registers with L1 prefetch, or staged in a
    shared-memory ring by bulk copies on mbarriers -- give the oracle's bytes, on a stand-alone
    processor (mixed primitives) and on a batch."""
    monkeypatch.setenv("RDP_BLEND_KERNEL", kernel)
    m = cmdgen.default_params(cmdgen.CONFIG_MIXED, seed=61, num_prims=4000, num_frames=1)
    words, rdram, _ = cmdgen.generate_stream(m)
    assert_parity(words, rdram)
    streams = []
    for i in range(6):
        q = cmdgen.batched_instance_params(i, min_prims=500, max_prims=3000, seed_base=90)
        w, rd, _ = cmdgen.generate_stream(q)
        streams.append((w, rd))
    with Batch() as b:
        insts = [b.add_instance(rd.copy()) for _, rd in streams]
        for cp, (w, _) in zip(insts, streams):
            cp.enqueue_command(w)
        b.idle()
        for cp, (w, rd) in zip(insts, streams):
            single = run_gpu(w, rd)
            assert np.array_equal(cp.begin_read_rdram(), single[0])
            assert np.array_equal(cp.begin_read_hidden_rdram(), single[1])
