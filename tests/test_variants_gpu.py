"""Kernel specialisations: every compiled variant of the shading kernel produces the same
RDRAM / hidden RDRAM / TMEM bytes, and the autotuner settles on one of them."""
import numpy as np
import pytest

from rdp_gb300 import SHADE_VARIANTS, Batch, cmdgen, get_shade_variant, set_shade_variant
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
    results = []
    for v in range(SHADE_VARIANTS):
        set_shade_variant(v)
        assert get_shade_variant() == v
        if v == SHADE_VARIANTS - 1:
            assert_parity(words, rdram)  # one variant also against the oracle
        results.append((run_gpu(words, rdram)[:3], run_gpu(fwords, frdram)[:3]))
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
