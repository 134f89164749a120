"""The fused fallback (k_raster): a launch whose (primitive, tile) pairs or span rows do not fit the
executor's scratch shades and blends each tile in one kernel instead of taking the pair path.  It
must write the same bytes as the pair path, i.e. match the oracle.  RDP_PAIR_CAPACITY and
RDP_SPAN_ROW_CAPACITY (read when a processor or a batch is created) shrink the starting
capacities so that the launches overflow."""
import numpy as np
import pytest

from rdp_gb300 import Batch, cmdgen
from rdp_testutil import assert_parity, run_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("var", ["RDP_PAIR_CAPACITY", "RDP_SPAN_ROW_CAPACITY"])
def test_standalone_overflow_takes_fallback_bit_exact(monkeypatch, var):
    # A stand-alone processor keeps its starting capacity, so every pass of these streams
    # (~10k pairs and thousands of span rows per pass) overflows it.
    monkeypatch.setenv(var, "64")
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=11, num_prims=1500)
    words, rdram, _ = cmdgen.generate_stream(p)
    assert_parity(words, rdram)
    q = cmdgen.default_params(cmdgen.CONFIG_MIXED, seed=12, num_prims=1200, num_frames=1)
    words, rdram, _ = cmdgen.generate_stream(q)
    assert_parity(words, rdram)
    # Fuzzed state on an I8 image (visible pass boundaries, image switches, loads from
    # rendered images).
    f = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=13, num_prims=600, fb_format=cmdgen.FB_I8,
                              flags=cmdgen.FLAGS["FUZZ"] | cmdgen.FLAGS["CLEAR"])
    words, rdram, _ = cmdgen.generate_stream(f)
    assert_parity(words, rdram)


def test_batch_overflows_then_grows_to_the_pair_path(monkeypatch):
    # First sync point: the batch's launches overflow and take the fallback; at idle the batch
    # grows its scratch to the counts it saw, so the second frame takes the pair path.  Both
    # frames must land exactly where the oracle puts them.
    monkeypatch.setenv("RDP_PAIR_CAPACITY", "256")
    monkeypatch.setenv("RDP_SPAN_ROW_CAPACITY", "256")
    streams = []
    for i in range(4):
        p = cmdgen.batched_instance_params(i, min_prims=300, max_prims=1500, seed_base=90)
        w, rd, _ = cmdgen.generate_stream(p)
        streams.append((w, rd))
    with Batch() as b:
        insts = [b.add_instance(np.array(rd, copy=True)) for _, rd in streams]
        for _ in range(2):
            for cp, (w, _) in zip(insts, streams):
                cp.enqueue_command(w)
            b.idle()
        for i, (cp, (w, rd)) in enumerate(zip(insts, streams)):
            o_rd, o_hid, o_tmem, _ = run_oracle(np.concatenate([w, w]), rd)
            assert np.array_equal(cp.begin_read_rdram(), o_rd), "instance %d rdram" % i
            assert np.array_equal(cp.begin_read_hidden_rdram(), o_hid), "instance %d hidden" % i
            assert np.array_equal(cp.get_tmem().view(np.uint8), o_tmem.view(np.uint8)), "instance %d tmem" % i
