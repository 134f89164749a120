"""Shared helpers for the parity tests: run one command stream through the GPU
path (C ABI) and through the CPU oracle, and compare RDRAM + hidden RDRAM."""
import numpy as np


def run_oracle(words, rdram_init, rdram_size=8 << 20):
    from oracle import Oracle
    o = Oracle(rdram_size)
    o.write_rdram(rdram_init[:rdram_size])
    consumed = o.enqueue(words)
    assert consumed == len(words)
    run_oracle.reference_passes = o.reference_passes()
    return o.rdram(), o.hidden(), o.tmem(), o.fragments()


def run_gpu(words, rdram_init, rdram_size=8 << 20, chunks=1):
    from rdp_gb300 import CommandProcessor
    rd = np.array(rdram_init[:rdram_size], dtype=np.uint8, copy=True)
    with CommandProcessor(rd, rdram_size=rdram_size) as cp:
        if chunks == 1:
            cp.enqueue_command(words)
        else:
            # Split at arbitrary word boundaries to exercise partial-command carry.
            cuts = np.linspace(0, len(words), chunks + 1).astype(int)
            for a, b in zip(cuts[:-1], cuts[1:]):
                cp.enqueue_command(words[a:b])
        v = cp.signal_timeline()
        cp.wait_for_timeline(v)
        rdram = cp.begin_read_rdram().copy()
        hidden = cp.begin_read_hidden_rdram()
        tmem = cp.get_tmem()
        stats = cp.stats()
    return rdram, hidden, tmem, stats


def diff_report(name, a, b):
    if np.array_equal(a, b):
        return None
    idx = np.nonzero(a != b)[0]
    return "%s: %d bytes differ, first at 0x%x (gpu=%d oracle=%d)" % (name, idx.size, idx[0], a[idx[0]], b[idx[0]])


def assert_parity(words, rdram_init, rdram_size=8 << 20, chunks=1):
    g_rd, g_hid, g_tmem, stats = run_gpu(words, rdram_init, rdram_size, chunks)
    o_rd, o_hid, o_tmem, frags = run_oracle(words, rdram_init, rdram_size)
    errs = [e for e in (diff_report("rdram", g_rd, o_rd), diff_report("hidden", g_hid, o_hid),
                        diff_report("tmem", g_tmem.view(np.uint8), o_tmem.view(np.uint8))) if e]
    assert not errs, "; ".join(errs)
    assert stats["fragments"] == frags, (stats["fragments"], frags)
    # The throughput unit: both sides count the reference's render passes the same way.
    assert stats["reference_passes"] == run_oracle.reference_passes, (stats["reference_passes"],
                                                                      run_oracle.reference_passes)
    return stats
