"""RDRAM coherency with the caller's memory (the reference's incoherent-host path,
rdp_renderer.cpp:2523-2907): the GPU reads the pages a pass needs from the caller's RDRAM (masked:
bytes the GPU wrote and has not yet returned stay the GPU's), and a timeline value writes back only
the bytes the GPU wrote, so the caller's own writes elsewhere in a rendered page survive.

* CPU writes inside a framebuffer between two passes, without idling: pass A draws into the top of a
  320x240 RGBA5551 image (scissor rows 0-99); the CPU then writes random bytes into rows 120-239 of
  the same image (pages that A's write-back also covers); pass B blends over the whole image and
  reads those bytes.  The caller's RDRAM must equal the oracle's for A, the same CPU write, then B.
* Texture pages refreshed without any call: after a frame has completed, the CPU rewrites the
  texture data in its RDRAM and enqueues the frame again; the second image must use the new texels.
Exact comparisons (integer data)."""
import numpy as np
import pytest

from rdp_gb300 import CommandProcessor, cmdgen
from rdp_testutil import run_oracle

pytestmark = pytest.mark.gpu
F = cmdgen.FLAGS


def _with_scissor_rows(words, rows):
    """The stream with every SetScissor (op 0x2d) limited to rows [0, rows)."""
    w = words.copy()
    i = 0
    lengths = {0x08: 8, 0x09: 12, 0x0a: 24, 0x0b: 28, 0x0c: 24, 0x0d: 28, 0x0e: 40, 0x0f: 44, 0x24: 4, 0x25: 4}
    while i < len(w):
        op = (int(w[i]) >> 24) & 63
        if op == 0x2d:
            w[i + 1] = (int(w[i + 1]) & ~0xfff) | (rows << 2)
        i += lengths.get(op, 2)
    return w


def test_cpu_writes_in_a_rendered_page_between_passes_without_idle():
    pa = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=41, num_prims=400, flags=0)
    a_words, rdram, _ = cmdgen.generate_stream(pa)
    a_words = _with_scissor_rows(a_words, 100)
    pb = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=42, num_prims=300, flags=F["FUZZ"])
    b_words, _, _ = cmdgen.generate_stream(pb)
    base = cmdgen.color_addr()
    lo, hi = base + 120 * 320 * 2, base + 240 * 320 * 2
    cpu = np.random.default_rng(5).integers(0, 256, hi - lo, dtype=np.uint8)

    from oracle import Oracle
    o = Oracle(8 << 20)
    o.write_rdram(rdram)
    o.enqueue(a_words)
    mid = o.rdram().copy()
    assert np.array_equal(mid[lo:hi], rdram[lo:hi])  # A does not write the CPU's rows
    mid[lo:hi] = cpu
    o.write_rdram(mid)
    o.enqueue(b_words)
    want_rd, want_hid = o.rdram().copy(), o.hidden().copy()
    o.close()

    rd = rdram.copy()
    with CommandProcessor(rd) as cp:
        cp.enqueue_command(a_words)
        cp.flush()                # pass A is submitted; no wait
        rd[lo:hi] = cpu           # the CPU writes into the image A rendered into
        cp.enqueue_command(b_words)
        v = cp.signal_timeline()
        cp.wait_for_timeline(v)
        got_rd = rd.copy()
        got_hid = cp.begin_read_hidden_rdram().copy()
    assert np.array_equal(got_rd, want_rd), "RDRAM differs in %d bytes" % int((got_rd != want_rd).sum())
    assert np.array_equal(got_hid, want_hid)


def test_texture_pages_are_read_from_the_callers_rdram():
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=43, num_prims=600)
    words, rdram, _ = cmdgen.generate_stream(p)
    textures = np.nonzero(rdram)[0]  # the generator's texture and TLUT data
    assert textures.size > 1000
    new = rdram.copy()
    new[textures] = np.random.default_rng(6).integers(0, 256, textures.size, dtype=np.uint8)

    from oracle import Oracle
    o = Oracle(8 << 20)
    o.write_rdram(rdram)
    o.enqueue(words)
    mid = o.rdram().copy()
    mid[textures] = new[textures]
    o.write_rdram(mid)
    o.enqueue(words)
    want = o.rdram().copy()
    o.close()
    first = run_oracle(words, rdram)[0]

    rd = rdram.copy()
    with CommandProcessor(rd) as cp:
        cp.enqueue_command(words)
        cp.wait_for_timeline(cp.signal_timeline())
        assert np.array_equal(rd, first)
        rd[textures] = new[textures]  # no API call: the next loads read the caller's pages
        cp.enqueue_command(words)
        cp.wait_for_timeline(cp.signal_timeline())
        got = rd.copy()
    assert not np.array_equal(want, first)  # the new texels change the image
    assert np.array_equal(got, want), "RDRAM differs in %d bytes" % int((got != want).sum())
