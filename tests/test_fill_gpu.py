"""Passes drawn only by the fill pipe (a frame's clears) take their own kernel: set-up, binning,
TMEM and one per-tile fill (RdpLaunch.fill_only).  Bit-exact against the CPU oracle on hand-built
streams: fill rectangles with sub-pixel edges, rectangles partly or wholly outside the image,
empty ones, interlaced scissor fields, every framebuffer format that fills, and image switches
between them.  That the fill kernel ran is checked through the launch count: three kernels per
fill-only pass (k_prim_setup, k_bin, k_fill)."""
import numpy as np
import pytest

from rdp_gb300 import cmdgen
from rdp_testutil import assert_parity

pytestmark = pytest.mark.gpu

# (format, size) of SetColorImage: RGBA5551, RGBA8888, IA88, I8.
FORMATS = [(0, 2), (0, 3), (3, 2), (4, 1)]


def _color_image(fmt, size, width, addr):
    return [(0x3f << 24) | (fmt << 21) | (size << 19) | (width - 1), addr]


def _scissor(x0, y0, x1, y1, field=0):
    # 10.2 fixed point; field: 0 off, 2 keep even lines, 3 keep odd lines.
    return [(0x2d << 24) | (x0 << 12) | y0, (field << 24) | (x1 << 12) | y1]


def _fill_rect(xl, yl, xh, yh):
    # 10.2 fixed point: (xl, yl) lower right, (xh, yh) upper left.
    return [(0x36 << 24) | (xl << 12) | yl, (xh << 12) | yh]


FILL_MODE = [(0x2f << 24) | (3 << 20), 0]
SYNC_FULL = [0x29 << 24, 0]


def _fill_stream(seed, formats, width=320, height=240, rects=40, field=False):
    rng = np.random.default_rng(seed)
    words = []
    base = 0x100000
    for i, (fmt, size) in enumerate(formats):
        addr = base + i * 0x80000
        words += _color_image(fmt, size, width, addr)
        f = int(rng.choice([2, 3])) if field else 0
        words += _scissor(int(rng.integers(0, 40)), int(rng.integers(0, 40)), (width << 2) - int(rng.integers(0, 40)),
                          (height << 2) - int(rng.integers(0, 40)), f)
        words += FILL_MODE
        for _ in range(rects):
            words += [0x37 << 24, int(rng.integers(0, 1 << 32, dtype=np.uint64))]
            x0 = int(rng.integers(-64, width * 4))
            y0 = int(rng.integers(-64, height * 4))
            x1 = x0 + int(rng.integers(-8, width * 3))
            y1 = y0 + int(rng.integers(-8, height * 3))
            words += _fill_rect(max(x1, 0) & 0xfff, max(y1, 0) & 0xfff, max(x0, 0) & 0xfff, max(y0, 0) & 0xfff)
    words += SYNC_FULL
    return np.array(words, dtype=np.uint32)


@pytest.mark.parametrize("seed", [0, 1])
def test_fill_passes_every_format(seed):
    words = _fill_stream(seed, FORMATS)
    rdram = np.random.default_rng(100 + seed).integers(0, 256, 8 << 20, dtype=np.uint8)
    stats = assert_parity(words, rdram)
    assert stats["kernel_launches"] == 3 * stats["passes"], stats


def test_fill_passes_interlaced_fields_and_odd_width():
    words = _fill_stream(7, FORMATS[:2] * 2, width=301, height=203, rects=25, field=True)
    rdram = np.random.default_rng(7).integers(0, 256, 8 << 20, dtype=np.uint8)
    assert_parity(words, rdram)


def test_full_frame_clear_then_geometry():
    # A depth clear (its own image: fill-only) and the colour clear sharing a pass with triangles.
    p = cmdgen.default_params(cmdgen.CONFIG_TEXTURED, seed=9, num_prims=500)
    words, rdram, _ = cmdgen.generate_stream(p)
    assert_parity(words, rdram)


def test_fill_passes_in_a_batch_round():
    # Several instances whose passes are all fills share rounds of the batched executor.
    from rdp_gb300 import Batch
    from rdp_testutil import run_oracle
    streams = [_fill_stream(20 + i, FORMATS[i % 4:i % 4 + 1] * 2, rects=30) for i in range(6)]
    inits = [np.random.default_rng(200 + i).integers(0, 256, 8 << 20, dtype=np.uint8) for i in range(6)]
    with Batch() as b:
        insts = [b.add_instance(r.copy()) for r in inits]
        for cp, w in zip(insts, streams):
            cp.enqueue_command(w)
        values = [cp.signal_timeline() for cp in insts]
        b.submit()
        for cp, v in zip(insts, values):
            cp.wait_for_timeline(v)
        st = b.stats()
        assert st["rounds"] < st["passes"], st
        for i, (cp, w, r) in enumerate(zip(insts, streams, inits)):
            got = cp.begin_read_rdram().copy()
            o_rd, o_hid, _, frags = run_oracle(w, r)
            assert np.array_equal(got, o_rd), "instance %d: %d bytes differ" % (i, int((got != o_rd).sum()))
            assert np.array_equal(cp.begin_read_hidden_rdram(), o_hid), "instance %d hidden" % i
            assert cp.stats()["fragments"] == frags


def test_fill_then_fused_path_keeps_tile_counts_clean():
    # A fill-only pass bins without counting tiles; the pair path of the next pass must see
    # only its own counts.
    # (SyncFull ends each pass.)
    fill = _fill_stream(31, FORMATS[:1], rects=20)
    p = cmdgen.default_params(cmdgen.CONFIG_PLAIN, seed=31, num_prims=400)
    geo, rdram, _ = cmdgen.generate_stream(p)
    words = np.concatenate([fill, geo, fill, geo, SYNC_FULL])
    stats = assert_parity(words, rdram.copy())
    assert stats["passes"] >= 4, stats
