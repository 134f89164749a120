"""TMEM loads written two ways: as RDP command words, and as the upload plans a processor derives
from them (the 64-byte plan record of rdp_tmem_update_noalloc).  The plans are derived by hand from
the reference's load planning (parallel-rdp/rdp_renderer.cpp:3099-3486: load_tile and
load_tile_iteration); tests/test_tmem_plans.py checks each one against the oracle's own planning on
the CPU before the GPU test relies on it.

A load is (kind, texture address, parameters); kinds:
  tile  -- LoadTile of an RGBA16 width x height texture (tile 7, `stride` bytes per TMEM line)
  tlut  -- LoadTLUT of `entries` RGBA16 palette entries into TMEM's upper half
  block -- LoadBlock of `texels` texels of `bits` (16 or 32) bits, TMEM line `stride` bytes, dxt
"""
import numpy as np

UPLOAD = np.dtype([("width", "<i4"), ("height", "<i4"), ("min_t_mod", "<f4"), ("max_t_mod", "<f4"),
                   ("vram_addr", "<i4"), ("vram_width", "<i4"), ("vram_size", "<i4"),
                   ("vram_effective_width", "<i4"), ("tmem_offset", "<i4"), ("tmem_stride_words", "<i4"),
                   ("tmem_size", "<i4"), ("tmem_fmt", "<i4"), ("mode", "<i4"), ("inv_tmem_stride_words", "<f4"),
                   ("dxt", "<i4"), ("padding", "<i4")])
assert UPLOAD.itemsize == 64


def _f32_recip(x):
    with np.errstate(divide="ignore"):
        return np.float32(1.0) / np.float32(x)


def _set_texture_image(addr, size, width):
    return [(0x3d << 24) | (0 << 21) | (size << 19) | (width - 1), addr]


def _set_tile(size, stride_bytes, tmem_bytes, tile=7):
    return [(0x35 << 24) | (0 << 21) | (size << 19) | ((stride_bytes // 8) << 9) | (tmem_bytes // 8), tile << 24]


def commands(load):
    kind, addr = load[0], load[1]
    if kind == "tile":
        _, _, width, height, stride, tmem = load
        return (_set_texture_image(addr, 2, width) + _set_tile(2, stride, tmem) +
                [0x34 << 24, (7 << 24) | (((width - 1) << 2) << 12) | ((height - 1) << 2)])
    if kind == "tlut":
        _, _, entries, tmem = load
        return (_set_texture_image(addr, 2, entries) + _set_tile(2, 0, tmem) +
                [0x30 << 24, (7 << 24) | (((entries - 1) << 2) << 12)])
    if kind == "block":
        _, _, texels, bits, stride, tmem, dxt = load
        size = 2 if bits == 16 else 3
        return (_set_texture_image(addr, size, 1) + _set_tile(size, stride, tmem) +
                [0x33 << 24, (7 << 24) | ((texels - 1) << 12) | dxt])
    raise ValueError(kind)


def plan(load):
    """The upload plan of one load (load_tile_iteration, rdp_renderer.cpp:3222-3486)."""
    u = np.zeros(1, UPLOAD)
    kind, addr = load[0], load[1]
    if kind == "tile":
        _, _, width, height, stride, tmem = load
        eff = (width + 3) & ~3
        u["width"], u["height"] = eff, height
        u["vram_addr"], u["vram_width"], u["vram_size"], u["vram_effective_width"] = addr, width, 2, eff
        u["tmem_offset"], u["tmem_stride_words"] = tmem & 0xfff, stride // 2
        u["tmem_size"], u["tmem_fmt"], u["mode"] = 2, 0, 0
        u["inv_tmem_stride_words"] = _f32_recip(stride // 2)
    elif kind == "tlut":
        _, _, entries, tmem = load
        u["width"], u["height"] = (entries + 3) & ~3, 1
        u["vram_addr"], u["vram_width"], u["vram_size"], u["vram_effective_width"] = addr, entries, 2, entries
        u["tmem_offset"], u["tmem_stride_words"] = tmem & 0xfff, 0
        u["tmem_size"], u["tmem_fmt"], u["mode"] = 2, 0, 1
        u["inv_tmem_stride_words"] = _f32_recip(0)
    elif kind == "block":
        _, _, texels, bits, stride, tmem, dxt = load
        isize = 2 if bits == 16 else 3
        stride_words = stride // 2
        max_iter = (texels - 1) >> (4 - isize)
        max_t = (max_iter * dxt) >> 11
        u["vram_addr"], u["vram_size"] = addr, isize
        u["tmem_offset"], u["tmem_size"], u["tmem_fmt"] = tmem & 0xfff, isize, 0
        eff = (texels + 3) & ~3 if isize == 2 else (texels + 1) & ~1
        u["vram_effective_width"] = eff
        u["width"], u["height"] = eff, 1
        if max_t:
            maxn, minn = (2048 + dxt - 1) // dxt, 2048 // dxt
            assert maxn == minn or (dxt * maxn - 2048) * max_t < dxt, "uneven LoadBlock cases are not planned here"
            if isize == 3:
                stride_words <<= 1
            u["dxt"] = dxt << 5
            u["min_t_mod"] = _f32_recip(maxn + (stride_words >> 2))
            u["max_t_mod"] = _f32_recip(maxn + (stride_words >> 2))
            stride_words >>= 2
            u["mode"], u["vram_width"] = 2, eff
        else:
            stride_words = 0
            u["mode"], u["vram_width"] = 0, 1  # a one-line block is a LoadTile of the image's width
        u["tmem_stride_words"] = stride_words
        u["inv_tmem_stride_words"] = _f32_recip(stride_words)
    else:
        raise ValueError(kind)
    return u


# Two groups of loads, applied one group after the other.  Together they cover the three upload
# modes: LoadTile (0), LoadTLUT (1) and LoadBlock (2, the fp32 line-stepping path), plus a
# one-line LoadBlock that is planned as a LoadTile.
GROUP_FIRST = [("tile", 0x600000, 32, 32, 64, 0), ("tlut", 0x604000, 256, 0x800),
               ("block", 0x605000, 1024, 16, 64, 0x400, 256)]
GROUP_SECOND = [("tile", 0x602000, 16, 32, 32, 512), ("block", 0x606000, 256, 32, 64, 0, 256),
                ("tlut", 0x604400, 16, 0xe00), ("block", 0x607000, 16, 16, 32, 0xc00, 512)]
TEXTURE_BYTES = (0x600000, 0x608000)  # every load reads inside this range
