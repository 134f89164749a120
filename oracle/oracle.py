"""ctypes binding of the CPU oracle (oracle/rdp_oracle.cpp) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use this
module, as the checker.  The product library never loads it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PATH = os.path.join(_HERE, "_build", "liboracle_rdp.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _PATH


def _load():
    global _lib
    if _lib is None:
        # RDP_ORACLE_LIB selects another build of the same sources (the op-count build of
        # make_op_table.py); by default the optimised build is used.
        path = os.environ.get("RDP_ORACLE_LIB", _PATH)
        if path == _PATH and not os.path.exists(_PATH):
            build()
        L = ctypes.CDLL(path)
        vp, u32 = ctypes.c_void_p, ctypes.c_uint32
        L.oracle_create.argtypes = [u32, u32]
        L.oracle_create.restype = vp
        L.oracle_destroy.argtypes = [vp]
        for n in ("oracle_write_rdram", "oracle_read_rdram", "oracle_read_hidden", "oracle_write_hidden"):
            getattr(L, n).argtypes = [vp, vp, u32, u32]
        L.oracle_read_tmem.argtypes = [vp, vp]
        L.oracle_apply_upload_plans.argtypes = [vp, vp, u32]
        L.oracle_enqueue.argtypes = [vp, vp, u32]
        L.oracle_enqueue.restype = u32
        L.oracle_fragments.argtypes = [vp]
        L.oracle_fragments.restype = ctypes.c_uint64
        L.oracle_primitive_count.argtypes = [vp]
        L.oracle_primitive_count.restype = u32
        L.oracle_reference_passes.argtypes = [vp]
        L.oracle_reference_passes.restype = ctypes.c_uint64
        L.oracle_blender_lut.argtypes = [vp, vp]
        for n in ("oracle_z_compress", "oracle_z_decompress", "oracle_dz_compress", "oracle_clamp_9bit",
                  "oracle_clamp_z"):
            getattr(L, n).argtypes = [ctypes.c_int]
            getattr(L, n).restype = ctypes.c_int
        L.oracle_perspective_divide.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.oracle_set_vi_register.argtypes = [vp, u32, u32]
        L.oracle_vi_begin_per_scanline.argtypes = [vp, u32]
        L.oracle_vi_set_for_scanline.argtypes = [vp, u32, u32]
        L.oracle_vi_latch_scanline.argtypes = [vp, u32]
        L.oracle_vi_end_per_scanline.argtypes = [vp]
        L.oracle_scanout.argtypes = [vp, vp, vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
        L.oracle_set_upscaling.argtypes = [vp, u32, u32, u32]
        L.oracle_set_upscaling.restype = ctypes.c_int
        L.oracle_upscaling_factor.argtypes = [vp]
        L.oracle_upscaling_factor.restype = u32
        for n in ("oracle_read_upscaled_rdram", "oracle_read_upscaled_hidden"):
            getattr(L, n).argtypes = [vp, vp, ctypes.c_uint64, ctypes.c_uint64]
        L.oracle_upscale_pre_external.argtypes = [vp, u32, u32, u32]
        L.oracle_noise.argtypes = [u32, u32, u32]
        L.oracle_noise.restype = ctypes.c_int
        _lib = L
    return _lib


def lib():
    return _load()


class Oracle:
    """Sequential per-pixel RDP oracle with its own RDRAM, hidden RDRAM and TMEM."""

    def __init__(self, rdram_size=8 << 20, hidden_size=None):
        if hidden_size is None:
            hidden_size = rdram_size // 2
        self.L = _load()
        self.h = self.L.oracle_create(rdram_size, hidden_size)
        if not self.h:
            raise ValueError("bad RDRAM sizes")
        self.rdram_size = rdram_size
        self.hidden_size = hidden_size

    def close(self):
        if self.h:
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def write_rdram(self, data, offset=0):
        d = np.ascontiguousarray(data, dtype=np.uint8)
        self.L.oracle_write_rdram(self.h, d.ctypes.data, offset, d.size)

    def rdram(self):
        out = np.zeros(self.rdram_size, dtype=np.uint8)
        self.L.oracle_read_rdram(self.h, out.ctypes.data, 0, out.size)
        return out

    def hidden(self):
        out = np.zeros(self.hidden_size, dtype=np.uint8)
        self.L.oracle_read_hidden(self.h, out.ctypes.data, 0, out.size)
        return out

    def tmem(self):
        out = np.zeros(2048, dtype=np.uint16)
        self.L.oracle_read_tmem(self.h, out.ctypes.data)
        return out

    def enqueue(self, words):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        return self.L.oracle_enqueue(self.h, w.ctypes.data, w.size)

    def fragments(self):
        return self.L.oracle_fragments(self.h)

    def write_hidden(self, data, offset=0):
        d = np.ascontiguousarray(data, dtype=np.uint8)
        self.L.oracle_write_hidden(self.h, d.ctypes.data, offset, d.size)

    def set_vi_register(self, reg, value):
        self.L.oracle_set_vi_register(self.h, int(reg), value & 0xffffffff)

    def begin_vi_register_per_scanline(self, flags):
        self.L.oracle_vi_begin_per_scanline(self.h, flags)

    def set_vi_register_for_scanline(self, reg_bit, value):
        self.L.oracle_vi_set_for_scanline(self.h, reg_bit, value & 0xffffffff)

    def latch_vi_register_for_scanline(self, line):
        self.L.oracle_vi_latch_scanline(self.h, line)

    def end_vi_register_per_scanline(self):
        self.L.oracle_vi_end_per_scanline(self.h)

    def set_upscaling(self, factor, super_sampled=False, dither=False):
        """Internal upscaling by 1, 2, 4 or 8, optionally with super-sampled readback; before any command."""
        if self.L.oracle_set_upscaling(self.h, factor, int(super_sampled), int(dither)) != 0:
            raise ValueError("unsupported upscaling")

    def upscaling_factor(self):
        return self.L.oracle_upscaling_factor(self.h)

    def upscaled_rdram(self):
        """The multisampled RDRAM: factor^2 slices of RDRAM, slice (y % f) * f + x % f."""
        f = self.upscaling_factor()
        out = np.zeros(self.rdram_size * f * f, dtype=np.uint8)
        self.L.oracle_read_upscaled_rdram(self.h, out.ctypes.data, 0, out.size)
        return out

    def upscaled_hidden(self):
        f = self.upscaling_factor()
        out = np.zeros(self.hidden_size * f * f, dtype=np.uint8)
        self.L.oracle_read_upscaled_hidden(self.h, out.ctypes.data, 0, out.size)
        return out

    def scanout(self, option_words):
        """option_words: the ScanoutOptions fields in C-ABI order (15, or 16 with downscale_steps).
        Returns uint32[h, w] or None."""
        words = list(option_words) + [0] * (16 - len(option_words))
        opts = np.array(words[:16], dtype=np.uint32)
        f = self.upscaling_factor()
        buf = np.zeros(640 * 576 * f * f, dtype=np.uint32)
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        self.L.oracle_scanout(self.h, opts.ctypes.data, buf.ctypes.data, ctypes.byref(w), ctypes.byref(h))
        return buf[:w.value * h.value].reshape(h.value, w.value) if w.value else None

    def primitive_count(self):
        return self.L.oracle_primitive_count(self.h)

    def reference_passes(self):
        """Render passes the reference would submit for the stream so far (rdp_renderer.cpp:1564-1590)."""
        return self.L.oracle_reference_passes(self.h)
