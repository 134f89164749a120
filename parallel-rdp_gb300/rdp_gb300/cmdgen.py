"""Binding of the seeded synthetic command-stream generator (include/rdp_cmdgen.h)."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PATH = os.path.join(os.path.dirname(_HERE), "csrc", "_build", "librdp_cmdgen.so")

CONFIG_PLAIN = 0      # 320x240 RGBA5551, 2,000 Gouraud triangles, 1-cycle
CONFIG_TEXTURED = 1   # 320x240 RGBA5551 + Z16, 10,000 textured 2-cycle triangles
CONFIG_MIXED = 2      # 640x480 RGBA8888, 16 frames x 50,000 mixed primitives

FLAGS = dict(CLEAR=1 << 0, Z=1 << 1, TWO_CYCLE=1 << 2, PERSPECTIVE=1 << 3, BILINEAR=1 << 4, AA=1 << 5,
             DITHER=1 << 6, FOG=1 << 7, RANDOM_COMBINER=1 << 8, Z_HALF=1 << 9, ALPHA_TEST_HALF=1 << 10,
             LOD=1 << 11, RUNS=1 << 12, FUZZ=1 << 13, HOTSPOT=1 << 14)

FB_RGBA5551, FB_RGBA8888, FB_I8, FB_IA88, FB_I4 = 0, 1, 2, 3, 4


class GenParams(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("fb_format", ctypes.c_uint32), ("num_prims", ctypes.c_uint32), ("num_frames", ctypes.c_uint32),
                ("area_median", ctypes.c_float), ("area_sigma", ctypes.c_float),
                ("w_shade_tri", ctypes.c_uint32), ("w_tex_tri", ctypes.c_uint32), ("w_copy_rect", ctypes.c_uint32),
                ("w_ci8_tri", ctypes.c_uint32), ("w_fill_rect", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("rdram_size", ctypes.c_uint32)]

    def describe(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_PATH):
            raise RuntimeError("librdp_cmdgen.so is not built (%s); run parallel-rdp_gb300/build.py" % _PATH)
        L = ctypes.CDLL(_PATH)
        L.rdpgen_default_params.argtypes = [ctypes.POINTER(GenParams), ctypes.c_int]
        L.rdpgen_build.argtypes = [ctypes.POINTER(GenParams)]
        L.rdpgen_build.restype = ctypes.c_void_p
        L.rdpgen_destroy.argtypes = [ctypes.c_void_p]
        L.rdpgen_num_words.argtypes = [ctypes.c_void_p]
        L.rdpgen_num_words.restype = ctypes.c_uint32
        L.rdpgen_num_prims.argtypes = [ctypes.c_void_p]
        L.rdpgen_num_prims.restype = ctypes.c_uint32
        L.rdpgen_words.argtypes = [ctypes.c_void_p]
        L.rdpgen_words.restype = ctypes.POINTER(ctypes.c_uint32)
        L.rdpgen_init_rdram.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
        L.rdpgen_num_frames.argtypes = [ctypes.c_void_p]
        L.rdpgen_num_frames.restype = ctypes.c_uint32
        L.rdpgen_frame_word_offset.argtypes = [ctypes.c_void_p, ctypes.c_uint32]
        L.rdpgen_frame_word_offset.restype = ctypes.c_uint32
        L.rdpgen_color_addr.restype = ctypes.c_uint32
        L.rdpgen_depth_addr.restype = ctypes.c_uint32
        _lib = L
    return _lib


def default_params(config, **overrides):
    p = GenParams()
    _load().rdpgen_default_params(ctypes.byref(p), config)
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def generate_stream(params):
    """Returns (words uint32[n], rdram_init uint8[rdram_size], num_prims)."""
    L = _load()
    g = L.rdpgen_build(ctypes.byref(params))
    try:
        n = L.rdpgen_num_words(g)
        words = np.ctypeslib.as_array(L.rdpgen_words(g), shape=(n,)).copy()
        rdram = np.zeros(params.rdram_size, dtype=np.uint8)
        L.rdpgen_init_rdram(g, rdram.ctypes.data, rdram.size)
        return words, rdram, L.rdpgen_num_prims(g)
    finally:
        L.rdpgen_destroy(g)


def generate_frames(params):
    """Returns (words, rdram_init, num_prims, frame_offsets): frame f's words are
    words[frame_offsets[f]:frame_offsets[f + 1]]."""
    L = _load()
    g = L.rdpgen_build(ctypes.byref(params))
    try:
        n = L.rdpgen_num_words(g)
        words = np.ctypeslib.as_array(L.rdpgen_words(g), shape=(n,)).copy()
        rdram = np.zeros(params.rdram_size, dtype=np.uint8)
        L.rdpgen_init_rdram(g, rdram.ctypes.data, rdram.size)
        nf = L.rdpgen_num_frames(g)
        offsets = [L.rdpgen_frame_word_offset(g, f) for f in range(nf + 1)]
        return words, rdram, L.rdpgen_num_prims(g), offsets
    finally:
        L.rdpgen_destroy(g)


def color_addr():
    return _load().rdpgen_color_addr()


def depth_addr():
    return _load().rdpgen_depth_addr()


BATCH_RESOLUTIONS = ((320, 240), (640, 240), (640, 480))


def batched_instance_params(instance, min_prims=500, max_prims=50000, seed_base=0):
    """Generator parameters of one instance of the batched-instances workload: the
    mixed RGBA8888 primitive mix of CONFIG_MIXED, one frame, a resolution drawn from
    BATCH_RESOLUTIONS and a primitive count log-uniform in [min_prims, max_prims],
    both drawn from the instance seed (seed_base + instance)."""
    import math
    seed = seed_base + instance
    rng = np.random.default_rng(0x5EED0000 + seed)
    w, h = BATCH_RESOLUTIONS[int(rng.integers(0, len(BATCH_RESOLUTIONS)))]
    u = float(rng.random())
    n = int(round(math.exp(math.log(min_prims) + u * (math.log(max_prims) - math.log(min_prims)))))
    return default_params(CONFIG_MIXED, seed=seed, width=w, height=h, num_prims=n, num_frames=1)
