"""ctypes binding of librdp_cuda.so (include/rdp_cuda.h)."""
import ctypes
import enum
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(os.path.dirname(_HERE), "csrc", "_build")

RDP_OK = 0
RDP_ERR_UNSUPPORTED = 1
RDP_ERR_OOM = 2
RDP_ERR_TIMEOUT = 3
RDP_ERR_INVALID = 4
RDP_ERR_DEVICE = 5
_ERR_NAMES = {1: "unsupported", 2: "out of memory", 3: "timeout", 4: "invalid argument", 5: "CUDA error"}


class RdpError(RuntimeError):
    def __init__(self, code, what):
        super().__init__("%s failed: %s (%d)" % (what, _ERR_NAMES.get(code, "error"), code))
        self.code = code


class RdpTimeout(RdpError):
    pass


class VIRegister(enum.IntEnum):
    """rdp_common.hpp:286-302"""
    Control = 0
    Origin = 1
    Width = 2
    Intr = 3
    VCurrentLine = 4
    Timing = 5
    VSync = 6
    HSync = 7
    Leap = 8
    HStart = 9
    VStart = 10
    VBurst = 11
    XScale = 12
    YScale = 13


class _CreateInfo(ctypes.Structure):
    _fields_ = [("rdram", ctypes.c_void_p), ("rdram_offset", ctypes.c_size_t), ("rdram_size", ctypes.c_size_t),
                ("hidden_rdram_size", ctypes.c_size_t), ("flags", ctypes.c_uint32), ("device", ctypes.c_int)]


class ScanoutOptions(ctypes.Structure):
    """ScanoutOptions (video_interface.hpp:31-81) at 1x scale; defaults as the reference."""
    _fields_ = [("crop_overscan_pixels", ctypes.c_uint32), ("crop_rect_enable", ctypes.c_uint32),
                ("crop_left", ctypes.c_uint32), ("crop_right", ctypes.c_uint32), ("crop_top", ctypes.c_uint32),
                ("crop_bottom", ctypes.c_uint32), ("persist_frame_on_invalid_input", ctypes.c_uint32),
                ("blend_previous_frame", ctypes.c_uint32), ("upscale_deinterlacing", ctypes.c_uint32),
                ("vi_aa", ctypes.c_uint32), ("vi_scale", ctypes.c_uint32), ("vi_serrate", ctypes.c_uint32),
                ("vi_dither_filter", ctypes.c_uint32), ("vi_divot_filter", ctypes.c_uint32),
                ("vi_gamma_dither", ctypes.c_uint32), ("downscale_steps", ctypes.c_uint32)]

    def __init__(self, **kw):
        super().__init__()
        self.upscale_deinterlacing = 1
        for k in ("vi_aa", "vi_scale", "vi_serrate", "vi_dither_filter", "vi_divot_filter", "vi_gamma_dither"):
            setattr(self, k, 1)
        for k, v in kw.items():
            setattr(self, k, int(v))

    def as_words(self):
        return [getattr(self, k) for k, _ in self._fields_]


class _Stats(ctypes.Structure):
    _fields_ = [("primitives", ctypes.c_uint64), ("passes", ctypes.c_uint64), ("reference_passes", ctypes.c_uint64),
                ("fragments", ctypes.c_uint64), ("tmem_uploads", ctypes.c_uint64), ("touched_tiles", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint64), ("staging_bytes", ctypes.c_uint64),
                ("tile_instances", ctypes.c_uint64)]


_VALIDATION_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p)

EXPORTED_SYMBOLS = [
    "rdp_cp_create", "rdp_cp_destroy", "rdp_device_is_supported", "rdp_cp_enqueue", "rdp_cp_signal_timeline",
    "rdp_cp_wait_timeline", "rdp_cp_flush", "rdp_cp_idle", "rdp_cp_begin_frame_context", "rdp_cp_set_quirks",
    "rdp_cp_set_validation_callback", "rdp_cp_begin_read_rdram", "rdp_cp_end_write_rdram",
    "rdp_cp_begin_read_hidden_rdram", "rdp_cp_end_write_hidden_rdram", "rdp_cp_get_rdram_size",
    "rdp_cp_get_hidden_rdram_size", "rdp_cp_get_tmem", "rdp_cp_set_vi_register", "rdp_cp_scanout_sync",
    "rdp_cp_get_stats", "rdp_cp_capture_begin", "rdp_cp_capture_end", "rdp_graph_replay", "rdp_graph_kernel_count",
    "rdp_graph_destroy", "rdp_graph_last_shade_ms", "rdp_graph_shade_launches", "rdp_scanout_options_default",
    "rdp_cp_begin_vi_register_per_scanline", "rdp_cp_set_vi_register_for_scanline",
    "rdp_cp_latch_vi_register_for_scanline", "rdp_cp_end_vi_register_per_scanline",
    "rdp_batch_create", "rdp_batch_destroy", "rdp_batch_add_instance", "rdp_batch_submit", "rdp_batch_idle",
    "rdp_batch_get_stats", "rdp_batch_capture_begin", "rdp_batch_capture_end", "rdp_set_shade_variant",
    "rdp_get_shade_variant", "rdp_set_shade_order", "rdp_get_shade_order", "rdp_batch_set_schedule", "rdp_batch_get_model", "rdp_batch_set_model",
    "rdp_mlp_gradients", "rdp_mlp_forward", "rdp_batch_get_tile_samples", "rdp_graph_last_blend_ms",
    "rdp_serve_run", "rdp_batch_enqueue_many", "rdp_dump_writer_open", "rdp_dump_writer_flush_rdram",
    "rdp_dump_writer_flush_hidden_rdram", "rdp_dump_writer_command", "rdp_dump_writer_set_vi_register",
    "rdp_dump_writer_end_frame", "rdp_dump_writer_signal_complete", "rdp_dump_writer_close", "rdp_dump_replay",
    "rdp_cp_get_scaling_factor", "rdp_cp_read_upscaled_rdram", "rdp_cp_read_upscaled_hidden_rdram",
]


class _ServeRequest(ctypes.Structure):
    _fields_ = [("instance", ctypes.c_uint32), ("num_words", ctypes.c_uint32), ("words", ctypes.c_void_p),
                ("arrival_s", ctypes.c_double), ("footprint_bytes", ctypes.c_uint64)]


class _ServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_in_flight", ctypes.c_uint32),
                ("timeout_s", ctypes.c_double)]


class _ServeResult(ctypes.Structure):
    _fields_ = [("admit_s", ctypes.c_double), ("done_s", ctypes.c_double), ("latency_s", ctypes.c_double)]


class _ServeStats(ctypes.Structure):
    _fields_ = [("submits", ctypes.c_uint64), ("max_in_flight", ctypes.c_uint64), ("max_footprint", ctypes.c_uint64),
                ("elapsed_s", ctypes.c_double)]


class _BatchCreateInfo(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("flags", ctypes.c_uint32)]


class _BatchStats(ctypes.Structure):
    _fields_ = [("instances", ctypes.c_uint64), ("rounds", ctypes.c_uint64), ("passes", ctypes.c_uint64),
                ("kernel_launches", ctypes.c_uint64), ("staging_bytes", ctypes.c_uint64)]


CREATE_COMMAND_THREAD = 1 << 0
CREATE_UPSCALING_2X = 1 << 2
CREATE_UPSCALING_4X = 1 << 3
CREATE_UPSCALING_8X = 1 << 4
CREATE_SUPER_SAMPLED_READ_BACK = 1 << 5
CREATE_SUPER_SAMPLED_DITHER = 1 << 6
_UPSCALING_FLAGS = {1: 0, 2: CREATE_UPSCALING_2X, 4: CREATE_UPSCALING_4X, 8: CREATE_UPSCALING_8X}
BATCH_TILE_ORDER_LEARNED = 1 << 0
BATCH_RECORD_TILE_CYCLES = 1 << 1


def library_path():
    return os.path.join(_BUILD, "librdp_cuda.so")


_lib = None


def lib():
    """Loads librdp_cuda.so; raises when it is missing (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError("librdp_cuda.so is not built (%s); run parallel-rdp_gb300/build.py" % path)
    L = ctypes.CDLL(path)
    vp, u32, u64, sz = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t
    L.rdp_cp_create.argtypes = [ctypes.POINTER(_CreateInfo), ctypes.POINTER(vp)]
    L.rdp_cp_destroy.argtypes = [vp]
    L.rdp_cp_destroy.restype = None
    L.rdp_device_is_supported.argtypes = [ctypes.c_int]
    L.rdp_cp_enqueue.argtypes = [vp, u32, vp]
    L.rdp_cp_signal_timeline.argtypes = [vp, ctypes.POINTER(u64)]
    L.rdp_cp_wait_timeline.argtypes = [vp, u64, u64]
    for n in ("rdp_cp_flush", "rdp_cp_idle", "rdp_cp_begin_frame_context", "rdp_cp_end_write_rdram",
              "rdp_cp_end_write_hidden_rdram"):
        getattr(L, n).argtypes = [vp]
    L.rdp_cp_set_quirks.argtypes = [vp, u32]
    L.rdp_cp_set_validation_callback.argtypes = [vp, _VALIDATION_CB, vp]
    L.rdp_cp_begin_read_rdram.argtypes = [vp]
    L.rdp_cp_begin_read_rdram.restype = vp
    L.rdp_cp_begin_read_hidden_rdram.argtypes = [vp]
    L.rdp_cp_begin_read_hidden_rdram.restype = vp
    L.rdp_cp_get_rdram_size.argtypes = [vp]
    L.rdp_cp_get_rdram_size.restype = sz
    L.rdp_cp_get_hidden_rdram_size.argtypes = [vp]
    L.rdp_cp_get_hidden_rdram_size.restype = sz
    L.rdp_cp_get_tmem.argtypes = [vp, vp]
    L.rdp_cp_get_scaling_factor.argtypes = [vp]
    L.rdp_cp_get_scaling_factor.restype = u32
    for n in ("rdp_cp_read_upscaled_rdram", "rdp_cp_read_upscaled_hidden_rdram"):
        getattr(L, n).argtypes = [vp, vp, u64, u64]
    L.rdp_cp_set_vi_register.argtypes = [vp, u32, u32]
    L.rdp_cp_scanout_sync.argtypes = [vp, ctypes.POINTER(ScanoutOptions), vp, ctypes.POINTER(u32),
                                      ctypes.POINTER(u32)]
    L.rdp_cp_begin_vi_register_per_scanline.argtypes = [vp, u32]
    L.rdp_cp_set_vi_register_for_scanline.argtypes = [vp, u32, u32]
    L.rdp_cp_latch_vi_register_for_scanline.argtypes = [vp, u32]
    L.rdp_cp_end_vi_register_per_scanline.argtypes = [vp]
    L.rdp_cp_get_stats.argtypes = [vp, ctypes.POINTER(_Stats)]
    L.rdp_cp_capture_begin.argtypes = [vp]
    L.rdp_cp_capture_end.argtypes = [vp, ctypes.POINTER(vp)]
    L.rdp_graph_replay.argtypes = [vp, u32, ctypes.POINTER(ctypes.c_float)]
    L.rdp_graph_kernel_count.argtypes = [vp]
    L.rdp_graph_kernel_count.restype = u32
    L.rdp_graph_destroy.argtypes = [vp]
    L.rdp_graph_destroy.restype = None
    L.rdp_graph_last_shade_ms.argtypes = [vp]
    L.rdp_graph_last_shade_ms.restype = ctypes.c_float
    L.rdp_graph_last_blend_ms.argtypes = [vp]
    L.rdp_graph_last_blend_ms.restype = ctypes.c_float
    L.rdp_graph_shade_launches.argtypes = [vp]
    L.rdp_graph_shade_launches.restype = u32
    L.rdp_set_shade_variant.argtypes = [ctypes.c_int, ctypes.c_int]
    L.rdp_get_shade_variant.argtypes = [ctypes.c_int]
    L.rdp_set_shade_order.argtypes = [ctypes.c_int, ctypes.c_int]
    L.rdp_get_shade_order.argtypes = [ctypes.c_int]
    L.rdp_batch_set_schedule.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, u32]
    L.rdp_batch_get_model.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_float)]
    L.rdp_batch_set_model.argtypes = [vp, vp]
    L.rdp_batch_get_tile_samples.argtypes = [vp, vp, vp, vp, u32, ctypes.POINTER(u32)]
    L.rdp_mlp_gradients.argtypes = [ctypes.c_int, vp, vp, vp, u32, vp, ctypes.POINTER(ctypes.c_float)]
    L.rdp_mlp_forward.argtypes = [ctypes.c_int, vp, vp, u32, vp]
    L.rdp_serve_run.argtypes = [vp, vp, u32, vp, u32, ctypes.POINTER(_ServeConfig), vp, ctypes.POINTER(_ServeStats)]
    L.rdp_batch_create.argtypes = [ctypes.POINTER(_BatchCreateInfo), ctypes.POINTER(vp)]
    L.rdp_batch_destroy.argtypes = [vp]
    L.rdp_batch_add_instance.argtypes = [vp, ctypes.POINTER(_CreateInfo), ctypes.POINTER(vp)]
    L.rdp_batch_submit.argtypes = [vp]
    L.rdp_batch_enqueue_many.argtypes = [vp, u32, vp, vp, vp, vp, u32]
    L.rdp_batch_idle.argtypes = [vp]
    L.rdp_batch_get_stats.argtypes = [vp, ctypes.POINTER(_BatchStats)]
    L.rdp_batch_capture_begin.argtypes = [vp]
    L.rdp_batch_capture_end.argtypes = [vp, ctypes.POINTER(vp)]
    _lib = L
    return L


SHADE_VARIANTS = 8


def set_shade_variant(variant, device=0):
    """Forces the shading-kernel variant (0..7) of a device, or restarts autotuning (-1)."""
    _check(lib().rdp_set_shade_variant(device, variant), "set_shade_variant")


def get_shade_variant(device=0):
    """The device's shading-kernel variant; -1 while the autotuner is still timing them."""
    return lib().rdp_get_shade_variant(device)


SHADE_ORDERS = {"strided": 0, "sm_queues": 1, "primitive_major": 2}


def set_shade_order(order, device=0):
    """How the shading kernel takes a launch's pairs: 0 = tile order, fixed stride per CTA;
    1 = tile order through per-SM work queues; 2 (default) = primitive-major order through the
    queues.  Small launches take the next simpler order (thresholds: RDP_SHADE_PERM_MIN_PRIMS,
    RDP_SHADE_QUEUE_MIN, read when a processor or batch is created)."""
    _check(lib().rdp_set_shade_order(device, order), "set_shade_order")


def get_shade_order(device=0):
    return lib().rdp_get_shade_order(device)


MLP_PARAMS = 5313
MLP_IN = 16


def mlp_gradients(params, features, targets, device=0):
    """GPU loss gradients of the tile-cost model (the scheduler's own kernels); (grads, loss)."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(features, dtype=np.float32)
    y = np.ascontiguousarray(targets, dtype=np.float32)
    assert p.size == MLP_PARAMS and x.shape == (y.size, MLP_IN)
    g = np.zeros(MLP_PARAMS, dtype=np.float32)
    loss = ctypes.c_float()
    _check(lib().rdp_mlp_gradients(device, p.ctypes.data, x.ctypes.data, y.ctypes.data, y.size, g.ctypes.data,
                                   ctypes.byref(loss)), "mlp_gradients")
    return g, loss.value


def mlp_forward(params, features, device=0):
    p = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(features, dtype=np.float32)
    out = np.zeros(x.shape[0], dtype=np.float32)
    _check(lib().rdp_mlp_forward(device, p.ctypes.data, x.ctypes.data, x.shape[0], out.ctypes.data), "mlp_forward")
    return out


def device_is_supported(device=0):
    return bool(lib().rdp_device_is_supported(device))


def _check(code, what):
    if code == RDP_ERR_TIMEOUT:
        raise RdpTimeout(code, what)
    if code != RDP_OK:
        raise RdpError(code, what)


class CommandProcessor:
    """RDP::CommandProcessor over librdp_cuda (rdp_device.hpp:111-197).

    `rdram` is a caller-owned numpy uint8 array (RDRAM as host-order 32-bit
    words, N64 byte address a at index a ^ 3), or None to let the processor own
    a zero-initialised one.
    """

    def __init__(self, rdram=None, rdram_size=8 << 20, hidden_rdram_size=None, device=0, batch=None,
                 command_thread=False, upscaling=1, super_sampled_readback=False, super_sampled_dither=False):
        """upscaling: internal upscaling factor 1, 2, 4 or 8 (COMMAND_PROCESSOR_FLAG_UPSCALING_*_BIT);
        super_sampled_readback / super_sampled_dither: resolve the scaled rendering into RDRAM."""
        if hidden_rdram_size is None:
            hidden_rdram_size = rdram_size // 2
        if rdram is None:
            rdram = np.zeros(rdram_size, dtype=np.uint8)
        assert rdram.dtype == np.uint8 and rdram.flags["C_CONTIGUOUS"] and rdram.size >= rdram_size
        self._rdram = rdram
        self._batch = batch
        if upscaling not in _UPSCALING_FLAGS:
            raise ValueError("upscaling must be 1, 2, 4 or 8")
        flags = (CREATE_COMMAND_THREAD if command_thread else 0) | _UPSCALING_FLAGS[upscaling]
        flags |= (CREATE_SUPER_SAMPLED_READ_BACK if super_sampled_readback else 0)
        flags |= (CREATE_SUPER_SAMPLED_DITHER if super_sampled_dither else 0)
        info = _CreateInfo(rdram.ctypes.data, 0, rdram_size, hidden_rdram_size, flags, device)
        h = ctypes.c_void_p()
        if batch is None:
            _check(lib().rdp_cp_create(ctypes.byref(info), ctypes.byref(h)), "rdp_cp_create")
        else:
            _check(lib().rdp_batch_add_instance(batch._h, ctypes.byref(info), ctypes.byref(h)),
                   "rdp_batch_add_instance")
        self._h = h
        self.rdram_size = rdram_size
        self.hidden_rdram_size = hidden_rdram_size
        self._cb = None

    def close(self):
        if getattr(self, "_h", None):
            lib().rdp_cp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- command stream ---------------------------------------------------
    def enqueue_command(self, words):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        _check(lib().rdp_cp_enqueue(self._h, w.size, w.ctypes.data), "enqueue_command")

    def signal_timeline(self):
        v = ctypes.c_uint64()
        _check(lib().rdp_cp_signal_timeline(self._h, ctypes.byref(v)), "signal_timeline")
        return v.value

    def wait_for_timeline(self, value, timeout_s=30.0):
        _check(lib().rdp_cp_wait_timeline(self._h, value, int(timeout_s * 1e9)), "wait_for_timeline")

    def flush(self):
        _check(lib().rdp_cp_flush(self._h), "flush")

    def idle(self):
        _check(lib().rdp_cp_idle(self._h), "idle")

    def begin_frame_context(self):
        _check(lib().rdp_cp_begin_frame_context(self._h), "begin_frame_context")

    def set_quirks(self, quirks_word):
        _check(lib().rdp_cp_set_quirks(self._h, quirks_word), "set_quirks")

    def set_validation_interface(self, fn):
        """fn(error_code, message) is called for illegal RDP state (rdp_renderer.hpp:75-95)."""
        if fn is None:
            self._cb = None
            _check(lib().rdp_cp_set_validation_callback(self._h, _VALIDATION_CB(), None), "set_validation")
            return
        self._cb = _VALIDATION_CB(lambda user, err, msg: fn(err, msg.decode()))
        _check(lib().rdp_cp_set_validation_callback(self._h, self._cb, None), "set_validation")

    # -- memory -----------------------------------------------------------
    def begin_read_rdram(self):
        p = lib().rdp_cp_begin_read_rdram(self._h)
        if not p:
            raise RdpError(RDP_ERR_DEVICE, "begin_read_rdram")
        return self._rdram[:self.rdram_size]

    def end_write_rdram(self):
        _check(lib().rdp_cp_end_write_rdram(self._h), "end_write_rdram")

    def begin_read_hidden_rdram(self):
        p = lib().rdp_cp_begin_read_hidden_rdram(self._h)
        if not p:
            raise RdpError(RDP_ERR_DEVICE, "begin_read_hidden_rdram")
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)),
                                     shape=(self.hidden_rdram_size,)).copy()

    def get_tmem(self):
        out = np.zeros(2048, dtype=np.uint16)
        _check(lib().rdp_cp_get_tmem(self._h, out.ctypes.data), "get_tmem")
        return out

    # -- internal upscaling -------------------------------------------------
    def get_scaling_factor(self):
        return lib().rdp_cp_get_scaling_factor(self._h)

    def upscaled_rdram(self):
        """The multisampled RDRAM: factor^2 slices of RDRAM, slice (y % f) * f + x % f."""
        f = self.get_scaling_factor()
        out = np.zeros(self.rdram_size * f * f, dtype=np.uint8)
        _check(lib().rdp_cp_read_upscaled_rdram(self._h, out.ctypes.data, 0, out.size), "read_upscaled_rdram")
        return out

    def upscaled_hidden_rdram(self):
        f = self.get_scaling_factor()
        out = np.zeros(self.hidden_rdram_size * f * f, dtype=np.uint8)
        _check(lib().rdp_cp_read_upscaled_hidden_rdram(self._h, out.ctypes.data, 0, out.size),
               "read_upscaled_hidden_rdram")
        return out

    # -- video interface ----------------------------------------------------
    def set_vi_register(self, reg, value):
        _check(lib().rdp_cp_set_vi_register(self._h, int(reg), value & 0xffffffff), "set_vi_register")

    def scanout_sync(self, options=None, **kw):
        """Returns the RGBA8 scanout as uint32[h, w] (r | g << 8 | b << 16 | a << 24), or None."""
        opts = options if options is not None else ScanoutOptions(**kw)
        f = self.get_scaling_factor()
        buf = np.zeros(640 * 576 * f * f, dtype=np.uint32)
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        _check(lib().rdp_cp_scanout_sync(self._h, ctypes.byref(opts), buf.ctypes.data, ctypes.byref(w),
                                         ctypes.byref(h)), "scanout_sync")
        return buf[:w.value * h.value].reshape(h.value, w.value) if w.value else None

    def capture(self, words):
        """Records the passes of `words` into a CUDA graph (inputs resident in HBM)."""
        _check(lib().rdp_cp_capture_begin(self._h), "capture_begin")
        self.enqueue_command(words)
        g = ctypes.c_void_p()
        _check(lib().rdp_cp_capture_end(self._h, ctypes.byref(g)), "capture_end")
        return Graph(g)

    def begin_vi_register_per_scanline(self, flags):
        _check(lib().rdp_cp_begin_vi_register_per_scanline(self._h, flags), "begin_vi_register_per_scanline")

    def set_vi_register_for_scanline(self, reg_bit, value):
        _check(lib().rdp_cp_set_vi_register_for_scanline(self._h, reg_bit, value & 0xffffffff), "set_for_scanline")

    def latch_vi_register_for_scanline(self, line):
        _check(lib().rdp_cp_latch_vi_register_for_scanline(self._h, line), "latch_for_scanline")

    def end_vi_register_per_scanline(self):
        _check(lib().rdp_cp_end_vi_register_per_scanline(self._h), "end_vi_register_per_scanline")

    def write_hidden_rdram(self, data):
        """Replaces hidden RDRAM (begin_read_hidden_rdram + end_write_hidden_rdram)."""
        p = lib().rdp_cp_begin_read_hidden_rdram(self._h)
        if not p:
            raise RdpError(RDP_ERR_DEVICE, "begin_read_hidden_rdram")
        d = np.ascontiguousarray(data, dtype=np.uint8)[:self.hidden_rdram_size]
        ctypes.memmove(p, d.ctypes.data, d.size)
        _check(lib().rdp_cp_end_write_hidden_rdram(self._h), "end_write_hidden_rdram")

    def write_rdram(self, data):
        """Replaces RDRAM contents in the caller-owned buffer and uploads it (end_write_rdram)."""
        self.idle()
        self._rdram[:self.rdram_size] = np.ascontiguousarray(data, dtype=np.uint8)[:self.rdram_size]
        self.end_write_rdram()

    def stats(self):
        s = _Stats()
        _check(lib().rdp_cp_get_stats(self._h, ctypes.byref(s)), "get_stats")
        return {k: getattr(s, k) for k, _ in _Stats._fields_}


class Graph:
    """A captured sync point (rdp_cp_capture_*): replay with inputs resident in HBM."""

    def __init__(self, handle):
        self._h = handle
        self.kernels = lib().rdp_graph_kernel_count(handle)
        self.shade_launches = lib().rdp_graph_shade_launches(handle)

    def replay(self, count=1):
        ms = ctypes.c_float()
        _check(lib().rdp_graph_replay(self._h, count, ctypes.byref(ms)), "graph_replay")
        return ms.value

    def last_shade_ms(self):
        return lib().rdp_graph_last_shade_ms(self._h)

    def last_blend_ms(self):
        return lib().rdp_graph_last_blend_ms(self._h)

    def close(self):
        if self._h:
            lib().rdp_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Batch:
    """Many emulator instances rendered together (rdp_batch_*): every instance is a
    CommandProcessor whose passes are deferred; submit() launches one kernel chain
    per round of at most one pass per instance."""

    def __init__(self, device=0, learned_order=False, record_tile_cycles=False):
        flags = (BATCH_TILE_ORDER_LEARNED if learned_order else 0) | (BATCH_RECORD_TILE_CYCLES if record_tile_cycles else 0)
        info = _BatchCreateInfo(device, flags)
        h = ctypes.c_void_p()
        _check(lib().rdp_batch_create(ctypes.byref(info), ctypes.byref(h)), "rdp_batch_create")
        self._h = h
        self.device = device
        self._instances = []

    def add_instance(self, rdram=None, rdram_size=8 << 20, hidden_rdram_size=None):
        cp = CommandProcessor(rdram, rdram_size, hidden_rdram_size, self.device, batch=self)
        self._instances.append(cp)
        return cp

    def submit(self):
        _check(lib().rdp_batch_submit(self._h), "batch_submit")

    def enqueue_many(self, instances, words_list, signal=True, threads=0):
        """Enqueues words_list[i] to instances[i] on host threads; returns timeline values when signal."""
        n = len(instances)
        arrs = [np.ascontiguousarray(w, dtype=np.uint32) for w in words_list]
        handles = (ctypes.c_void_p * n)(*[cp._h.value for cp in instances])
        ptrs = (ctypes.c_void_p * n)(*[a.ctypes.data for a in arrs])
        counts = (ctypes.c_uint32 * n)(*[a.size for a in arrs])
        values = (ctypes.c_uint64 * n)() if signal else None
        _check(lib().rdp_batch_enqueue_many(self._h, n, handles, ptrs, counts, values, threads), "batch_enqueue_many")
        return list(values) if signal else None

    def set_schedule(self, learned_order, train=False, learning_rate=1e-3, train_stride=1):
        """Learned tile order on/off; online training of the tile-cost model on/off."""
        _check(lib().rdp_batch_set_schedule(self._h, int(learned_order), int(train), learning_rate, train_stride),
               "batch_set_schedule")

    def get_model(self):
        """(FP32 parameters of the tile-cost model, mean squared error of the last training step)."""
        p = np.zeros(MLP_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        _check(lib().rdp_batch_get_model(self._h, p.ctypes.data, ctypes.byref(loss)), "batch_get_model")
        return p, loss.value

    def tile_samples(self, max_tiles=1 << 22, features=True, predicted=True, cycles=True):
        """The last launch's non-empty tiles: dict of features [n,16], predicted [n], cycles [n]."""
        f = np.zeros((max_tiles, MLP_IN), dtype=np.float32) if features else None
        p = np.zeros(max_tiles, dtype=np.float32) if predicted else None
        c = np.zeros(max_tiles, dtype=np.uint32) if cycles else None
        n = ctypes.c_uint32()
        _check(lib().rdp_batch_get_tile_samples(self._h, f.ctypes.data if f is not None else None,
                                                p.ctypes.data if p is not None else None,
                                                c.ctypes.data if c is not None else None, max_tiles, ctypes.byref(n)),
               "batch_get_tile_samples")
        k = n.value
        return {"features": f[:k] if f is not None else None, "predicted": p[:k] if p is not None else None,
                "cycles": c[:k] if c is not None else None}

    def serve(self, instances, requests, hbm_budget_bytes=16 << 30, max_in_flight=0, timeout_s=600.0):
        """Runs a request trace through the serving loop (rdp_serve_run).

        instances: CommandProcessors of this batch; requests: sequence of
        (instance index, words uint32 array, arrival seconds), sorted by arrival.
        Returns (dict of numpy arrays admit_s / done_s / latency_s, stats dict)."""
        n = len(requests)
        reqs = (_ServeRequest * max(n, 1))()
        keep = []
        for i, (inst, words, arrival) in enumerate(requests):
            w = np.ascontiguousarray(words, dtype=np.uint32)
            keep.append(w)
            reqs[i] = _ServeRequest(int(inst), w.size, w.ctypes.data, float(arrival), 0)
        handles = (ctypes.c_void_p * len(instances))(*[cp._h.value for cp in instances])
        res = (_ServeResult * max(n, 1))()
        st = _ServeStats()
        cfg = _ServeConfig(int(hbm_budget_bytes), int(max_in_flight), float(timeout_s))
        _check(lib().rdp_serve_run(self._h, handles, len(instances), reqs, n, ctypes.byref(cfg), res, ctypes.byref(st)),
               "serve_run")
        out = {k: np.array([getattr(res[i], k) for i in range(n)]) for k in ("admit_s", "done_s", "latency_s")}
        return out, {k: getattr(st, k) for k, _ in _ServeStats._fields_}

    def set_model(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(lib().rdp_batch_set_model(self._h, p.ctypes.data), "batch_set_model")

    def idle(self):
        _check(lib().rdp_batch_idle(self._h), "batch_idle")

    def stats(self):
        s = _BatchStats()
        _check(lib().rdp_batch_get_stats(self._h, ctypes.byref(s)), "batch_get_stats")
        return {k: getattr(s, k) for k, _ in _BatchStats._fields_}

    def capture(self, per_instance_words):
        """Records one sync point of every instance (words[i] for instance i) into a CUDA graph."""
        _check(lib().rdp_batch_capture_begin(self._h), "batch_capture_begin")
        for cp, w in zip(self._instances, per_instance_words):
            cp.enqueue_command(w)
        g = ctypes.c_void_p()
        _check(lib().rdp_batch_capture_end(self._h, ctypes.byref(g)), "batch_capture_end")
        return Graph(g)

    def close(self):
        if getattr(self, "_h", None):
            for cp in self._instances:
                cp.close()
            self._instances = []
            lib().rdp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
