"""RDPDUMP2 capture files (the reference's format, parallel-rdp/rdp_dump_write.cpp and
rdp_dump.cpp): a Python writer / reader for tooling and tests, and the native replayer
(rdp_dump_replay) that plays a file into a CommandProcessor."""
import ctypes
import struct

import numpy as np

UPDATE_DRAM, RDP_COMMAND, SET_VI_REGISTER, END_FRAME, SIGNAL_COMPLETE, EOF, UPDATE_DRAM_FLUSH, \
    UPDATE_HIDDEN_DRAM, UPDATE_HIDDEN_DRAM_FLUSH = range(1, 10)
BLOCK = 4096


def command_length(op):
    """Words of an RDP command (rdp_common.hpp command sizes)."""
    return {0x08: 8, 0x09: 12, 0x0a: 24, 0x0b: 28, 0x0c: 24, 0x0d: 28, 0x0e: 40, 0x0f: 44,
            0x24: 4, 0x25: 4}.get(op, 2)


def split_commands(words):
    """Yields (op, words) for each whole command of a word stream."""
    w = np.asarray(words, dtype=np.uint32)
    i = 0
    while i < w.size:
        op = int(w[i] >> 24) & 63
        n = command_length(op)
        if i + n > w.size:
            break
        yield op, w[i:i + n]
        i += n


class DumpWriter:
    """Mirrors RDP::RDPDumpWriter: flushes emit only the 4 KiB blocks that changed."""

    def __init__(self, path, rdram_size=8 << 20, hidden_size=4 << 20):
        self.f = open(path, "wb")
        self.f.write(b"RDPDUMP2" + struct.pack("<II", rdram_size, hidden_size))
        self.dram = np.zeros(rdram_size, np.uint8)
        self.hidden = np.zeros(hidden_size, np.uint8)

    def _w(self, *vals):
        self.f.write(struct.pack("<%dI" % len(vals), *vals))

    def _flush(self, data, cache, block_cmd, flush_cmd):
        data = np.ascontiguousarray(data, dtype=np.uint8)[:cache.size]
        for off in range(0, data.size, BLOCK):
            blk = data[off:off + BLOCK]
            if not np.array_equal(blk, cache[off:off + blk.size]):
                self._w(block_cmd, off, blk.size)
                self.f.write(blk.tobytes())
                cache[off:off + blk.size] = blk
        self._w(flush_cmd)

    def flush_dram(self, rdram):
        self._flush(rdram, self.dram, UPDATE_DRAM, UPDATE_DRAM_FLUSH)

    def flush_hidden_dram(self, hidden):
        self._flush(hidden, self.hidden, UPDATE_HIDDEN_DRAM, UPDATE_HIDDEN_DRAM_FLUSH)

    def command(self, op, words):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        self._w(RDP_COMMAND, op, w.size)
        self.f.write(w.tobytes())

    def commands(self, words):
        for op, w in split_commands(words):
            self.command(op, w)

    def set_vi_register(self, reg, value):
        self._w(SET_VI_REGISTER, int(reg), value & 0xffffffff)

    def end_frame(self):
        self._w(END_FRAME)

    def signal_complete(self):
        self._w(SIGNAL_COMPLETE)

    def close(self):
        if self.f:
            self._w(EOF)
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_dump(path):
    """Yields (kind, payload) records; block records are applied to caches and the flush
    records carry the full cache: ("rdram", bytes), ("hidden", bytes), ("command", (op, words)),
    ("vi", (reg, value)), ("end_frame", None), ("signal_complete", None)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"RDPDUMP2":
        raise ValueError("not an RDPDUMP2 file")
    dram_size, hidden_size = struct.unpack_from("<II", data, 8)
    dram = np.zeros(dram_size, np.uint8)
    hidden = np.zeros(hidden_size, np.uint8)
    pos = 16

    def u32():
        nonlocal pos
        v = struct.unpack_from("<I", data, pos)[0]
        pos += 4
        return v

    while pos < len(data):
        c = u32()
        if c == EOF:
            return
        if c in (UPDATE_DRAM, UPDATE_HIDDEN_DRAM):
            off, n = u32(), u32()
            dst = dram if c == UPDATE_DRAM else hidden
            dst[off:off + n] = np.frombuffer(data, np.uint8, n, pos)
            pos += n
        elif c == UPDATE_DRAM_FLUSH:
            yield "rdram", dram.copy()
        elif c == UPDATE_HIDDEN_DRAM_FLUSH:
            yield "hidden", hidden.copy()
        elif c == RDP_COMMAND:
            op, n = u32(), u32()
            words = np.frombuffer(data, np.uint32, n, pos).copy()
            pos += 4 * n
            yield "command", (op, words)
        elif c == SET_VI_REGISTER:
            reg, v = u32(), u32()
            yield "vi", (reg, v)
        elif c == END_FRAME:
            yield "end_frame", None
        elif c == SIGNAL_COMPLETE:
            yield "signal_complete", None
        else:
            raise ValueError("unknown RDPDUMP2 record %d at %d" % (c, pos - 4))


_FRAME_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32,
                             ctypes.c_uint32)


def replay(cp, path):
    """Plays an RDPDUMP2 file into CommandProcessor `cp` (rdp_dump_replay); returns the list of
    scanout images (uint32 [h, w], r | g << 8 | b << 16 | a << 24), one per end-of-frame record."""
    from .native import _check, lib
    L = lib()
    if not getattr(L, "_dump_bound", False):
        L.rdp_dump_replay.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _FRAME_CB, ctypes.c_void_p,
                                      ctypes.POINTER(ctypes.c_uint32)]
        L._dump_bound = True
    frames = []

    def on_frame(user, index, rgba, w, h):
        frames.append(np.ctypeslib.as_array(rgba, shape=(w * h,)).copy().reshape(h, w) if w else None)

    cb = _FRAME_CB(on_frame)
    n = ctypes.c_uint32()
    _check(L.rdp_dump_replay(cp._h, str(path).encode(), cb, None, ctypes.byref(n)), "dump_replay")
    return frames
