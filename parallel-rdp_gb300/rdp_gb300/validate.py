"""Dump validation (the reference's rdp-validate-dump, rdp_validate_dump.cpp): an RDPDUMP2 capture is
played into two renderers side by side, and after every draw command -- or, with sync_only, every
SyncFull -- their TMEM, RDRAM and hidden RDRAM must be identical.  The first difference is reported
with its frame, its draw (or sync) number, its address and, when it lies in the current colour or
depth image, its pixel coordinate.

A renderer is any object with enqueue(words), idle(), rdram(), hidden(), tmem(), write_rdram(bytes)
and write_hidden(bytes).  GpuTarget adapts a CommandProcessor; a CPU renderer with the same methods
(for example the project's CPU oracle) serves as the other side.
"""
import numpy as np

from .dump import read_dump, split_commands

DRAW_OPS = frozenset(list(range(0x08, 0x10)) + [0x24, 0x25, 0x36])
SYNC_FULL = 0x29


class GpuTarget:
    """A CommandProcessor as one side of the validation."""

    def __init__(self, cp):
        self.cp = cp

    def enqueue(self, words):
        self.cp.enqueue_command(words)

    def idle(self):
        self.cp.idle()

    def rdram(self):
        return self.cp.begin_read_rdram()

    def hidden(self):
        return self.cp.begin_read_hidden_rdram()

    def tmem(self):
        return self.cp.get_tmem()

    def write_rdram(self, data):
        self.cp.write_rdram(data)

    def write_hidden(self, data):
        self.cp.write_hidden_rdram(data)


def _first_difference(a, b):
    a = np.asarray(a).view(np.uint8).reshape(-1)
    b = np.asarray(b).view(np.uint8).reshape(-1)
    n = min(a.size, b.size)
    d = np.nonzero(a[:n] != b[:n])[0]
    if d.size:
        return int(d[0])
    return None if a.size == b.size else n


def _coordinate(fb, addr, hidden):
    """The pixel of the colour or depth image that byte `addr` belongs to (rdp_validate_dump.cpp:
    140-186): hidden RDRAM bytes stand for 16-bit halfwords."""
    if not fb["width"]:
        return None
    if hidden:
        addr *= 2
    color = addr - fb["addr"]
    depth = (addr - fb["depth_addr"]) >> 1
    color >>= {2: 1, 3: 2}.get(fb["size"], 0)
    w = fb["width"]
    if color >= 0 and (color <= depth or depth < 0):
        return {"image": "color", "x": color % w, "y": color // w, "hidden": hidden}
    if depth >= 0:
        return {"image": "depth", "x": depth % w, "y": depth // w, "hidden": hidden}
    return None


def validate_dump(path, reference, candidate, sync_only=False, begin_frame=0, max_checks=None):
    """Plays the dump at `path` into both renderers and compares them after every draw (or every
    SyncFull with sync_only) from frame `begin_frame` on.  Returns a report:
    {"passed", "frames", "checks", "failure": None or {"frame", "draw" or "sync", "memory",
    "address", "coordinate"}}."""
    frame = draws = syncs = checks = 0
    fb = {"addr": 0, "width": 0, "size": 0, "depth_addr": 0}

    def compare(kind):
        nonlocal checks
        reference.idle()
        candidate.idle()
        checks += 1
        where = {"frame": frame, kind: draws if kind == "draw" else syncs}
        for name, get, hidden in (("TMEM", lambda r: r.tmem(), False), ("RDRAM", lambda r: r.rdram(), False),
                                  ("hidden RDRAM", lambda r: r.hidden(), True)):
            at = _first_difference(get(reference), get(candidate))
            if at is not None:
                where.update(memory=name, address=at,
                             coordinate=None if name == "TMEM" else _coordinate(fb, at, hidden))
                return where
        return None

    for kind, payload in read_dump(path):
        if kind == "rdram":
            reference.write_rdram(payload)
            candidate.write_rdram(payload)
        elif kind == "hidden":
            reference.write_hidden(payload)
            candidate.write_hidden(payload)
        elif kind == "command":
            op, words = payload
            for cop, w in split_commands(words):
                reference.enqueue(w)
                candidate.enqueue(w)
                if cop == 0x3f:
                    fb.update(addr=int(w[1]) & 0xffffff, width=(int(w[0]) & 0x3ff) + 1, size=(int(w[0]) >> 19) & 3)
                elif cop == 0x3e:
                    fb["depth_addr"] = int(w[1]) & 0xffffff
                check = None
                if cop in DRAW_OPS:
                    draws += 1
                    if not sync_only and frame >= begin_frame:
                        check = "draw"
                elif cop == SYNC_FULL:
                    syncs += 1
                    if sync_only and frame >= begin_frame:
                        check = "sync"
                if check:
                    failure = compare(check)
                    if failure:
                        return {"passed": False, "frames": frame, "checks": checks, "failure": failure}
                    if max_checks is not None and checks >= max_checks:
                        return {"passed": True, "frames": frame, "checks": checks, "failure": None}
        elif kind == "end_frame":
            frame += 1
    return {"passed": True, "frames": frame, "checks": checks, "failure": None}
