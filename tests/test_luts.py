"""Hardware tables against the reference's luts.hpp (read as text when the
reference tree is present; skipped otherwise) and against committed checksums."""
import hashlib
import os
import re

import numpy as np
import pytest

# The reference tree's luts.hpp, when a copy of the reference is present (RDP_REFERENCE_DIR, the
# directory that holds parallel-rdp/); the checksum tests below run either way.
REF_LUTS = os.path.join(os.environ.get("RDP_REFERENCE_DIR", "/nonexistent"), "parallel-rdp", "luts.hpp")
# sha256 of the 32 KiB blender divider table and of the 16,640-entry gamma table.
BLENDER_SHA256 = "8072c219888f51694d2cd13cef8e83db02f0a41c0be3ba039415c79374634a3d"
GAMMA_SHA256 = "4879d9c57ad78e61759e10546fa8bba2bad70bcae1dd5b34b2d4c7b17a8c18a4"


def _oracle_blender():
    from oracle import Oracle
    o = Oracle(1 << 20)
    lut = np.zeros(0x8000, np.uint8)
    o.L.oracle_blender_lut(o.h, lut.ctypes.data)
    return lut


def gamma_table():
    """VI gamma table regenerated from its closed form: isqrt(4 * v) & ~1 over the
    14-bit (value << 6 | dither) index; the first 256 entries are the undithered
    table (the reference stores both, luts.hpp:1034)."""
    import math
    g = [math.isqrt(i * 256) & ~1 for i in range(256)]
    g += [math.isqrt(i * 4) & ~1 for i in range(256 * 64)]
    return np.array(g, np.uint8)


def _ref_table(name):
    src = open(REF_LUTS).read()
    m = re.search(name + r"\[[^\]]*\]\s*=\s*\{(.*?)\};", src, re.S)
    return np.array([int(x) for x in re.findall(r"\d+", m.group(1))], np.uint8)


def test_blender_divider_checksum():
    assert hashlib.sha256(_oracle_blender().tobytes()).hexdigest() == BLENDER_SHA256


def test_gamma_checksum():
    assert hashlib.sha256(gamma_table().tobytes()).hexdigest() == GAMMA_SHA256


@pytest.mark.skipif(not os.path.exists(REF_LUTS), reason="reference tree not present")
def test_blender_divider_matches_reference():
    assert np.array_equal(_oracle_blender(), _ref_table("blender_lut"))


@pytest.mark.skipif(not os.path.exists(REF_LUTS), reason="reference tree not present")
def test_gamma_matches_reference():
    assert np.array_equal(gamma_table(), _ref_table("gamma_table"))
