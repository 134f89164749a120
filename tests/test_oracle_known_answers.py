"""Known-answer checks that pin the oracle's fixed-point primitives.

The reference ships no golden images (its oracle, Angrylion-Plus, is an empty
submodule), so these hand-derived answers -- taken from the ranges and
identities the reference documents in its shader sources -- pin the oracle.
"""
import ctypes

import numpy as np
import pytest

from oracle import lib


def test_z_decompress_endpoints():
    L = lib()
    assert L.oracle_z_decompress(0) == 0
    assert L.oracle_z_decompress(0x3fff) == 0x3ffff  # exponent 7, full mantissa
    assert L.oracle_z_compress(0x3ffff) == 0x3fff
    assert L.oracle_z_compress(0) == 0


def test_z_compress_inverts_decompress():
    # Every 14-bit compressed depth decompresses to an 18-bit value that compresses back to itself
    # (z_encode.h:28-46).
    L = lib()
    for c in range(0, 0x4000, 7):
        assert L.oracle_z_compress(L.oracle_z_decompress(c)) == c


def test_z_compress_monotonic():
    L = lib()
    prev = -1
    for z in range(0, 0x40000, 97):
        c = L.oracle_z_compress(z)
        assert c >= prev
        prev = c


def test_dz_compress_is_log2_of_powers_of_two():
    # rdp_renderer.cpp:728-740: the bit-OR tree yields log2 for powers of two.
    L = lib()
    for k in range(16):
        assert L.oracle_dz_compress(1 << k) == k


@pytest.mark.parametrize("v,expected", [(0, 0), (255, 255), (128, 128), (-1, 0), (-128, 0), (-129, 0xff),
                                        (-256, 0xff), (256, 0xff), (383, 0xff), (384, 0), (511, 0)])
def test_clamp_9bit_ranges(v, expected):
    # clamping.h:42-45: [-128,-1] -> 0, [-256,-129] -> 0xff, 9-bit wrap above.
    assert lib().oracle_clamp_9bit(v) == expected


@pytest.mark.parametrize("v,expected", [(0, 0), (0x3ffff, 0x3ffff), (0x1234, 0x1234), (0x40000, 0x3ffff),
                                        (0x5ffff, 0x3ffff), (0x60000, 0), (0x7ffff, 0)])
def test_clamp_z_ranges(v, expected):
    # clamping.h:71-73.
    assert lib().oracle_clamp_z(v) == expected


def _persp(s, t, w):
    out = (ctypes.c_int * 2)()
    ov = ctypes.c_int()
    lib().oracle_perspective_divide(s, t, w, out, ctypes.byref(ov))
    return out[0], out[1], ov.value


def test_perspective_divide_unit_w():
    # w = 0x7fff (1.0 in s1.15): the LUT reciprocal is exactly 0x2000, so s/w == s.
    assert _persp(256, -100, 0x7fff) == (256, -100, 0)


def test_perspective_divide_half_w():
    # w = 0x4000 (0.5): reciprocal 0x4000, result doubles.
    assert _persp(256, 40, 0x4000) == (512, 80, 0)


def test_perspective_divide_nonpositive_w_saturates():
    s, t, ov = _persp(10, 10, 0)
    assert (s, t, ov) == (0x7fff, 0x7fff, 1)


def _noise_py(x, y, p):
    # noise.h:29-37, restated independently.
    P = 1103515245
    m = 0xffffffff
    s = [x & m, y & m, p & m]
    for _ in range(3):
        s = [(((s[0] >> 8) ^ s[1]) * P) & m, (((s[1] >> 8) ^ s[2]) * P) & m, (((s[2] >> 8) ^ s[0]) * P) & m]
    return s[0] >> 16


@pytest.mark.parametrize("x,y,p", [(0, 0, 0), (1, 2, 3), (319, 239, 1999), (1023 + 5, 7 + 9, 11 + 123456)])
def test_noise_hash_matches_independent_restatement(x, y, p):
    assert lib().oracle_noise(x, y, p) == _noise_py(x, y, p)


def test_blender_divider_regular_rows():
    # Rows 1..8 below the 8-bit overflow are plain integer division (blender.h:124-136).
    from oracle import Oracle
    o = Oracle(1 << 20)
    lut = np.zeros(0x8000, np.uint8)
    o.L.oracle_blender_lut(o.h, lut.ctypes.data)
    lut = lut.reshape(16, 2048)
    for d in range(1, 9):
        n = np.arange(min(2048, 256 * d))
        assert np.array_equal(lut[d][n], n // d)
    assert not lut[0].any()
