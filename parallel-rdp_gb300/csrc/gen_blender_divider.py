"""Generate blender_divider_runs.inc from the reference's luts.hpp.

The RDP blender divider (used by the final blender cycle when force-blend is
off) is hardware behaviour captured as a 16 x 2048 table in the reference
(parallel-rdp/luts.hpp:7, indexed as (blend_sum << 11) | blended, see
parallel-rdp/shaders/blender.h:124-136).  Rows whose entries follow
floor(n / d) & 0xff are regenerated by formula at run time (build_blender_lut in
rdp_cp.cpp, and the oracle's own table builder); only the entries that deviate
from that formula are stored, as (row, start, length, value) runs.

Usage: python gen_blender_divider.py <path-to-luts.hpp> > blender_divider_runs.inc
"""
import re
import sys


def main():
    src = open(sys.argv[1]).read()
    m = re.search(r'blender_lut\[[^\]]*\]\s*=\s*\{(.*?)\};', src, re.S)
    vals = [int(x) for x in re.findall(r'\d+', m.group(1))]
    assert len(vals) == 0x8000
    runs = []
    for d in range(16):
        row = vals[d * 2048:(d + 1) * 2048]
        base = [((n // d) & 0xff) if d else 0 for n in range(2048)]
        i = 0
        while i < 2048:
            if row[i] == base[i]:
                i += 1
                continue
            j = i
            while j < 2048 and row[j] != base[j] and row[j] == row[i]:
                j += 1
            runs.append((d, i, j - i, row[i]))
            i = j
    print("/* Generated by gen_blender_divider.py: entries of the RDP blender divider")
    print(" * table that differ from floor(n / d) & 0xff, as {row, start, length, value}. */")
    print("#define RDP_BLENDER_DIVIDER_NUM_RUNS %d" % len(runs))
    print("static const unsigned short rdp_blender_divider_runs[RDP_BLENDER_DIVIDER_NUM_RUNS][4] = {")
    line = []
    for r in runs:
        line.append("{%d,%d,%d,%d}" % r)
        if len(line) == 8:
            print("\t" + ",".join(line) + ",")
            line = []
    if line:
        print("\t" + ",".join(line) + ",")
    print("};")


if __name__ == "__main__":
    main()
