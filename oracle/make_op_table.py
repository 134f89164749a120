"""Integer-op table of the RDP path, from instrumented counters of the CPU oracle (test
infrastructure: the product never reads this script; bench.py reads its output as data).

What it measures.  The oracle (rdp_oracle.cpp) restates the reference's per-stage functions
(shading.h, coverage.h, interpolation.h, perspective.h, texture.h, combiner.h, depth_test.h,
blender.h, memory_interfacing.h, span_setup.comp, binning.h, tmem_update.comp, and the host-side
decode / set-up of rdp_device.cpp and rdp_renderer.cpp).  This script builds a second copy of it
with GCC at -O1 without inlining, with line-execution counters (gcov) and the final GIMPLE dump with
source lines.  For every source line it counts the integer / logic operations of that line's
GIMPLE statements -- add, subtract, multiply, divide, shift, rotate, and / or / xor / not, negate,
compare, min / max / abs, select (?:), bit-count builtins, and the compare of a branch or switch;
not loads, stores, copies or width casts -- and multiplies by how often the line ran.  A function's
dynamic ops are the sum over its lines; a stage's are the sum over its functions.

  K(stage)   = ops(stage) / units(stage), units = calls of the stage's unit function
  OPS(step)  = sum over stages of units(stage) * K(stage)   (= sum of ops(stage))

Approximations, stated: counts are per source line, so a line whose operations sit on both arms of
a branch counts both arms every time it runs (K is an upper estimate for such lines); the oracle's
own bookkeeping (its per-pixel loop over binned tiles, pixel cache, pass counting, RDRAM helpers
that only mask an address) is kept out by listing the stages' functions explicitly.

Workloads (the benchmark's, regenerated from their seeds):
  batched64 -- one frame of each of the 64 batched instances (seeds 0-63), one sync point
  plain     -- the plain 320x240 frame (2,000 Gouraud triangles, seed 0)
  textured  -- the textured, depth-tested 320x240 frame (10,000 triangles, seed 0)
  mixed16   -- the mixed 640x480 sequence (16 frames of 50,000 primitives, seed 0), one step

Usage: python oracle/make_op_table.py [--jobs N]   -> writes oracle/op_table.json
"""
import argparse
import glob
import json
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "opcount")
LIB = os.path.join(OUT, "liboracle_opcount.so")

# Stage -> (unit function, unit name, member functions of the oracle's Oracle struct).
STAGES = {
    "command decode": ("command", "commands",
                       ["command", "set_other_modes", "set_combine", "set_tile", "rect", "cmd_length",
                        "decode_triangle_setup", "decode_rgba", "decode_tex", "decode_z"]),
    "primitive set-up": ("draw_primitive", "primitives",
                         ["draw_primitive", "fixup_triangle_setup", "build_derived", "build_combiner_constants",
                          "normalize_dzpix", "dz_compress_host", "deduce_static_texture_state",
                          "deduce_noise_state", "normalize_static_state", "acc_texel0", "acc_texel1", "norm_mul",
                          "norm_muladd", "norm_mulsub", "norm_add", "norm_aaddsub", "norm_amul"]),
    "TMEM update": ("apply_upload", "uploads",
                    ["apply_upload", "update_tmem_32", "update_tmem_16", "update_tmem_lut", "compute_upload_t",
                     "load_tile", "load_tile_iteration"]),
    "binning": ("bin_primitive", "primitive x tile tests", ["bin_primitive", "interpolate_xs"]),
    "span set-up": ("span_setup", "span rows", ["span_setup", "quantize_x"]),
    "coverage": ("compute_coverage", "candidate pixels", ["compute_coverage"]),
    "shade interpolation": ("interpolate_rgba", "shaded pixels", ["interpolate_rgba"]),
    "STZ + perspective": ("interpolate_stz", "shaded pixels",
                          ["interpolate_stz", "perspective_divide", "perspective_get_lut", "st_divide",
                           "interpolate_st_single", "interpolate_st_copy", "clamp_z"]),
    "LOD": ("compute_lod_2cycle", "LOD evaluations", ["compute_lod_2cycle"]),
    "texel fetch + filter": ("sample_texture", "texture samples",
                             ["sample_texture", "sample_texture_copy", "sample_texture_copy_word", "texel_mask_s",
                              "texel_mask_t", "byte_index", "hw_index", "clamp_and_shift_coord", "shift_coord",
                              "bilinear_3tap", "bilinear_3tap2", "texture_convert_factors", "convert_rgba16",
                              "convert_ia16", "texel_rgba4", "texel_ia4", "texel_ci4", "texel_ci8", "texel_ci16",
                              "texel_ci32", "texel_rgba8", "texel_ia8", "texel_i4", "texel_i8", "texel_yuv16",
                              "texel_rgba16", "texel_ia16", "texel_rgba32", "fetch_texel", "tlut_lookup"]),
    "combiner": ("combiner_cycle1", "combiner passes",
                 ["combiner_cycle0", "combiner_cycle1", "sel", "combiner_equation", "clamp_9bit",
                  "clamp_9bit_notrunc", "special_expand", "noise_combiner", "alpha_cvg"]),
    "dither + noise": ("dither_coefficients", "shaded pixels",
                       ["dither_coefficients", "reseed_noise", "rgb_dither", "noise_blend_threshold",
                        "noise_get_combiner", "noise_get_dither_alpha", "noise_get_dither_color",
                        "noise_get_blend_threshold"]),
    "shading control + alpha test": ("shade_pixel", "pixel tests", ["shade_pixel"]),
    "depth test + blender": ("depth_blend_op", "blended pixels",
                             ["depth_blend_op", "depth_test", "blender", "blend_coverage", "decode_memory_color",
                              "z_decompress", "z_compress", "dz_decompress", "dz_compress", "write_color",
                              "copy_pipeline", "fill_color_op"]),
    "framebuffer load / store": ("load_color", "pixels loaded",
                                 ["load_color", "load_depth", "store_color", "store_depth", "alias_color_to_depth",
                                  "alias_depth_to_color"]),
}
# The oracle's own loops and bookkeeping (not the reference's arithmetic): its per-pixel walk over
# the binned tiles, its pixel cache and pass flush, span-row cache, pass counting, set-up of the
# oracle object and the C entry points.
BOOKKEEPING = {"render_primitive", "end_pass", "span_row", "begin_span_rows", "prim", "cut", "hard", "total",
               "oracle_enqueue", "oracle_create", "oracle_destroy", "init_luts", "Oracle", "upload_needs_flush",
               "upload", "upload_reads_pass", "enqueue", "rv_end", "flush_pass"}
# Stages whose work the shading kernel (k_shade) does; the rest is set-up, binning, TMEM, blend.
SHADING_STAGES = ["span set-up", "coverage", "shade interpolation", "STZ + perspective", "LOD",
                  "texel fetch + filter", "combiner", "dither + noise", "shading control + alpha test"]

_BIN = r"(\+|-|\*|/|%|<<|>>|r<<|r>>|&|\||\^|<|<=|>|>=|==|!=|w\*|h\*|/\[fl\]|/\[ex\]|%\[fl\])"
_RE_BIN = re.compile(r"^\S+ = \S+ " + _BIN + r" \S+;$")
_RE_UN = re.compile(r"^\S+ = (-|~|!)\S+;$")
_RE_FN = re.compile(r"^\S+ = (MIN_EXPR|MAX_EXPR|ABS_EXPR|ABSU_EXPR) <")
_RE_SEL = re.compile(r"^\S+ = \S+ \? \S+ : \S+;$")
_RE_BUILTIN = re.compile(r"^\S+ = __builtin_(popcount|clz|ctz|ffs|parity|bswap)\w* ")
# Calls of the standard library's arithmetic helpers (not inlined in this build) are their ops.
_RE_STDCALL = re.compile(r"^(?:\S+ = )?std::(min|max|abs|clamp)\b")
_RE_IF = re.compile(r"^if \(\S+ " + _BIN + r" \S+\)$")
_RE_SWITCH = re.compile(r"^switch \(")
_RE_LOC = re.compile(r"^\s*\[([^:\]]+):(\d+):\d+(?: discrim \d+)?\] (.*)$")


def count_ops(stmt):
    s = stmt.strip()
    if _RE_BIN.match(s) or _RE_UN.match(s) or _RE_FN.match(s) or _RE_SEL.match(s) or _RE_BUILTIN.match(s):
        return 1
    if _RE_IF.match(s) or _RE_SWITCH.match(s):
        return 1
    m = _RE_STDCALL.match(s)
    if m:
        return 2 if m.group(1) == "clamp" else 1
    return 0


_RE_CALLEE = re.compile(r"\{anonymous\}::(?:Oracle::)?([A-Za-z_][A-Za-z_0-9]*) \(")


def ops_per_line(dump_path, source_name):
    """({line: ops}, {line: [callee, ...]}) of `source_name`'s statements; a statement without a
    location takes the last location seen in its basic block."""
    ops, calls = {}, {}
    last = None
    for raw in open(dump_path):
        line = raw.rstrip("\n")
        st = line.strip()
        if st.startswith("<bb ") or st.startswith(";;") or not st:
            last = None
            continue
        m = _RE_LOC.match(line)
        if m:
            fname, ln, stmt = m.group(1), int(m.group(2)), m.group(3)
            last = (fname, ln)
        else:
            if last is None or st.startswith("#") or st.startswith("goto") or st.startswith("else"):
                continue
            fname, ln = last
            stmt = st
        if os.path.basename(fname) != source_name:
            continue
        n = count_ops(stmt)
        if n:
            ops[ln] = ops.get(ln, 0) + n
        for callee in _RE_CALLEE.findall(stmt):
            calls.setdefault(ln, []).append(callee)
    return ops, calls


def build():
    if os.path.exists(OUT):
        shutil.rmtree(OUT)
    os.makedirs(OUT)
    flags = ["-O1", "-fno-inline", "-fwrapv", "-ffp-contract=off", "-std=c++20", "-fPIC"]
    subprocess.run(["g++"] + flags + ["-fprofile-arcs", "-ftest-coverage", "-fprofile-update=atomic",
                                      "-fdump-tree-optimized-lineno", "-c", os.path.join(HERE, "rdp_oracle.cpp"),
                                      "-o", "rdp_oracle.o"], cwd=OUT, check=True)
    subprocess.run(["g++"] + flags + ["-c", os.path.join(HERE, "vi_oracle.cpp"), "-o", "vi_oracle.o"], cwd=OUT,
                   check=True)
    subprocess.run(["g++", "-shared", "-fprofile-arcs", "-o", LIB, "rdp_oracle.o", "vi_oracle.o", "-lpthread"],
                   cwd=OUT, check=True)
    dumps = glob.glob(os.path.join(OUT, "*optimized"))
    assert len(dumps) == 1, dumps
    return dumps[0]


_CHILD = r"""
import os, sys
sys.path[:0] = [%(pkg)r, %(oracle)r]
from rdp_gb300 import cmdgen
from oracle import Oracle
kind, lo, hi = sys.argv[1], int(sys.argv[2]), int(sys.argv[3])
configs = {"plain": cmdgen.CONFIG_PLAIN, "textured": cmdgen.CONFIG_TEXTURED, "mixed16": cmdgen.CONFIG_MIXED}
for i in range(lo, hi):
    p = cmdgen.batched_instance_params(i) if kind == "batched64" else cmdgen.default_params(configs[kind], seed=0)
    words, rdram, prims = cmdgen.generate_stream(p)
    o = Oracle(8 << 20)
    o.write_rdram(rdram)
    o.enqueue(words)
    print("fragments", o.fragments(), "passes", o.reference_passes(), flush=True)
    o.close()
"""


def run_workload(kind, jobs):
    for g in glob.glob(os.path.join(OUT, "*.gcda")):
        os.unlink(g)
    n = 64 if kind == "batched64" else 1
    # Big instances first so that the processes finish together.
    chunks = [(i, i + 1) for i in range(n)]
    env = dict(os.environ, RDP_ORACLE_LIB=LIB)
    code = _CHILD % {"pkg": os.path.join(ROOT, "parallel-rdp_gb300"), "oracle": HERE}
    frags = passes = 0
    running = []
    pending = list(chunks)
    while pending or running:
        while pending and len(running) < jobs:
            lo, hi = pending.pop(0)
            running.append(subprocess.Popen([sys.executable, "-c", code, kind, str(lo), str(hi)], env=env,
                                            stdout=subprocess.PIPE, text=True))
        p = running.pop(0)
        out, _ = p.communicate()
        assert p.returncode == 0, out
        for line in out.splitlines():
            f = line.split()
            frags += int(f[1])
            passes += int(f[3])
    return frags, passes


def gcov_lines():
    r = subprocess.run(["gcov", "--json-format", "--stdout", "-o", OUT, os.path.join(OUT, "rdp_oracle.o")],
                       cwd=OUT, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, check=True)
    data = json.loads(r.stdout)
    for f in data["files"]:
        if os.path.basename(f["file"]) == "rdp_oracle.cpp":
            return f
    raise RuntimeError("no gcov data for rdp_oracle.cpp")


def method(demangled):
    """The bare name of a (member) function from its demangled signature."""
    m = re.search(r"([A-Za-z_][A-Za-z_0-9]*)(?:<[^()]*>)?\(", demangled)
    return m.group(1) if m else demangled


def table(kind, line_ops, line_calls, jobs):
    frags, passes = run_workload(kind, jobs)
    g = gcov_lines()
    fn_name = {f["name"]: method(f["demangled_name"]) for f in g["functions"]}
    fn_calls = {}
    for f in g["functions"]:
        fn_calls[method(f["demangled_name"])] = fn_calls.get(method(f["demangled_name"]), 0) + f["execution_count"]
    # Per function: its own lines' ops, and how often each line calling another oracle function ran.
    self_ops, call_sites = {}, {}
    for ln in g["lines"]:
        n = ln["line_number"]
        if not ln["count"]:
            continue
        name = fn_name.get(ln.get("function_name"), "?")
        if line_ops.get(n):
            self_ops[name] = self_ops.get(name, 0) + line_ops[n] * ln["count"]
        for callee in line_calls.get(n, []):
            cs = call_sites.setdefault(name, {})
            cs[callee] = cs.get(callee, 0) + ln["count"]
    assigned = {f for _, _, fns in STAGES.values() for f in fns}
    # Helpers (arithmetic and RDRAM-access functions called by the stages) count where they are
    # called: each call adds the helper's inclusive ops per call.
    helpers = {f for f in set(self_ops) | set(fn_calls) if f not in assigned and f not in BOOKKEEPING}
    k_incl = {h: 0.0 for h in helpers}
    for _ in range(8):
        for h in helpers:
            tot = self_ops.get(h, 0) + sum(c * k_incl.get(cal, 0.0) for cal, c in call_sites.get(h, {}).items()
                                           if cal in helpers)
            k_incl[h] = tot / fn_calls[h] if fn_calls.get(h) else 0.0

    def inclusive(f):
        return self_ops.get(f, 0) + sum(c * k_incl.get(cal, 0.0) for cal, c in call_sites.get(f, {}).items()
                                        if cal in helpers)

    stages = {}
    for st, (unit_fn, unit, fns) in STAGES.items():
        ops = sum(inclusive(f) for f in fns)
        units = fn_calls.get(unit_fn, 0)
        stages[st] = {"units": units, "unit": unit + " (calls of %s)" % unit_fn, "ops": ops,
                      "K_ops_per_unit": ops / units if units else 0.0}
    excluded = {f: inclusive(f) for f in sorted(BOOKKEEPING, key=lambda f: -inclusive(f)) if inclusive(f)}
    helper_k = {h: k_incl[h] for h in sorted(helpers) if k_incl[h]}
    total = sum(s["ops"] for s in stages.values())
    shading = sum(stages[s]["ops"] for s in SHADING_STAGES)
    return {"fragments": frags, "reference_passes": passes, "ops_total": total, "ops_shading_stages": shading,
            "ops_per_fragment": total / frags if frags else 0.0, "stages": stages,
            "helper_ops_per_call": helper_k, "excluded_oracle_bookkeeping_ops": excluded}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    dump = build()
    line_ops, line_calls = ops_per_line(dump, "rdp_oracle.cpp")
    out = {
        "what": "dynamic integer/logic ops of the reference's RDP algorithm, per stage, counted on the CPU oracle "
                "(GIMPLE ops per source line at -O1 without inlining x gcov line counts)",
        "command": "python oracle/make_op_table.py",
        "op_kinds": "add sub mul div mod shl shr rotate and or xor not neg compare min max abs select popcount/clz/"
                    "ctz/ffs branch-compare switch; not loads, stores, copies, width casts",
        "shading_stages": SHADING_STAGES,
        "workloads": {},
    }
    for kind in ("plain", "textured", "mixed16", "batched64"):
        out["workloads"][kind] = table(kind, line_ops, line_calls, args.jobs)
        w = out["workloads"][kind]
        print("%s: %.3e ops, %d fragments, %.1f ops/fragment" % (kind, w["ops_total"], w["fragments"],
                                                                w["ops_per_fragment"]))
    with open(os.path.join(HERE, "op_table.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
