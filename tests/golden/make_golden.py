"""Generates tests/golden/golden.json: seeded command streams (by generator
parameters) with the CPU oracle's RDRAM / hidden RDRAM / TMEM digests, fragment
counts and VI scanout digests.

The reference ships no golden images or hashes for this path (its conformance
suites compare against a live Angrylion-Plus run), so these fixtures pin the
oracle against itself across changes and give the GPU tests an expected answer
that does not need the oracle at run time.  Regenerate only after a deliberate,
reviewed change to the oracle:

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "parallel-rdp_gb300"), os.path.dirname(HERE)]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def render_cases():
    from rdp_gb300 import cmdgen
    F = cmdgen.FLAGS
    cases = [
        ("plain_full_seed0", cmdgen.CONFIG_PLAIN, dict(seed=0)),
        ("plain_seed5_300", cmdgen.CONFIG_PLAIN, dict(seed=5, num_prims=300)),
        ("textured_full_seed0", cmdgen.CONFIG_TEXTURED, dict(seed=0)),
        ("mixed_seed0_4000", cmdgen.CONFIG_MIXED, dict(seed=0, num_prims=4000, num_frames=1)),
        ("mixed_seed1_2x600", cmdgen.CONFIG_MIXED, dict(seed=1, num_prims=600, num_frames=2)),
    ]
    for fmt_name, fmt in (("5551", cmdgen.FB_RGBA5551), ("8888", cmdgen.FB_RGBA8888), ("i8", cmdgen.FB_I8),
                          ("ia88", cmdgen.FB_IA88), ("i4", cmdgen.FB_I4)):
        cases.append(("fuzz_%s_seed11" % fmt_name, cmdgen.CONFIG_PLAIN,
                      dict(seed=11, num_prims=300, fb_format=fmt, flags=F["FUZZ"] | F["CLEAR"])))
    return cases


def vi_cases():
    # (name, variant key of the VI parity suite, frames)
    return [("vi_5551_aa_divot_dither_gamma", "5551_aa_divot_dither_gamma", 2),
            ("vi_8888_aa_divot", "8888_aa_divot", 2),
            ("vi_5551_serrate_pal", "5551_serrate_pal", 2),
            ("vi_5551_scale_bias", "5551_scale_bias", 2)]


def oracle_render(config, kw):
    from rdp_gb300 import cmdgen
    from rdp_testutil import run_oracle
    p = cmdgen.default_params(config, **kw)
    words, rdram, _ = cmdgen.generate_stream(p)
    rd, hid, tmem, frags = run_oracle(words, rdram)
    return {"config": config, "params": kw, "words_sha256": sha(words), "num_words": int(words.size),
            "rdram_sha256": sha(rd), "hidden_sha256": sha(hid), "tmem_sha256": sha(tmem), "fragments": int(frags)}


def vi_frames(variant, frames, backend):
    """Yields the scanout digest of each frame; backend is 'oracle' or a CommandProcessor."""
    import zlib
    import test_vi_parity_gpu as t
    from rdp_gb300 import ScanoutOptions
    v = t.VARIANTS[variant]
    rng = np.random.default_rng(zlib.crc32(variant.encode()))
    opts = ScanoutOptions(blend_previous_frame=1, upscale_deinterlacing=0)
    out = []
    for it in range(frames):
        rd = rng.integers(0, 256, t.RDRAM, dtype=np.uint8)
        hid = rng.integers(0, 4, t.RDRAM // 2, dtype=np.uint8)
        regs = t._variant_regs(rng, v, it)
        if backend == "oracle":
            from oracle import Oracle
            if it == 0:
                vi_frames.o = Oracle(t.RDRAM)
            o = vi_frames.o
            o.write_rdram(rd)
            o.write_hidden(hid)
            for r, val in regs.items():
                o.set_vi_register(r, val)
            img = o.scanout(opts.as_words())
        else:
            backend.write_rdram(rd)
            backend.write_hidden_rdram(hid)
            for r, val in regs.items():
                backend.set_vi_register(r, val)
            img = backend.scanout_sync(opts)
        out.append(None if img is None else [int(img.shape[1]), int(img.shape[0]), sha(img)])
    return out


def main():
    import oracle
    oracle.build()
    g = {"render": {}, "vi": {}}
    for name, config, kw in render_cases():
        g["render"][name] = oracle_render(config, kw)
        print(name, g["render"][name]["fragments"])
    for name, variant, frames in vi_cases():
        g["vi"][name] = {"variant": variant, "frames": vi_frames(variant, frames, "oracle")}
        print(name)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(g, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
