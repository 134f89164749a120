"""Generates tests/golden/configs.json: the CPU oracle's answers for the two benchmark-size
configurations, so that the GPU tests can check them without running the oracle.

  instances -- every instance of the batched-instances workload (seeds 0-63, the mixed RGBA8888
               primitive mix, 500-50,000 primitives, resolutions 320x240 / 640x240 / 640x480)
               and of the serving workload, which draws its 256 instances the same way (seeds
               0-255): RDRAM and hidden RDRAM digests, fragment and reference-pass counts of one
               frame.
  mixed16   -- the mixed 640x480 RGBA8888 sequence as configured: 16 frames of 50,000
               primitives (textured triangles, copy-mode TextureRectangles, CI8 + TLUT triangles,
               FillRects; alpha compare, LOD / detail and Z on half the primitives), rendered in
               order; after each frame the RDRAM and hidden RDRAM digests and the VI scanout
               (AA filter, divot, dither filter, interlaced 640x480) digest.

Regenerate only after a deliberate, reviewed change to the oracle or the generator (takes a few
minutes on 8 cores):

    python tests/golden/make_golden_configs.py
"""
import json
import os
import sys
from concurrent.futures import ProcessPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "parallel-rdp_gb300"), os.path.dirname(HERE)]

from golden.make_golden import sha  # noqa: E402

RDRAM = 8 << 20


def mixed_vi_regs(frame):
    """VI registers scanning out the 640x480 RGBA8888 colour image of the mixed sequence: AA
    filter with resampling, divot, dither filter, interlaced (serrate, field = frame parity)."""
    from rdp_gb300 import VIRegister, cmdgen

    def start(a, b):
        return ((a & 0x3ff) << 16) | (b & 0x3ff)

    ctrl = (0 << 8) | 3 | (1 << 4) | (1 << 16) | (1 << 6)
    return {
        VIRegister.Control: ctrl,
        VIRegister.Origin: cmdgen.color_addr(),
        VIRegister.Width: 640,
        VIRegister.VSync: 525,
        VIRegister.VStart: start(34, 34 + 480),
        VIRegister.HStart: start(108, 108 + 640),
        VIRegister.XScale: 1024,
        VIRegister.YScale: 2048,
        VIRegister.VCurrentLine: frame & 1,
    }


def mixed_scanout_options():
    from rdp_gb300 import ScanoutOptions
    return ScanoutOptions(blend_previous_frame=1, upscale_deinterlacing=0)


# The batched instances' frames are also rendered again on the same RDRAM (a benchmark step renders
# every instance's frame each time): digests after 3 and 5 renders.  Rendering a frame twice does
# not always give the first image again (copy-mode rectangles land on an image the frame does not
# clear, textures are read from rendered images), so each count has its own answer.
RERENDERS = (3, 5)


def _batched_instance(i):
    from oracle import Oracle
    from rdp_gb300 import cmdgen
    p = cmdgen.batched_instance_params(i)
    words, rdram, prims = cmdgen.generate_stream(p)
    o = Oracle(RDRAM)
    o.write_rdram(rdram)
    o.enqueue(words)
    out = {"instance": i, "width": p.width, "height": p.height, "primitives": int(prims),
           "words_sha256": sha(words), "rdram_sha256": sha(o.rdram()), "hidden_sha256": sha(o.hidden()),
           "fragments": int(o.fragments()), "reference_passes": int(o.reference_passes())}
    if i < 64:
        done, out["renders"] = 1, {}
        for k in RERENDERS:
            while done < k:
                o.enqueue(words)
                done += 1
            out["renders"][str(k)] = {"rdram_sha256": sha(o.rdram()), "hidden_sha256": sha(o.hidden())}
    o.close()
    return out


def mixed16():
    from oracle import Oracle
    from rdp_gb300 import cmdgen
    p = cmdgen.default_params(cmdgen.CONFIG_MIXED)
    words, rdram, prims, offsets = cmdgen.generate_frames(p)
    o = Oracle(RDRAM)
    o.write_rdram(rdram)
    frames = []
    opts = mixed_scanout_options()
    for f in range(len(offsets) - 1):
        o.enqueue(words[offsets[f]:offsets[f + 1]])
        for r, v in mixed_vi_regs(f).items():
            o.set_vi_register(r, v)
        img = o.scanout(opts.as_words())
        frames.append({"rdram_sha256": sha(o.rdram()), "hidden_sha256": sha(o.hidden()),
                       "fragments": int(o.fragments()),
                       "vi": None if img is None else [int(img.shape[1]), int(img.shape[0]), sha(img)]})
        print("mixed frame", f, frames[-1]["fragments"], flush=True)
    out = {"params": p.describe(), "primitives": int(prims), "words_sha256": sha(words), "frames": frames,
           "reference_passes": int(o.reference_passes())}
    o.close()
    return out


def main():
    import oracle
    oracle.build()
    with ProcessPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        fut_mixed = ex.submit(mixed16)
        batched = list(ex.map(_batched_instance, sorted(range(256), key=lambda i: -_prims(i))))
        mixed = fut_mixed.result()
    g = {"instances": sorted(batched, key=lambda r: r["instance"]), "mixed16": mixed}
    with open(os.path.join(HERE, "configs.json"), "w") as f:
        json.dump(g, f, indent=1, sort_keys=True)


def _prims(i):
    from rdp_gb300 import cmdgen
    return cmdgen.batched_instance_params(i).num_prims


if __name__ == "__main__":
    main()
