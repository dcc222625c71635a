"""Regenerates tests/golden/oracle_frames.json: SHA-256 of the oracle's colour
and depth attachments plus its counters for small seeded scenes.

The fixtures pin the oracle against accidental change and across host
architectures (the GPU hosts are aarch64, this container x86_64): the same
restatement must give the same bits on both.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from swiftshader_gb300 import abi, scenes  # noqa: E402


def golden_scenes():
    return {
        "tris1000_256x256": scenes.scene_small(),
        "textured200_trilinear_repeat_blend": scenes.scene_textured_small(),
        "textured200_bilinear_clamp": scenes.scene_textured_small(mip=False, address=abi.ADDRESS_CLAMP_TO_EDGE, blend=False),
        "heightfield_160x80_320x180": scenes.scene_heightfield(quads_x=160, quads_y=80, width=320, height=180, tex_size=256),
    }


def digest(scene, nthreads=2):
    import oracle
    c, d, cnt = oracle.render(scene, nthreads)
    # the draw counters (the adjoint's counters are not the oracle's)
    cnt = {k: v for k, v in cnt.items() if not k.startswith("adjoint_")}
    return {"color_sha256": hashlib.sha256(c.tobytes()).hexdigest(),
            "depth_sha256": hashlib.sha256(d.tobytes()).hexdigest(),
            "counters": cnt}


if __name__ == "__main__":
    out = {name: digest(sc) for name, sc in golden_scenes().items()}
    with open(os.path.join(HERE, "oracle_frames.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", len(out), "fixtures")
