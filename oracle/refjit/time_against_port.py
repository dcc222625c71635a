"""TEST INFRASTRUCTURE ONLY: times SwiftShader's own routines against the
oracle port on the same host cores (x86-64, after build_refjit.py).

For each draw (colour writes off, so both sides do the same depth work): the
reference harness's setup loop and JIT-compiled pixel routine (refjit_raster,
one thread, one cluster) and the oracle port's checker and timing builds (one
thread).  Prints one JSON line per draw.

    python oracle/refjit/time_against_port.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), HERE]

import numpy as np  # noqa: E402

import oracle  # noqa: E402
import refjit  # noqa: E402
from swiftshader_gb300 import scenes  # noqa: E402


def best_of(n, f):
    t = 1e9
    r = None
    for _ in range(n):
        t0 = time.perf_counter()
        r = f()
        t = min(t, time.perf_counter() - t0)
    return t, r


def main():
    olib = oracle.lib()
    cases = {
        "1000 random triangles, 256^2": scenes.scene_small(),
        "20000 random triangles, 512^2": scenes.scene_small(n_tris=20000, width=512, height=512, seed_index=3),
        "62.5k-triangle height field, 480x270": scenes.scene_heightfield(quads_x=250, quads_y=125, width=480, height=270,
                                                                         tex_size=64),
    }
    for name, s in cases.items():
        s.color_write_mask = 0
        color, depth = scenes.clear_buffers(s)
        st, args, keep = oracle.host_state(s, color, depth)
        T = s.tri_count
        vf = np.zeros((T, 3 * refjit.VF), np.float32)
        vi = np.zeros((T, 3 * refjit.VI), np.int32)
        consts = scissor = nv = None
        for t in range(T):
            f, i, consts, scissor, nv = refjit.triangle_inputs(olib, st, args, t)
            vf[t], vi[t] = f, i
        refjit.raster(st, vf, vi, consts, scissor, T, nv)  # JIT compile
        setup_s = pixel_s = 1e9
        for _ in range(3):
            color[...] = 0
            depth[...] = s.clear_depth
            c = refjit.raster_timed(st, vf, vi, consts, scissor, T, nv)
            setup_s, pixel_s = min(setup_s, c[3] * 1e-9), min(pixel_s, c[4] * 1e-9)
        checker_s, r = best_of(3, lambda: oracle.render(s, 1))
        timing_s, _ = best_of(3, lambda: oracle.render(s, 1, timing=True))
        print(json.dumps({"draw": name, "triangles": T, "samples_passed": r[2]["fragments_passed"],
                          "reference_occlusion_samples": c[2],
                          "reference_setup_loop_ms": round(setup_s * 1e3, 2),
                          "reference_pixel_routine_ms": round(pixel_s * 1e3, 2),
                          "port_checker_ms": round(checker_s * 1e3, 2), "port_timing_ms": round(timing_s * 1e3, 2)}),
              flush=True)
        del keep


if __name__ == "__main__":
    main()
