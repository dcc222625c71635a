"""Writes tests/golden/refjit_fixtures.npz: outputs of SwiftShader's OWN routines.

Test infrastructure.  Run in a container holding the reference sources after
``python oracle/refjit/build_refjit.py`` (x86-64; the Subzero JIT backend):

    python tests/golden/make_refjit_fixtures.py

For every case of refjit_cases.py it feeds the oracle's vertex records and draw
constants (``oracle_triangle_inputs``) to the reference's routines and stores
what they return:

* setup.*   Clipper::Clip + SetupRoutine per triangle: {yMin, yMax, clipped,
            visible}, every sample's outline rows yMin-1 .. yMax, the x0/y0,
            z, w and varying plane equations and zBias;
* sampler.* a SamplerCore routine (implicit LOD) on seeded quads of texture
            coordinates, per texture format / filter / mipmap mode / address
            mode / border colour / LOD bias and clamps;
* raster.*  QuadRasterizer + PixelRoutine without a fragment shader over every
            triangle of a draw: the depth and stencil attachments afterwards
            and {visible, clipped, occlusion samples}.

Each case also stores the SHA-256 of the inputs it was made from, so the test
can tell a changed input from a changed result.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "oracle", "refjit"), HERE]

import oracle  # noqa: E402
import refjit  # noqa: E402
import refjit_cases  # noqa: E402
from swiftshader_gb300 import scenes  # noqa: E402

OUT = os.path.join(HERE, "refjit_fixtures.npz")


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def case_inputs(olib, st, args, ntri):
    T = ntri
    vf = np.zeros((T, 3 * refjit.VF), np.float32)
    vi = np.zeros((T, 3 * refjit.VI), np.int32)
    consts = scissor = None
    nv = 0
    for t in range(T):
        f, i, consts, scissor, nv = refjit.triangle_inputs(olib, st, args, t)
        vf[t], vi[t] = f, i
    return vf, vi, consts, scissor, nv


def main():
    olib = oracle.lib()
    out = {}
    for name, s in refjit_cases.setup_cases().items():
        color, depth = scenes.clear_buffers(s)
        st, args, keep = oracle.host_state(s, color, depth)
        vf, vi, consts, scissor, nv = case_inputs(olib, st, args, s.tri_count)
        rows = s.height + 4
        oi, spans, of = [], [], []
        for t in range(s.tri_count):
            ri, rs, rf = refjit.setup(st, vf[t], vi[t], consts, scissor, nv, rows)
            oi.append(ri)
            n = int(ri[1] - ri[0] + 2) if ri[3] else 0
            spans.append(rs[:s.samples, :n].reshape(-1, 2))
            f = np.zeros(8 + 3 * nv + 1, np.float32)
            if ri[3]:
                f[:] = rf
            of.append(f)
        out["setup.%s.inputs_sha256" % name] = np.array(digest(vf, vi, consts, scissor))
        out["setup.%s.out_i" % name] = np.asarray(oi, np.int32)
        out["setup.%s.spans" % name] = np.concatenate(spans).astype(np.uint16)
        out["setup.%s.out_f" % name] = np.asarray(of, np.float32)
        print("setup", name, s.tri_count, "triangles", flush=True)

    textures = refjit_cases.sampler_textures()
    cfgs = refjit_cases.sampler_configs()
    U, V, R = [], [], []
    for ci, cfg in enumerate(cfgs):
        chain = textures[(cfg[0], cfg[1], cfg[2])]
        tex = refjit_cases.texture_struct(chain, cfg)
        us, vs = refjit_cases.sampler_quads(ci, cfg[1], cfg[2])
        U.append(us)
        V.append(vs)
        R.append(np.stack([refjit.sample_quad(tex, us[q], vs[q]) for q in range(len(us))]))
    out["sampler.cfg"] = np.asarray(cfgs, np.float64)
    out["sampler.u"] = np.asarray(U, np.float32)
    out["sampler.v"] = np.asarray(V, np.float32)
    out["sampler.out"] = np.asarray(R, np.float32)  # [config, quad, component, lane]
    out["sampler.textures_sha256"] = np.array(digest(*[l for k in sorted(textures) for l in textures[k]]))
    print("sampler", len(cfgs), "configurations", flush=True)

    for name, s in refjit_cases.raster_cases().items():
        color, depth = scenes.clear_buffers(s)
        stencil = scenes.stencil_buffer(s)
        st, args, keep = oracle.host_state(s, color, depth, stencil)
        vf, vi, consts, scissor, nv = case_inputs(olib, st, args, s.tri_count)
        counts = refjit.raster(st, vf, vi, consts, scissor, s.tri_count, nv)
        out["raster.%s.inputs_sha256" % name] = np.array(digest(vf, vi, consts, scissor))
        out["raster.%s.depth" % name] = depth
        if stencil is not None:
            out["raster.%s.stencil" % name] = stencil
        out["raster.%s.counts" % name] = np.asarray(counts, np.uint64)
        print("raster", name, counts, flush=True)

    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
