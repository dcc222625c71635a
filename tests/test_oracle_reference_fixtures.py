"""The oracle against SwiftShader's OWN routines, bit for bit (CPU).

tests/golden/refjit_fixtures.npz holds what the reference's JIT-compiled
routines returned on the seeded cases of tests/golden/refjit_cases.py
(tests/golden/make_refjit_fixtures.py, run on a build of the reference
sources by oracle/refjit/build_refjit.py with Reactor's Subzero backend):

* setup   -- Clipper::Clip + SetupRoutine (src/Device/Clipper.cpp,
             src/Pipeline/SetupRoutine.cpp): y range, every sample's outline,
             plane equations and depth bias of every triangle;
* sampler -- SamplerCore (src/Pipeline/SamplerCore.cpp) with the implicit
             LOD: 5 texture formats, point / linear, mipmap nearest / linear,
             5 address modes, 3 border colours, LOD bias and clamps;
* raster  -- QuadRasterizer + PixelRoutine (src/Device/QuadRasterizer.cpp,
             src/Pipeline/PixelRoutine.cpp) without a fragment shader:
             coverage, depth interpolation, clamp, bias, D16, the 8 compare
             ops, depth bounds, stencil, 4x MSAA, occlusion counts.

The oracle feeds the reference the same vertex records it uses itself, and
each case checks the digest of those inputs first.  Subzero lowers Reactor's
MulAdd to a multiply and an add where the LLVM backend (the profile the oracle
restates) fuses it; the one MulAdd on these routines is
QuadRasterizer::interpolate's, so the raster cases run the oracle with that
interpolation unfused (oracle_set_interpolation_muladd(0)).  Fusion itself is
pinned by Reactor's FMulAdd known answers (tests/test_oracle_primitives.py).
"""
import ctypes as C
import hashlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), GOLDEN]

import oracle  # noqa: E402
import refjit_cases  # noqa: E402
from swiftshader_gb300 import scenes  # noqa: E402

VF, VI = 14, 3


@pytest.fixture(scope="module")
def fx():
    return np.load(os.path.join(GOLDEN, "refjit_fixtures.npz"))


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def oracle_inputs(olib, st, args, ntri):
    vf = np.zeros((ntri, 3 * VF), np.float32)
    vi = np.zeros((ntri, 3 * VI), np.int32)
    consts = np.zeros(6, np.float32)
    scissor = np.zeros(4, np.int32)
    for t in range(ntri):
        f = np.zeros(3 * VF, np.float32)
        i = np.zeros(3 * VI, np.int32)
        assert olib.oracle_triangle_inputs(C.byref(st), C.byref(args), t, f.ctypes.data, i.ctypes.data,
                                           consts.ctypes.data, scissor.ctypes.data) >= 0
        vf[t], vi[t] = f, i
    return vf, vi, consts, scissor


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32 if a.dtype.itemsize == 4 else np.uint16)


@pytest.mark.parametrize("name", list(refjit_cases.setup_cases()))
def test_setup_matches_reference(fx, name):
    s = refjit_cases.setup_cases()[name]
    olib = oracle.lib()
    color, depth = scenes.clear_buffers(s)
    st, args, keep = oracle.host_state(s, color, depth)
    vf, vi, consts, scissor = oracle_inputs(olib, st, args, s.tri_count)
    assert digest(vf, vi, consts, scissor) == str(fx["setup.%s.inputs_sha256" % name]), "inputs changed"
    ref_i, ref_spans, ref_f = fx["setup.%s.out_i" % name], fx["setup.%s.spans" % name], fx["setup.%s.out_f" % name]
    rows = s.height + 4
    nf = ref_f.shape[1]
    pos = 0
    visible = 0
    for t in range(s.tri_count):
        oi = np.zeros(4, np.int32)
        sp = np.zeros((4, rows, 2), np.uint16)
        of = np.zeros(8 + 3 * 8 + 1, np.float32)
        assert olib.oracle_setup_samples(C.byref(st), C.byref(args), t, oi.ctypes.data, sp.ctypes.data, rows,
                                         of.ctypes.data) >= 0
        assert (oi == ref_i[t]).all(), "triangle %d: {yMin, yMax, clipped, visible} oracle %s reference %s" % (
            t, oi, ref_i[t])
        if not oi[3]:
            continue
        visible += 1
        n = int(oi[1] - oi[0] + 2)
        mine = sp[:s.samples, :n].reshape(-1, 2)
        theirs = ref_spans[pos:pos + len(mine)]
        pos += len(mine)
        if not (mine == theirs).all():
            k = int(np.argwhere((mine != theirs).any(axis=1))[0, 0])
            raise AssertionError("triangle %d: outline row %d (sample %d) oracle %s reference %s" % (
                t, k % n, k // n, mine[k], theirs[k]))
        diff = bits(of[:nf]) != bits(ref_f[t])
        assert not diff.any(), "triangle %d: plane value %d oracle %r reference %r" % (
            t, int(np.argmax(diff)), of[int(np.argmax(diff))], ref_f[t][int(np.argmax(diff))])
    assert pos == len(ref_spans)
    assert visible > 0


def test_sampler_matches_reference(fx):
    olib = oracle.lib()
    textures = refjit_cases.sampler_textures()
    assert digest(*[l for k in sorted(textures) for l in textures[k]]) == str(fx["sampler.textures_sha256"])
    cfgs = refjit_cases.sampler_configs()
    assert np.array_equal(np.asarray(cfgs, np.float64), fx["sampler.cfg"])
    U, V, R = fx["sampler.u"], fx["sampler.v"], fx["sampler.out"]
    bad = []
    for ci, cfg in enumerate(cfgs):
        chain = textures[(cfg[0], cfg[1], cfg[2])]
        tex = refjit_cases.texture_struct(chain, cfg)
        us, vs = refjit_cases.sampler_quads(ci, cfg[1], cfg[2])
        assert np.array_equal(us, U[ci]) and np.array_equal(vs, V[ci])
        for q in range(len(us)):
            o = np.zeros(16, np.float32)
            assert olib.oracle_sample_quad(C.byref(tex), us[q].ctypes.data_as(C.POINTER(C.c_float)),
                                           vs[q].ctypes.data_as(C.POINTER(C.c_float)),
                                           o.ctypes.data_as(C.POINTER(C.c_float))) == 0
            mine = np.ascontiguousarray(o.reshape(4, 4).T)  # oracle: [lane][component]
            if not (bits(mine) == bits(R[ci, q])).all():
                bad.append((cfg, q, mine, R[ci, q]))
    assert not bad, "%d of %d quads differ; first: config %s quad %d\noracle\n%s\nreference\n%s" % (
        len(bad), len(cfgs) * refjit_cases.QUADS_PER_CONFIG, bad[0][0], bad[0][1], bad[0][2], bad[0][3])


@pytest.mark.parametrize("name", list(refjit_cases.raster_cases()))
def test_raster_depth_stencil_match_reference(fx, name):
    s = refjit_cases.raster_cases()[name]
    olib = oracle.lib()
    color, depth = scenes.clear_buffers(s)
    st, args, keep = oracle.host_state(s, color, depth)
    vf, vi, consts, scissor = oracle_inputs(olib, st, args, s.tri_count)
    assert digest(vf, vi, consts, scissor) == str(fx["raster.%s.inputs_sha256" % name]), "inputs changed"
    olib.oracle_set_interpolation_muladd(0)
    try:
        c, d, stn, cnt = oracle.render_stencil(s, 2)
    finally:
        olib.oracle_set_interpolation_muladd(1)
    ref_d = fx["raster.%s.depth" % name]
    diff = bits(d) != bits(ref_d)
    assert not diff.any(), "%d depth values differ; first at %s: oracle %r reference %r" % (
        int(diff.sum()), tuple(np.argwhere(diff)[0]), d[tuple(np.argwhere(diff)[0])], ref_d[tuple(np.argwhere(diff)[0])])
    if "raster.%s.stencil" % name in fx:
        assert np.array_equal(stn, fx["raster.%s.stencil" % name]), "stencil differs"
    visible, clipped, occlusion = (int(x) for x in fx["raster.%s.counts" % name])
    assert cnt["triangles_visible"] == visible
    assert cnt["triangles_clipped"] == clipped
    # the reference counts samples passing the depth and stencil tests
    # (PixelRoutine::occlusionSampleCount); the oracle's fragments_passed counts
    # the same samples
    assert cnt["fragments_passed"] == occlusion
