"""swgb_plan_batch on the CPU: how swgb_draw_batch splits draws into
segments that run concurrently.  Addresses are synthetic (nothing is
dereferenced); the rule is that no draw of a segment may write bytes that an
earlier draw of the segment writes or reads, or read bytes it writes, and all
draws of a segment share one raster variant."""
import ctypes as C

import pytest

from swiftshader_gb300 import abi, scenes

BASE = 1 << 40
MB = 1 << 20


@pytest.fixture(scope="module")
def lib():
    from swiftshader_gb300 import _lib, build
    build.build()
    return _lib.load()


def plan(lib, draws):
    n = len(draws)
    st = (abi.PipelineState * n)(*[d[0] for d in draws])
    ar = (abi.DrawArgs * n)(*[d[1] for d in draws])
    first = (C.c_uint32 * max(n, 1))()
    cnt = C.c_uint32()
    assert lib.swgb_plan_batch(st, ar, n, first, C.byref(cnt)) == abi.OK
    return list(first)[:cnt.value]


def draw(scene, color, depth, vertex=BASE + (900 << 20), levels=None, color_pitch=None, depth_pitch=None):
    levels = levels or [BASE + (950 << 20) + k * MB for k in range(len(scene.texture_levels))]
    return (scenes.build_state(scene, color, depth, vertex, levels, color_pitch, depth_pitch), scenes.build_args(scene))


def small(w=96, h=64, seed=0, **kw):
    s = scenes.scene_small(n_tris=8, width=w, height=h, seed_index=seed)
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def test_disjoint_unaligned_adjacent_attachments_form_one_segment(lib):
    """Attachments packed back to back at addresses that are not multiples of
    the row pitch (as a caching allocator returns them): one segment."""
    sz = 96 * 64 * 4
    draws = [draw(small(seed=i), BASE + 512 + i * sz, BASE + (200 << 20) + 512 + i * sz) for i in range(12)]
    assert plan(lib, draws) == [0]


def test_msaa_planes_back_to_back(lib):
    sz = 4 * 96 * 64 * 8
    draws = []
    for i in range(6):
        s = small(seed=i, samples=4, color_format=abi.FORMAT_R16G16B16A16_SFLOAT)
        draws.append(draw(s, BASE + 768 + i * sz, BASE + (300 << 20) + 768 + i * (sz // 2)))
    assert plan(lib, draws) == [0]


def test_same_target_splits_at_every_dependency(lib):
    draws = [draw(small(seed=i), BASE, BASE + (200 << 20)) for i in range(4)]
    assert plan(lib, draws) == [0, 1, 2, 3]


def test_disjoint_scissors_on_one_target(lib):
    draws = []
    for k in range(8):
        s = small(w=256, h=128, seed=k, scissor=((k % 4) * 64, (k // 4) * 64, 64, 64))
        draws.append(draw(s, BASE, BASE + (200 << 20)))
    assert plan(lib, draws) == [0]
    # a ninth draw over two of the scissors depends on both
    draws.append(draw(small(w=256, h=128, seed=9, scissor=(32, 0, 64, 32)), BASE, BASE + (200 << 20)))
    assert plan(lib, draws) == [0, 8]


def test_depth_only_conflict_and_depth_test_off(lib):
    sz = 96 * 64 * 4
    a = draw(small(seed=1), BASE, BASE + (200 << 20))
    b = draw(small(seed=2), BASE + 4 * sz, BASE + (200 << 20))  # other colour, same depth
    assert plan(lib, [a, b]) == [0, 1]
    b[0].depth_test_enable = 0  # no depth access: independent
    assert plan(lib, [a, b]) == [0]


def test_aliasing_with_another_pitch(lib):
    """A colour attachment of one pitch overlapping the depth attachment of
    another draw (different pitch) is a conflict."""
    a = draw(small(w=96, h=64, seed=1, color_format=abi.FORMAT_R32G32B32A32_SFLOAT), BASE, BASE + (200 << 20))
    b = draw(small(w=96, h=64, seed=2), BASE + (100 << 20), BASE + 4096)
    assert plan(lib, [a, b]) == [0, 1]


def test_reading_a_texture_written_earlier(lib):
    tex = scenes.scene_textured_small(n_tris=8, width=64, height=64, tex_size=32, mip=False, seed_index=3)
    a = draw(small(w=64, h=64, seed=1), BASE, BASE + (200 << 20))
    b = draw(tex, BASE + (10 << 20), BASE + (210 << 20), levels=[BASE + 1024])  # samples a's colour bytes
    assert plan(lib, [a, b]) == [0, 1]
    c = draw(tex, BASE + (10 << 20), BASE + (210 << 20), levels=[BASE + (400 << 20)])
    assert plan(lib, [a, c]) == [0]


def test_variant_changes_and_empty_draws(lib):
    sz = 4 * 96 * 64 * 16
    d0 = draw(small(seed=0), BASE, BASE + (200 << 20))
    d1 = draw(small(seed=1, color_format=abi.FORMAT_R32G32B32A32_SFLOAT), BASE + sz, BASE + (200 << 20) + sz)
    d2 = draw(small(seed=2), BASE + 2 * sz, BASE + (200 << 20) + 2 * sz)
    d2[1].count = 0
    d3 = draw(small(seed=3), BASE + 3 * sz, BASE + (200 << 20) + 3 * sz)
    assert plan(lib, [d0, d1, d2, d3]) == [0, 1, 3]
