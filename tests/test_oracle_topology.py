"""Triangle strips and fans in the oracle (setBatchIndices with the first
vertex provoking, src/Device/Renderer.cpp:97-134): every triangle of a regular
strip or a convex fan has the winding of the first one, and the index types
(uint8 / uint16 / uint32, or none) give the same frame."""
import numpy as np
import pytest

from swiftshader_gb300 import abi, scenes


def regular(topology, n, reverse=False):
    if topology == abi.TOPOLOGY_TRIANGLE_STRIP:
        xs = np.linspace(-0.9, 0.9, n // 2 + 2)
        pts = [(x, y) for x in xs for y in (-0.5, 0.5)][:n + 2]
    else:
        ang = np.linspace(0.0, 2.0 * np.pi, n + 1)
        pts = [(0.0, 0.0)] + [(0.8 * np.cos(a), 0.8 * np.sin(a)) for a in ang]
    if reverse:
        pts = [(x, -y) for x, y in pts]
    v = np.zeros((len(pts), scenes.VERTEX_FLOATS), np.float32)
    v[:, 0:2] = pts
    v[:, 2] = 0.5
    v[:, 3] = 1.0
    v[:, 4:8] = 1.0
    return scenes.Scene(name="regular", width=64, height=64, vertices=v, tri_count=n, topology=topology,
                        cull_mode=abi.CULL_BACK)


@pytest.mark.parametrize("topology", [abi.TOPOLOGY_TRIANGLE_STRIP, abi.TOPOLOGY_TRIANGLE_FAN])
def test_regular_strip_and_fan_keep_one_winding(oracle_mod, topology):
    _, _, a = oracle_mod.render(regular(topology, 20))
    _, _, b = oracle_mod.render(regular(topology, 20, reverse=True))
    # one orientation is entirely front-facing, the mirrored one entirely back-facing
    assert sorted([a["triangles_visible"], b["triangles_visible"]]) == [0, 20]


@pytest.mark.parametrize("topology", [abi.TOPOLOGY_TRIANGLE_STRIP, abi.TOPOLOGY_TRIANGLE_FAN])
def test_index_types_give_the_same_frame(oracle_mod, topology):
    ref = oracle_mod.render(scenes.strip_fan_scene(topology, n_tris=200))
    for dt in (np.uint8, np.uint16, np.uint32):
        got = oracle_mod.render(scenes.strip_fan_scene(topology, n_tris=200, indexed=dt))
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]) and got[2] == ref[2]


def test_first_and_base_vertex(oracle_mod):
    """first_vertex (non-indexed) and base_vertex shift the vertices read."""
    sc = scenes.strip_fan_scene(abi.TOPOLOGY_TRIANGLE_STRIP, n_tris=100)
    ref = oracle_mod.render(sc)
    pad = np.zeros((7, scenes.VERTEX_FLOATS), np.float32)
    shifted = scenes.strip_fan_scene(abi.TOPOLOGY_TRIANGLE_STRIP, n_tris=100)
    shifted.vertices = np.concatenate([pad, sc.vertices])
    shifted.first_vertex = 7
    got = oracle_mod.render(shifted)
    assert np.array_equal(got[0], ref[0]) and got[2] == ref[2]
