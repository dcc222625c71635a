"""CPU tests of the persistent autotuner table (swiftshader_gb300.tuning)."""
import json

import pytest

from swiftshader_gb300 import abi, scenes
from swiftshader_gb300.tuning import TuningTable, workload_class


def _draws(n=3, tris=1000, size=256, textured=False):
    S = (abi.PipelineState * n)()
    A = (abi.DrawArgs * n)()
    for i in range(n):
        sc = scenes.scene_small(n_tris=tris, width=size, height=size, seed_index=40 + i)
        if textured:
            sc = scenes.scene_heightfield(quads_x=8, quads_y=4, width=size, height=size, tex_size=64)
        S[i] = scenes.build_state(sc, 0, 0, 0, [0] * 16)  # key only: never passed to the library
        A[i] = scenes.build_args(sc)
    return S, A


def test_class_key_is_deterministic_and_separates_shapes():
    S, A = _draws()
    k1 = workload_class(S, A, True)
    assert k1 == workload_class(S, A, True)
    assert k1 != workload_class(S, A, False)
    S2, A2 = _draws(tris=64000)
    assert workload_class(S2, A2, True) != k1
    S3, A3 = _draws(size=1024)
    assert workload_class(S3, A3, True) != k1


def test_round_trip(tmp_path):
    S, A = _draws()
    key = workload_class(S, A, True)
    t = TuningTable()
    res = [({"bin": "%dx%d" % sh, "hiz": hz}, {"median": 1.0 + i, "min": 0.9 + i, "max": 1.2 + i})
           for i, (sh, hz) in enumerate((sh, hz) for sh in abi.BIN_SHAPES for hz in (1, 0))]
    t.record(key, {"bin": "32x16", "hiz": 0}, res)
    p = tmp_path / "tuning.json"
    t.save(str(p))
    u = TuningTable.load(str(p))
    assert u.entries == t.entries
    assert u.get(key)["bin"] == "32x16" and u.get(key)["hiz"] == 0
    assert set(u.get(key)["candidates_ms"]) == {"16x16 hiz1", "16x16 hiz0", "32x16 hiz1", "32x16 hiz0",
                                                "32x32 hiz1", "32x32 hiz0"}
    assert TuningTable.load(str(tmp_path / "absent.json")).entries == {}


def test_rejects_bad_tables(tmp_path):
    p = tmp_path / "t.json"
    p.write_text(json.dumps({"version": 99, "entries": {}}))
    with pytest.raises(ValueError):
        TuningTable.load(str(p))
    p.write_text(json.dumps({"version": 1, "entries": {"k": {"bin": "8x8", "hiz": 1, "candidates_ms": {}}}}))
    with pytest.raises(ValueError):
        TuningTable.load(str(p))
