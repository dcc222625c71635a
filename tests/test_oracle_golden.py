"""The oracle against its committed fixtures (tests/golden/oracle_frames.json,
made by tests/golden/make_golden.py): same bits on every host architecture and
for every thread count."""
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402

with open(os.path.join(HERE, "golden", "oracle_frames.json")) as f:
    GOLDEN = json.load(f)


@pytest.mark.parametrize("name", sorted(GOLDEN))
@pytest.mark.parametrize("nthreads", [1, 3])
def test_oracle_reproduces_fixture(oracle_mod, name, nthreads):
    scene = make_golden.golden_scenes()[name]
    assert make_golden.digest(scene, nthreads) == GOLDEN[name]
