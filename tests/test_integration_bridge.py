"""The reference-side binding (swiftshader_gb300/integration/swgb_vk_bridge.cpp):
every field of swgb_pipeline_state and swgb_draw_args has a source in it, and
it compiles against SwiftShader's own headers (syntax only, where the
reference sources are present; nothing runs)."""
import os
import re
import subprocess
import sys

import pytest

from swiftshader_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BRIDGE = os.path.join(ROOT, "swiftshader_gb300", "integration", "swgb_vk_bridge.cpp")


def _assigned(src, prefix):
    return set(re.findall(r"\b%s\.(\w+)" % re.escape(prefix), src))


def test_every_field_has_a_source():
    src = open(BRIDGE).read()
    state = _assigned(src, "out")
    for name, _ in abi.PipelineState._fields_:
        if name.startswith("reserved"):
            continue
        assert name in state, "swgb_pipeline_state.%s is never filled" % name
    tex = _assigned(src, "t")
    for name, _ in abi.Texture._fields_:
        assert name in tex, "swgb_texture.%s is never filled" % name
    sten = _assigned(src, "o")
    for name, _ in abi.StencilOpState._fields_:
        assert name in sten, "swgb_stencil_op_state.%s is never filled" % name
    for name, _ in abi.DrawArgs._fields_:
        assert name in state, "swgb_draw_args.%s is never filled" % name


def test_compiles_against_the_reference_headers():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "refjit"))
    import build_refjit
    if not build_refjit.REF.is_dir():
        pytest.skip("reference sources not present")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wno-ignored-attributes"] + build_refjit.pipeline_flags() + [BRIDGE]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "warning" not in r.stderr, r.stderr[-3000:]
