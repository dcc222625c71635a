"""Persistent table of raster configurations chosen by swgb_autotune.

No counterpart in the reference (SwiftShader JIT-compiles one routine per
state and has no tunable launch shape).  A table maps a *workload class* --
the properties of a set of draws that decide which bin shape and depth
rejection setting is fastest -- to the configuration the autotuner picked,
with every candidate's median time and spread.  ``Renderer.autotune(...,
table=t)`` consults the table first and tunes (then records) only on a miss;
``TuningTable.save`` / ``TuningTable.load`` keep it as JSON between runs.

The class key holds: batched or single draws, sample count, colour-attachment
format, whether a texture is sampled and its filter, the draws' total
triangle count and total framebuffer area rounded to powers of two.  Draws in
one class share a best configuration closely enough that re-tuning them is
not worth its runs.
"""
from __future__ import annotations

import json
import math
import os
import tempfile
import time

from . import abi

VERSION = 1


def _pow2(x: float) -> int:
    return int(round(math.log2(x))) if x > 0 else -1


def workload_class(states, args, batched: bool) -> str:
    """Class key of a set of draws (the same key for the same shape of work)."""
    n = len(states)
    tris = 0
    area = 0
    samples = set()
    fmts = set()
    tex = set()
    for i in range(n):
        st, a = states[i], args[i]
        tris += int(a.count)
        area += int(st.framebuffer_width) * int(st.framebuffer_height)
        samples.add(int(st.sample_count))
        fmts.add(int(st.color_format))
        if int(st.fragment_shader) == abi.FS_TEX_X_VCOLOR:
            t = st.texture
            tex.add("f%d.m%d.l%d" % (int(t.min_filter), int(t.mipmap_mode), int(t.level_count)))
        else:
            tex.add("none")
    return "|".join([
        "batch" if batched else "single",
        "ms" + ",".join(str(s) for s in sorted(samples)),
        "cf" + ",".join(str(f) for f in sorted(fmts)),
        "tex" + ",".join(sorted(tex)),
        "tris2^%d" % _pow2(tris),
        "px2^%d" % _pow2(area),
    ])


class TuningTable:
    """Workload class -> chosen raster configuration (and how it was chosen)."""

    def __init__(self, entries: dict | None = None):
        self.entries: dict[str, dict] = dict(entries or {})

    def __contains__(self, key: str) -> bool:
        return key in self.entries

    def __len__(self) -> int:
        return len(self.entries)

    def get(self, key: str) -> dict | None:
        return self.entries.get(key)

    def record(self, key: str, best: dict, table: list) -> dict:
        """Stores the autotuner's result: best = {"bin", "hiz"}, table =
        [(candidate, {"median", "min", "max"} or ms)]."""
        cands = {}
        for c, t in table:
            name = "%s hiz%d" % (c["bin"], c["hiz"])
            cands[name] = t if isinstance(t, dict) else {"median": float(t)}
        e = {"bin": best["bin"], "hiz": int(best["hiz"]), "candidates_ms": cands,
             "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
        self.entries[key] = e
        return e

    def to_json(self) -> dict:
        return {"version": VERSION, "entries": self.entries}

    @classmethod
    def from_json(cls, d: dict) -> "TuningTable":
        if d.get("version") != VERSION:
            raise ValueError("tuning table version %r, expected %d" % (d.get("version"), VERSION))
        entries = d.get("entries", {})
        for k, e in entries.items():
            w, h = (int(x) for x in e["bin"].split("x"))
            if (w, h) not in abi.BIN_SHAPES or int(e["hiz"]) not in (0, 1):
                raise ValueError("tuning table entry %r: unsupported configuration %r" % (k, e))
        return cls(entries)

    def save(self, path: str) -> None:
        """Writes the table atomically (temporary file + rename)."""
        d = os.path.dirname(os.path.abspath(path))
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=".tuning", dir=d)
        with os.fdopen(fd, "w") as f:
            json.dump(self.to_json(), f, indent=1, sort_keys=True)
        os.replace(tmp, path)

    @classmethod
    def load(cls, path: str) -> "TuningTable":
        """The table saved at path, or an empty table when there is none."""
        if not os.path.exists(path):
            return cls()
        with open(path) as f:
            return cls.from_json(json.load(f))
