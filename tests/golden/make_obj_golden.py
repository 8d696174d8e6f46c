"""Generate tests/golden/obj_corners.npz from the reference's own OBJ reader.

Runs obj_parse (raw-physics' src/render/obj.cpp, with the vendored tinyobj loader, compiled into
oracle/_ref/libref_harness.so by oracle/Makefile) on a few OBJ files written by `obj_cases()` —
triangles with texture / normal indices, quads, hexagons, negative indices — and stores, per case,
the OBJ text and the face-corner positions (FP32) the reader emits, in its order. rp_hull_from_obj
must hand the same corners to the hull builder. Also writes cube_half.rphull: the hull cache file
rp_hull_save produces for the triangulated cube of tri_cube scaled by 0.5 (the format's fixture).
Regenerate with
    make -C oracle ref && python tests/golden/make_obj_golden.py
"""
from __future__ import annotations

import math
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def _prism(n: int, negative: bool = False, decimals: int = 6) -> str:
    """An n-gonal prism of radius 1 and height 2: two n-gon caps and n quads, counter-clockwise
    seen from outside; positions rotated by 0.3 rad so that no cap edge is axis-aligned."""
    lines = ["# %d-gonal prism" % n]
    for z in (-1.0, 1.0):
        for k in range(n):
            a = 2.0 * math.pi * k / n + 0.3
            lines.append("v %.*f %.*f %.*f" % (decimals, math.cos(a), decimals, math.sin(a), decimals, z))
    nv = 2 * n

    def r(i):                       # 0-based position index -> OBJ reference
        return str(i - nv) if negative else str(i + 1)
    lines.append("f " + " ".join(r(k) for k in reversed(range(n))))          # bottom, facing -z
    lines.append("f " + " ".join(r(n + k) for k in range(n)))                # top, facing +z
    for k in range(n):
        k2 = (k + 1) % n
        lines.append("f %s %s %s %s" % (r(k), r(k2), r(n + k2), r(n + k)))
    return "\n".join(lines) + "\n"


def _tri_cube() -> str:
    v = [(x, y, z) for x in (-1.0, 1.0) for y in (-1.0, 1.0) for z in (-1.0, 1.0)]
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    lines = ["# triangulated cube with texture and normal indices"] + ["v %.6f %.6f %.6f" % p for p in v]
    lines += ["vt 0 0", "vt 1 0", "vt 1 1", "vn 0 0 1"]
    for q in quads:
        for t in ((q[0], q[1], q[2]), (q[0], q[2], q[3])):
            lines.append("f " + " ".join("%d/%d/1" % (i + 1, j + 1) for j, i in enumerate(t)))
    return "\n".join(lines) + "\n"


def obj_cases():
    return {
        "tri_cube": _tri_cube(),
        "quad_prism4": _prism(4),
        "hex_prism": _prism(6),
        "hex_prism_negative": _prism(6, negative=True),
        "oct_prism": _prism(8, decimals=4),
    }


def write_cache_fixture() -> None:
    sys.path.insert(0, os.path.join(ROOT, "raw-physics_gb300"))
    import rawphys
    rawphys.load_library()
    w = rawphys.World(-1, "fp64")
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "tri_cube.obj")
        with open(path, "w") as f:
            f.write(_tri_cube())
        h = w.hull_from_obj(path, (0.5, 0.5, 0.5))
        w.hull_save(h, os.path.join(HERE, "cube_half.rphull"))
    w.close()


def main() -> None:
    write_cache_fixture()
    from oracle.oracle import Oracle, reference_available
    if not reference_available():
        raise SystemExit("the reference harness is not built: make -C oracle ref")
    o = Oracle("ref")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, text in obj_cases().items():
            path = os.path.join(d, name + ".obj")
            with open(path, "w") as f:
                f.write(text)
            out[name + "_text"] = np.array(text)
            out[name + "_corners"] = o.obj_corners(path)
    np.savez_compressed(os.path.join(HERE, "obj_corners.npz"), **out)
    print("wrote", os.path.join(HERE, "obj_corners.npz"), sorted(k for k in out if k.endswith("_corners")))


if __name__ == "__main__":
    main()
