"""Procedural convex meshes in the form raw-physics' OBJ loader hands to its hull builder.

raw-physics builds every convex-hull collider from a de-indexed triangle list: float32 positions,
three per triangle, indices 0..n-1 (src/render/obj.cpp:45-106), pre-scaled in FP64 by the caller
(src/examples/examples_util.cpp:5-24) and merged into polygon faces by
collider_convex_hull_create (src/physics/collider.cpp:194-364). The meshes here are generated in
that form, wound counter-clockwise seen from outside so the hull builder's face normals point
outwards:

  cube        8 vertices at +-1, 12 triangles (6 quad faces after merging)
  icosahedron 12 vertices on the unit sphere, 20 triangles
  cylinder    2*segments vertices (radius 1, y in [-1, 1]); fan-triangulated caps merge into two
              segments-gons, each side quad into one face
  icosphere   the icosahedron subdivided once: 42 vertices, 80 triangles

No coordinate is negative zero: the hull builder deduplicates vertices by FP64 value and the
reference hashes the bit pattern, so +0/-0 would split a vertex there.
"""
from __future__ import annotations

import math
import numpy as np

__all__ = ["Mesh", "cube", "icosahedron", "cylinder", "icosphere", "hull_volume", "MESHES"]


class Mesh:
    """A de-indexed triangle mesh: positions float32 (3*T, 3), indices uint32 (3*T,)."""

    def __init__(self, name: str, tris: np.ndarray):
        tris = np.asarray(tris, dtype=np.float64)
        pos = tris.reshape(-1, 3).astype(np.float32) + np.float32(0.0)
        self.name = name
        self.positions = np.ascontiguousarray(pos, dtype=np.float32)
        self.indices = np.arange(pos.shape[0], dtype=np.uint32)

    @property
    def num_triangles(self) -> int:
        return self.positions.shape[0] // 3


def _orient_outward(tris: np.ndarray) -> np.ndarray:
    """Flip any triangle whose normal points towards the (origin-centred) mesh interior."""
    out = []
    for t in tris:
        a, b, c = (np.asarray(v, dtype=np.float64) for v in t)
        n = np.cross(b - a, c - a)
        if np.dot(n, (a + b + c) / 3.0) < 0.0:
            out.append([a, c, b])
        else:
            out.append([a, b, c])
    return np.asarray(out)


def cube() -> Mesh:
    tris = []
    for axis in range(3):
        for sign in (-1.0, 1.0):
            u, v = [(a) for a in range(3) if a != axis]
            corners = []
            for su, sv in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                p = [0.0, 0.0, 0.0]
                p[axis] = sign
                p[u] = float(su)
                p[v] = float(sv)
                corners.append(p)
            tris.append([corners[0], corners[1], corners[2]])
            tris.append([corners[0], corners[2], corners[3]])
    return Mesh("cube", _orient_outward(np.asarray(tris)))


def _icosahedron_vertices() -> np.ndarray:
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    v = []
    for a in (-1.0, 1.0):
        for b in (-phi, phi):
            v.append([0.0, a, b])
            v.append([a, b, 0.0])
            v.append([b, 0.0, a])
    v = np.asarray(v, dtype=np.float64)
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _icosahedron_faces(v: np.ndarray) -> list:
    n = len(v)
    d = np.linalg.norm(v[:, None, :] - v[None, :, :], axis=2)
    edge = np.min(d[d > 1e-9])
    adj = np.abs(d - edge) < 1e-6
    faces = []
    for i in range(n):
        for j in range(i + 1, n):
            if not adj[i, j]:
                continue
            for k in range(j + 1, n):
                if adj[i, k] and adj[j, k]:
                    faces.append((i, j, k))
    return faces


def icosahedron() -> Mesh:
    v = _icosahedron_vertices()
    tris = [[v[i], v[j], v[k]] for i, j, k in _icosahedron_faces(v)]
    return Mesh("icosahedron", _orient_outward(np.asarray(tris)))


def icosphere() -> Mesh:
    v = list(_icosahedron_vertices())
    faces = _icosahedron_faces(np.asarray(v))
    mid = {}

    def midpoint(i, j):
        key = (min(i, j), max(i, j))
        if key not in mid:
            m = (v[i] + v[j]) / 2.0
            v.append(m / np.linalg.norm(m))
            mid[key] = len(v) - 1
        return mid[key]

    tris = []
    for i, j, k in faces:
        a, b, c = midpoint(i, j), midpoint(j, k), midpoint(k, i)
        for t in ((i, a, c), (a, j, b), (c, b, k), (a, b, c)):
            tris.append([v[t[0]], v[t[1]], v[t[2]]])
    return Mesh("icosphere", _orient_outward(np.asarray(tris)))


def cylinder(segments: int = 32) -> Mesh:
    ang = 2.0 * math.pi * np.arange(segments) / segments
    ring = np.stack([np.cos(ang), np.zeros(segments), np.sin(ang)], axis=1)
    ring = np.round(ring, 15) + 0.0
    top = ring + np.array([0.0, 1.0, 0.0])
    bot = ring + np.array([0.0, -1.0, 0.0])
    tris = []
    for k in range(1, segments - 1):
        tris.append([top[0], top[k], top[k + 1]])
        tris.append([bot[0], bot[k + 1], bot[k]])
    for k in range(segments):
        k1 = (k + 1) % segments
        tris.append([bot[k], top[k], top[k1]])
        tris.append([bot[k], top[k1], bot[k1]])
    return Mesh("cylinder%d" % segments, _orient_outward(np.asarray(tris)))


def hull_volume(mesh: Mesh, scale=(1.0, 1.0, 1.0)) -> float:
    """Volume enclosed by the (scaled) triangle mesh, by the divergence theorem."""
    p = mesh.positions.astype(np.float64) * np.asarray(scale, dtype=np.float64)
    t = p.reshape(-1, 3, 3)
    return float(np.sum(np.einsum("ij,ij->i", t[:, 0], np.cross(t[:, 1], t[:, 2]))) / 6.0)


MESHES = {
    "cube": cube,
    "icosahedron": icosahedron,
    "cylinder32": lambda: cylinder(32),
    "icosphere42": icosphere,
}
