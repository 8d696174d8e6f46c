"""ctypes binding of the oracle harness (oracle/harness.h) — TEST INFRASTRUCTURE ONLY.

Loads either oracle/_build/liboracle.so (the plain-C restatement, kind "port") or
oracle/_ref/libref_harness.so (the reference's own physics sources compiled headless, kind
"reference"), and drives it with a rawphys.scenes.Scene. Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this module; it is the checker, never the thing measured.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_harness.so")
STATE_DOUBLES = 28
CONTACT_DOUBLES = 9

_D3 = C.c_double * 3
_D4 = C.c_double * 4


def build(ref: bool = False, ref_dir: str | None = None) -> None:
    """Compile the port (always) and, when the reference checkout is present, the reference
    (from ref_dir, else the Makefile's REF_DIR default)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if ref:
        extra = ["REF_DIR=" + os.path.abspath(ref_dir)] if ref_dir else []
        subprocess.run(["make", "-s", "-C", HERE, "ref", *extra], check=True)


def reference_available() -> bool:
    return os.path.exists(REF_LIB)


class Oracle:
    """One loaded harness library. Each instance of a kind shares process-global state, so use
    one scene at a time per library (reset() starts a new one)."""

    _cache = {}

    def __init__(self, kind: str = "port"):
        path = PORT_LIB if kind == "port" else REF_LIB
        if path not in Oracle._cache:
            if not os.path.exists(path):
                raise FileNotFoundError(path)
            lib = C.CDLL(path)
            d, i, u = C.c_double, C.c_int, C.c_uint32
            P = C.POINTER
            sig = {
                "orc_reset": (None, []),
                "orc_mesh_add": (i, [P(C.c_float), u, P(u), u]),
                "orc_colliders_begin": (None, []),
                "orc_colliders_add_hull": (i, [i, P(d)]),
                "orc_colliders_add_sphere": (i, [C.c_float]),
                "orc_entity_create": (i, [P(d), P(d), d, i, d, d, d]),
                "orc_entity_set_velocity": (None, [i, P(d), P(d)]),
                "orc_entity_add_force": (None, [i, P(d), P(d), i]),
                "orc_entity_get_inverse_mass": (d, [i]),
                "orc_entity_get_inertia": (None, [i, P(d), P(d)]),
                "orc_entity_get_radius": (d, [i]),
                "orc_constraint_positional": (i, [i, i, P(d), P(d), d, P(d)]),
                "orc_constraint_mutual_orientation": (i, [i, i, d]),
                "orc_constraint_hinge": (i, [i, i, P(d), P(d), d, i, i, i, i, i, d, d]),
                "orc_constraint_spherical": (i, [i, i, P(d), P(d), i, i, i, i, d, d, d, d]),
                "orc_step": (None, [d, u, u, i, d]),
                "orc_num_entities": (u, []),
                "orc_get_state": (None, [P(d)]),
                "orc_set_state": (None, [P(d)]),
                "orc_broad_pairs": (u, [P(u), u]),
                "orc_contacts": (u, [i, i, P(d), u]),
                "orc_gjk_epa": (i, [i, i, P(d)]),
                "orc_manifold": (u, [i, i, P(d), d, P(d), u]),
                "orc_hull_topology": (i, [i, i, i, P(C.c_int32), P(C.c_int32), C.c_int32, P(C.c_int32)]),
                "orc_hull_geometry": (i, [i, i, P(d), P(d), C.c_int32, C.c_int32, P(C.c_int32)]),
                "orc_last_contacts": (u, [P(C.c_int32), P(d), u]),
                "orc_obj_parse": (u, [C.c_char_p, P(C.c_float), u]),
                "orc_last_error": (i, []),
            }
            for name, (res, args) in sig.items():
                if not hasattr(lib, name):   # orc_last_contacts / orc_last_error: port only; orc_obj_parse: reference only
                    continue
                f = getattr(lib, name)
                f.restype = res
                f.argtypes = args
            Oracle._cache[path] = lib
        self.kind = kind
        self.lib = Oracle._cache[path]
        self.scene = None

    def error_bits(self) -> int:
        """Port only: the reference assert conditions met since the scene was loaded (orc_last_error):
        2 EPA face normal vanishes, 4 EPA polytope coplanar with the origin, 8 parallel skew lines,
        1 any other."""
        return int(self.lib.orc_last_error())

    def obj_corners(self, path: str) -> np.ndarray:
        """Reference harness only: the face-corner positions (FP32) the reference's OBJ reader emits
        for a file, in its order (obj_parse, src/render/obj.cpp:7-80)."""
        f = self.lib.orc_obj_parse
        n = f(os.fsencode(path), None, 0)
        out = np.zeros((max(n, 1), 3), dtype=np.float32)
        f(os.fsencode(path), out.ctypes.data_as(C.POINTER(C.c_float)), n)
        return out[:n]

    # -- scene -----------------------------------------------------------------------------
    def load(self, scene) -> "Oracle":
        L = self.lib
        L.orc_reset()
        for m in scene.meshes:
            pos = np.ascontiguousarray(m.positions, dtype=np.float32)
            idx = np.ascontiguousarray(m.indices, dtype=np.uint32)
            L.orc_mesh_add(pos.ctypes.data_as(C.POINTER(C.c_float)), pos.shape[0],
                           idx.ctypes.data_as(C.POINTER(C.c_uint32)), idx.shape[0])
        for b in range(scene.num_bodies):
            L.orc_colliders_begin()
            for c in scene.colliders[b]:
                if c.kind == "hull":
                    L.orc_colliders_add_hull(c.mesh, _D3(*c.scale))
                else:
                    L.orc_colliders_add_sphere(float(c.radius))
            L.orc_entity_create(_D3(*scene.pos[b]), _D4(*scene.rot[b]), float(scene.mass[b]), int(scene.fixed[b]),
                                float(scene.mus[b]), float(scene.mud[b]), float(scene.rest[b]))
            L.orc_entity_set_velocity(b, _D3(*scene.vel[b]), _D3(*scene.omega[b]))
        for c in scene.constraints:
            if c.kind == "positional":
                L.orc_constraint_positional(c.e1, c.e2, _D3(*c.r1), _D3(*c.r2), c.compliance, _D3(*c.distance))
            elif c.kind == "mutual_orientation":
                L.orc_constraint_mutual_orientation(c.e1, c.e2, c.compliance)
            elif c.kind == "hinge":
                L.orc_constraint_hinge(c.e1, c.e2, _D3(*c.r1), _D3(*c.r2), c.compliance, c.axis1, c.axis2,
                                       int(c.limited), c.limit_axis1, c.limit_axis2, c.lower, c.upper)
            elif c.kind == "spherical":
                L.orc_constraint_spherical(c.e1, c.e2, _D3(*c.r1), _D3(*c.r2), c.swing_axis1, c.swing_axis2,
                                           c.twist_axis1, c.twist_axis2, c.swing_lower, c.swing_upper,
                                           c.twist_lower, c.twist_upper)
            else:
                raise ValueError(c.kind)
        self.scene = scene
        return self

    def step(self, n: int = 1, dt=None, substeps=None, pos_iters=None, collisions=None, gravity=None) -> None:
        s = self.scene
        dt = s.dt if dt is None else dt
        substeps = s.substeps if substeps is None else substeps
        pos_iters = s.pos_iters if pos_iters is None else pos_iters
        collisions = s.collisions if collisions is None else collisions
        gravity = s.gravity if gravity is None else gravity
        for _ in range(n):
            self.lib.orc_step(dt, substeps, pos_iters, int(collisions), gravity)

    def add_force(self, e: int, position, force, local=False) -> None:
        self.lib.orc_entity_add_force(e, _D3(*position), _D3(*force), int(local))

    # -- state -----------------------------------------------------------------------------
    def num_entities(self) -> int:
        return int(self.lib.orc_num_entities())

    def get_state(self) -> np.ndarray:
        n = self.num_entities()
        out = np.zeros((n, STATE_DOUBLES), dtype=np.float64)
        self.lib.orc_get_state(out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def set_state(self, st: np.ndarray) -> None:
        st = np.ascontiguousarray(st, dtype=np.float64)
        assert st.shape == (self.num_entities(), STATE_DOUBLES)
        self.lib.orc_set_state(st.ctypes.data_as(C.POINTER(C.c_double)))

    def inverse_mass(self, e: int) -> float:
        return float(self.lib.orc_entity_get_inverse_mass(e))

    def inertia(self, e: int):
        I = np.zeros(9)
        Ii = np.zeros(9)
        self.lib.orc_entity_get_inertia(e, I.ctypes.data_as(C.POINTER(C.c_double)), Ii.ctypes.data_as(C.POINTER(C.c_double)))
        return I.reshape(3, 3), Ii.reshape(3, 3)

    def radius(self, e: int) -> float:
        return float(self.lib.orc_entity_get_radius(e))

    def broad_pairs(self) -> np.ndarray:
        cap = 1 << 16
        while True:
            out = np.zeros(2 * cap, dtype=np.uint32)
            n = self.lib.orc_broad_pairs(out.ctypes.data_as(C.POINTER(C.c_uint32)), cap)
            if n <= cap:
                return out[: 2 * n].reshape(-1, 2)
            cap = int(n)

    def contacts(self, e1: int, e2: int) -> np.ndarray:
        cap = 256
        out = np.zeros(cap * CONTACT_DOUBLES)
        n = self.lib.orc_contacts(e1, e2, out.ctypes.data_as(C.POINTER(C.c_double)), cap)
        return out[: min(n, cap) * CONTACT_DOUBLES].reshape(-1, CONTACT_DOUBLES)

    def hull_topology(self, e: int, k: int = 0):
        """(vertices (nv,3), normals (nf,3), {table: (start, data)}) of collider k of entity e."""
        nf = C.c_int32()
        nv = self.lib.orc_hull_geometry(e, k, None, None, 0, 0, C.byref(nf))
        verts, normals = np.zeros((nv, 3)), np.zeros((nf.value, 3))
        self.lib.orc_hull_geometry(e, k, verts.ctypes.data_as(C.POINTER(C.c_double)),
                                   normals.ctypes.data_as(C.POINTER(C.c_double)), nv, nf.value, C.byref(nf))
        tables = {}
        for which in range(4):
            nd = C.c_int32()
            rows = self.lib.orc_hull_topology(e, k, which, None, None, 0, C.byref(nd))
            start = np.zeros(rows + 1, dtype=np.int32)
            data = np.zeros(max(nd.value, 1), dtype=np.int32)
            self.lib.orc_hull_topology(e, k, which, start.ctypes.data_as(C.POINTER(C.c_int32)),
                                       data.ctypes.data_as(C.POINTER(C.c_int32)), nd.value, C.byref(nd))
            tables[which] = (start, data[: nd.value])
        return verts, normals, tables

    def last_contacts(self):
        """(pairs (k,2), constraints (k,11)) of the last substep of the last step (port only)."""
        cap = 1 << 16
        pairs = np.zeros(2 * cap, dtype=np.int32)
        out = np.zeros(11 * cap)
        n = self.lib.orc_last_contacts(pairs.ctypes.data_as(C.POINTER(C.c_int32)), out.ctypes.data_as(C.POINTER(C.c_double)), cap)
        n = min(n, cap)
        return pairs[: 2 * n].reshape(-1, 2), out[: 11 * n].reshape(-1, 11)

    def gjk_epa(self, e1: int, e2: int):
        out = np.zeros(4)
        r = self.lib.orc_gjk_epa(e1, e2, out.ctypes.data_as(C.POINTER(C.c_double)))
        return int(r), out

    def manifold(self, e1: int, e2: int, normal, penetration: float) -> np.ndarray:
        """clipping_get_contact_manifold of the two entities' first colliders for the given EPA
        result (normal from e1 to e2, penetration)."""
        cap = 256
        n = np.ascontiguousarray(normal, dtype=np.float64)
        out = np.zeros(cap * CONTACT_DOUBLES)
        k = self.lib.orc_manifold(e1, e2, n.ctypes.data_as(C.POINTER(C.c_double)), float(penetration),
                                  out.ctypes.data_as(C.POINTER(C.c_double)), cap)
        return out[: min(k, cap) * CONTACT_DOUBLES].reshape(-1, CONTACT_DOUBLES)
