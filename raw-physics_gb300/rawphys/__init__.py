"""Python binding of the GB300 rigid-body step (the C ABI of include/rp.h) via ctypes.

The library is built in place by raw-physics_gb300/build.py; importing this package never builds
or falls back to anything: World() raises if librawphys_gb300.so is missing or no CUDA device is
present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.environ.get("RAWPHYS_LIB") or os.path.join(PKG_DIR, "librawphys_gb300.so")

STATE_DOUBLES = 28
CONTACT_DOUBLES = 9
PRECISION = {"fp32": 0, "fp64": 1}
COLLIDER_SPHERE, COLLIDER_HULL = 0, 1
ERRORS = {0: "RP_OK", -1: "RP_ERR_INVALID", -2: "RP_ERR_CUDA", -3: "RP_ERR_NO_DEVICE", -4: "RP_ERR_CAPACITY",
          -5: "RP_ERR_DEGENERATE", -6: "RP_ERR_TIMEOUT", -7: "RP_ERR_STATE"}
STATUS_BITS = {1 << 0: "PAIR_OVERFLOW", 1 << 1: "CONTACT_OVERFLOW", 1 << 2: "EPA_OVERFLOW", 1 << 3: "CLIP_OVERFLOW",
               1 << 4: "BARRIER_TIMEOUT", 1 << 5: "DEGENERATE", 1 << 6: "LEVEL_OVERFLOW", 1 << 8: "EPA_NOT_CONVERGED",
               1 << 9: "DEG_EPA_NORMAL", 1 << 10: "DEG_EPA_COPLANAR", 1 << 11: "DEG_SKEW"}

# every exported symbol of include/rp.h with its ctypes signature
_d, _i, _u, _u64 = C.c_double, C.c_int32, C.c_uint32, C.c_uint64
_P = C.POINTER
_W = C.c_void_p


class ColliderDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("hull", C.c_int32), ("radius", C.c_float)]


SIGNATURES = {
    "rp_world_create": (_i, [_P(_W), _i, _i]),
    "rp_world_destroy": (None, [_W]),
    "rp_world_set_stream": (_i, [_W, C.c_void_p]),
    "rp_last_error": (C.c_char_p, []),
    "rp_scene_create": (_i, [_W, _P(_i)]),
    "rp_hull_create": (_i, [_W, _P(_d), _u, _P(_u), _u, _P(_i)]),
    "rp_hull_create_from_topology": (_i, [_W, _P(_d), _i, _P(_d), _i, _P(_i), _P(_i), _P(_i), _P(_i), _P(_i), _P(_i),
                                          _P(_i), _P(_i), _P(_i)]),
    "rp_hull_info": (_i, [_W, _i, _P(_i), _P(_i)]),
    "rp_hull_topology": (_i, [_W, _i, _i, _P(_i), _P(_i), _i, _P(_i), _P(_i)]),
    "rp_hull_geometry": (_i, [_W, _i, _P(_d), _P(_d)]),
    "rp_hull_from_obj": (_i, [_W, C.c_char_p, _P(_d), _P(_i)]),
    "rp_hull_save": (_i, [_W, _i, C.c_char_p]),
    "rp_hull_load": (_i, [_W, C.c_char_p, _P(_i)]),
    "rp_hull_face": (_i, [_W, _i, _i, _P(_d), _P(_i), _i, _P(_i)]),
    "rp_entity_create": (_i, [_W, _i, _P(_d), _P(_d), _d, _i, _P(ColliderDesc), _u, _d, _d, _d, _P(_i)]),
    "rp_entity_set_velocity": (_i, [_W, _i, _P(_d), _P(_d)]),
    "rp_entities_create": (_i, [_W, _u, _P(_i), _P(_d), _P(_d), _P(_d), _P(_i), _P(ColliderDesc), _P(_d), _P(_d),
                                _P(_d), _P(_d), _P(_d), _P(_i)]),
    "rp_entity_add_force": (_i, [_W, _i, _P(_d), _P(_d), _i]),
    "rp_entity_clear_forces": (_i, [_W, _i]),
    "rp_world_set_gravity": (_i, [_W, _d]),
    "rp_entity_get_mass_properties": (_i, [_W, _i, _P(_d), _P(_d), _P(_d), _P(_d)]),
    "rp_entity_set_mass_properties": (_i, [_W, _i, _d, _P(_d), _P(_d), _d]),
    "rp_num_entities": (_i, [_W]),
    "rp_constraint_positional": (_i, [_W, _i, _i, _P(_d), _P(_d), _d, _P(_d), _P(_i)]),
    "rp_constraint_mutual_orientation": (_i, [_W, _i, _i, _d, _P(_i)]),
    "rp_constraint_hinge": (_i, [_W, _i, _i, _P(_d), _P(_d), _d, _i, _i, _i, _i, _i, _d, _d, _P(_i)]),
    "rp_constraint_spherical": (_i, [_W, _i, _i, _P(_d), _P(_d), _i, _i, _i, _i, _d, _d, _d, _d, _P(_i)]),
    "rp_simulate": (_i, [_W, _d, _u, _u, _i, _u]),
    "rp_sync": (_i, [_W]),
    "rp_last_status": (_i, [_W, _P(_u)]),
    "rp_state_get": (_i, [_W, _P(_d)]),
    "rp_state_set": (_i, [_W, _P(_d)]),
    "rp_broad_pairs": (_i, [_W, _i, _P(_u), _u, _P(_u)]),
    "rp_contacts": (_i, [_W, _i, _i, _P(_d), _u, _P(_u)]),
    "rp_counters": (_i, [_W, _P(_u64)]),
    "rp_world_set_mode": (_i, [_W, _i]),
    "rp_world_set_wait_limit": (_i, [_W, _u64]),
    "rp_world_set_sweep_order": (_i, [_W, _i]),
    "rp_world_set_sweep_assignment": (_i, [_W, _i]),
    "rp_transformed_hulls_size": (_i, [_W, _P(_u64), _P(_u64)]),
    "rp_transformed_hulls": (_i, [_W, _P(_d), _P(_d)]),
    "rp_last_schedule": (_i, [_W, _i, _i, _P(_i), _P(_i), _u, _P(_u)]),
    "rp_degenerate_info": (_i, [_W, _P(C.c_int64)]),
    "rp_adjoint_profile": (_i, [_W, _P(_d)]),
    "rp_adjoint_trajectory": (_i, [_W, _d, _u, _u, _i, _u, _u, _P(_i), _P(_d), _P(_d), _P(_d), _P(_d), _P(_d), _P(_d)]),
    "rp_autotune": (_i, [_W, _d, _u, _u, _i, _u, _P(_i)]),
    "rp_kernel_launches": (_u64, [_W]),
    "rp_transfer_bytes": (_i, [_W, _P(_u64)]),
    "rp_phase_times": (_i, [_W, _P(_d)]),
    "rp_last_contacts": (_i, [_W, _i, _P(_i), _P(_d), _u, _P(_u)]),
    "rp_contacts_noalloc": (_i, [_W, _i, _i, _P(_d), _u, _P(_u)]),
    "rp_set_timing": (_i, [_W, _i]),
    "rp_last_step_ms": (_i, [_W, _P(_d)]),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """Load librawphys_gb300.so and bind every C ABI symbol (raises if the library is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError("raw-physics GB300 extension not built: %s (run raw-physics_gb300/build.py)" % path)
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


class RPError(RuntimeError):
    pass


def _dp(a):
    return a.ctypes.data_as(_P(_d))


def _arr(v, n=3):
    return (C.c_double * n)(*[float(x) for x in v])


class World:
    """One rp_world: a set of scenes stepped together on one GPU."""

    def __init__(self, device: int = 0, precision: str = "fp32"):
        self.lib = load_library()
        self.h = _W()
        self._check(self.lib.rp_world_create(C.byref(self.h), device, PRECISION[precision]))
        self.precision = precision
        self.scene = None
        self._hulls = {}

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.rp_last_error().decode()
            raise RPError("%s: %s" % (ERRORS.get(rc, rc), msg))
        return rc

    def close(self):
        if self.h:
            self.lib.rp_world_destroy(self.h)
            self.h = _W()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- construction ----------------------------------------------------------------------
    def new_scene(self) -> int:
        s = _i()
        self._check(self.lib.rp_scene_create(self.h, C.byref(s)))
        return s.value

    def hull(self, vertices: np.ndarray, indices: np.ndarray) -> int:
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, dtype=np.uint32)
        out = _i()
        self._check(self.lib.rp_hull_create(self.h, _dp(v), v.shape[0], idx.ctypes.data_as(_P(_u)), idx.shape[0],
                                            C.byref(out)))
        return out.value

    def hull_from_obj(self, path: str, scale=(1.0, 1.0, 1.0)) -> int:
        """A hull from an OBJ file, as the reference's examples build theirs (rp_hull_from_obj)."""
        sc = np.ascontiguousarray(scale, dtype=np.float64)
        out = _i()
        self._check(self.lib.rp_hull_from_obj(self.h, os.fsencode(path), _dp(sc), C.byref(out)))
        return out.value

    def hull_save(self, hull: int, path: str) -> None:
        """Write a built hull's topology to a binary cache file (rp_hull_save)."""
        self._check(self.lib.rp_hull_save(self.h, hull, os.fsencode(path)))

    def hull_load(self, path: str) -> int:
        """A hull restored from a cache file written by hull_save (rp_hull_load)."""
        out = _i()
        self._check(self.lib.rp_hull_load(self.h, os.fsencode(path), C.byref(out)))
        return out.value

    def hull_faces(self, hull: int):
        nv, nf = _i(), _i()
        self._check(self.lib.rp_hull_info(self.h, hull, C.byref(nv), C.byref(nf)))
        faces = []
        for f in range(nf.value):
            n = (C.c_double * 3)()
            el = (C.c_int32 * 256)()
            ne = _i()
            self._check(self.lib.rp_hull_face(self.h, hull, f, n, el, 256, C.byref(ne)))
            faces.append((tuple(n), list(el[: ne.value])))
        return nv.value, faces

    def hull_topology(self, hull: int):
        """(vertices (nv,3), normals (nf,3), {table: (start, data)}) of a hull, as built on the host."""
        nv, nf = _i(), _i()
        self._check(self.lib.rp_hull_info(self.h, hull, C.byref(nv), C.byref(nf)))
        verts, normals = np.zeros((nv.value, 3)), np.zeros((nf.value, 3))
        self._check(self.lib.rp_hull_geometry(self.h, hull, _dp(verts), _dp(normals)))
        tables = {}
        for which in range(4):
            rows, nd = _i(), _i()
            self._check(self.lib.rp_hull_topology(self.h, hull, which, None, None, 0, C.byref(rows), C.byref(nd)))
            start = np.zeros(rows.value + 1, dtype=np.int32)
            data = np.zeros(max(nd.value, 1), dtype=np.int32)
            self._check(self.lib.rp_hull_topology(self.h, hull, which, start.ctypes.data_as(_P(_i)),
                                                  data.ctypes.data_as(_P(_i)), nd.value, C.byref(rows), C.byref(nd)))
            tables[which] = (start, data[: nd.value])
        return verts, normals, tables

    def entity(self, scene, pos, rot, mass, fixed, colliders, mus, mud, rest) -> int:
        arr = (ColliderDesc * len(colliders))(*colliders)
        out = _i()
        self._check(self.lib.rp_entity_create(self.h, scene, _arr(pos), _arr(rot, 4), float(mass), int(fixed), arr,
                                              len(colliders), float(mus), float(mud), float(rest), C.byref(out)))
        return out.value

    def set_velocity(self, e, v, w):
        self._check(self.lib.rp_entity_set_velocity(self.h, e, _arr(v), _arr(w)))

    def add_force(self, e, position, force, local=False):
        self._check(self.lib.rp_entity_add_force(self.h, e, _arr(position), _arr(force), int(local)))

    def set_gravity(self, g: float):
        self._check(self.lib.rp_world_set_gravity(self.h, float(g)))

    def mass_properties(self, e):
        invm = _d()
        I, Ii = (C.c_double * 9)(), (C.c_double * 9)()
        r = _d()
        self._check(self.lib.rp_entity_get_mass_properties(self.h, e, C.byref(invm), I, Ii, C.byref(r)))
        return invm.value, np.array(I[:]).reshape(3, 3), np.array(Ii[:]).reshape(3, 3), r.value

    def set_mass_properties(self, e, inverse_mass, inertia, inverse_inertia, radius):
        I = np.ascontiguousarray(inertia, dtype=np.float64).reshape(9)
        Ii = np.ascontiguousarray(inverse_inertia, dtype=np.float64).reshape(9)
        self._check(self.lib.rp_entity_set_mass_properties(self.h, e, float(inverse_mass), _dp(I), _dp(Ii), float(radius)))

    def constraint(self, c, base: int = 0):
        o = _i()
        e1, e2 = base + c.e1, base + c.e2
        if c.kind == "positional":
            rc = self.lib.rp_constraint_positional(self.h, e1, e2, _arr(c.r1), _arr(c.r2), c.compliance, _arr(c.distance), C.byref(o))
        elif c.kind == "mutual_orientation":
            rc = self.lib.rp_constraint_mutual_orientation(self.h, e1, e2, c.compliance, C.byref(o))
        elif c.kind == "hinge":
            rc = self.lib.rp_constraint_hinge(self.h, e1, e2, _arr(c.r1), _arr(c.r2), c.compliance, c.axis1, c.axis2,
                                              int(c.limited), c.limit_axis1, c.limit_axis2, c.lower, c.upper, C.byref(o))
        elif c.kind == "spherical":
            rc = self.lib.rp_constraint_spherical(self.h, e1, e2, _arr(c.r1), _arr(c.r2), c.swing_axis1, c.swing_axis2,
                                                  c.twist_axis1, c.twist_axis2, c.swing_lower, c.swing_upper,
                                                  c.twist_lower, c.twist_upper, C.byref(o))
        else:
            raise ValueError(c.kind)
        self._check(rc)
        return o.value

    def load(self, scene, scene_id: int = 0) -> int:
        """Create every mesh hull, entity and constraint of a rawphys.scenes.Scene in scene_id.
        Returns the index of the scene's first entity."""
        first = None
        for b in range(scene.num_bodies):
            descs = []
            for c in scene.colliders[b]:
                if c.kind == "hull":
                    m = scene.meshes[c.mesh]
                    key = (id(m), tuple(c.scale))
                    if key not in self._hulls:
                        verts = m.positions.astype(np.float64) * np.asarray(c.scale, dtype=np.float64)
                        self._hulls[key] = self.hull(verts, m.indices)
                    descs.append(ColliderDesc(COLLIDER_HULL, self._hulls[key], 0.0))
                else:
                    descs.append(ColliderDesc(COLLIDER_SPHERE, -1, float(c.radius)))
            e = self.entity(scene_id, scene.pos[b], scene.rot[b], scene.mass[b], scene.fixed[b], descs,
                            scene.mus[b], scene.mud[b], scene.rest[b])
            if first is None:
                first = e
            if np.any(scene.vel[b]) or np.any(scene.omega[b]):
                self.set_velocity(e, scene.vel[b], scene.omega[b])
        for c in scene.constraints:
            self.constraint(c, base=first)
        self.set_gravity(scene.gravity)
        self.scene = scene
        return first

    def load_batch(self, batch) -> int:
        """Create every scene of a rawphys.scenes.SceneBatch (scene s of the batch becomes world scene
        first_scene + s; the world's scene 0 is used first when it is still empty). Returns the index
        of the first entity."""
        base = 0 if self.num_entities() == 0 else self.new_scene()
        for _ in range(batch.num_scenes - 1):
            self.new_scene()
        keys = {}
        hull_of = np.zeros(batch.num_bodies, dtype=np.int32)
        for i in range(batch.num_bodies):
            key = (int(batch.mesh[i]), tuple(batch.scale[i]))
            h = keys.get(key)
            if h is None:
                m = batch.meshes[key[0]]
                h = self.hull(m.positions.astype(np.float64) * np.asarray(key[1], dtype=np.float64), m.indices)
                keys[key] = h
            hull_of[i] = h
        cols = (ColliderDesc * batch.num_bodies)()
        for i in range(batch.num_bodies):
            cols[i].type = COLLIDER_HULL
            cols[i].hull = int(hull_of[i])
            cols[i].radius = 0.0
        scene = np.ascontiguousarray(batch.scene + base, dtype=np.int32)
        c64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        pos, rot, mass, vel, om = c64(batch.pos), c64(batch.rot), c64(batch.mass), c64(batch.vel), c64(batch.omega)
        mus, mud, rest = c64(batch.mus), c64(batch.mud), c64(batch.rest)
        fixed = np.ascontiguousarray(batch.fixed, dtype=np.int32)
        first = _i()
        self._check(self.lib.rp_entities_create(self.h, batch.num_bodies, scene.ctypes.data_as(_P(_i)), _dp(pos), _dp(rot),
                                                _dp(mass), fixed.ctypes.data_as(_P(_i)), cols, _dp(mus), _dp(mud),
                                                _dp(rest), _dp(vel), _dp(om), C.byref(first)))
        for c in batch.constraints:
            self.constraint(c, base=first.value)
        self.set_gravity(batch.gravity)
        self.scene = batch
        return first.value

    # -- stepping and state ----------------------------------------------------------------
    def simulate(self, dt, substeps, pos_iters=1, collisions=True, steps=1):
        self._check(self.lib.rp_simulate(self.h, float(dt), int(substeps), int(pos_iters), int(bool(collisions)), int(steps)))

    def step(self, n: int = 1):
        s = self.scene
        self.simulate(s.dt, s.substeps, s.pos_iters, s.collisions, n)

    def sync(self):
        self._check(self.lib.rp_sync(self.h))

    def num_entities(self) -> int:
        return int(self.lib.rp_num_entities(self.h))

    def get_state(self, out: np.ndarray = None) -> np.ndarray:
        """The state records (RP_STATE_DOUBLES per entity); into `out` when given (no allocation)."""
        if out is None:
            out = np.empty((self.num_entities(), STATE_DOUBLES))
        assert out.shape == (self.num_entities(), STATE_DOUBLES) and out.dtype == np.float64 and out.flags.c_contiguous
        self._check(self.lib.rp_state_get(self.h, _dp(out)))
        return out

    def set_state(self, st: np.ndarray):
        st = np.ascontiguousarray(st, dtype=np.float64)
        assert st.shape == (self.num_entities(), STATE_DOUBLES)
        self._check(self.lib.rp_state_set(self.h, _dp(st)))

    def status(self) -> int:
        b = _u()
        self._check(self.lib.rp_last_status(self.h, C.byref(b)))
        return b.value

    def broad_pairs(self, scene: int = 0) -> np.ndarray:
        cap = 1 << 16
        while True:
            out = np.zeros(2 * cap, dtype=np.uint32)
            n = _u()
            rc = self.lib.rp_broad_pairs(self.h, scene, out.ctypes.data_as(_P(_u)), cap, C.byref(n))
            if rc == 0 and n.value <= cap:
                return out[: 2 * n.value].reshape(-1, 2)
            if rc not in (0, -4):
                self._check(rc)
            cap = max(2 * cap, int(n.value))
            if cap > (1 << 26):
                self._check(rc)

    def contacts(self, e1: int, e2: int) -> np.ndarray:
        cap = 64
        out = np.zeros(cap * CONTACT_DOUBLES)
        n = _u()
        self._check(self.lib.rp_contacts(self.h, e1, e2, _dp(out), cap, C.byref(n)))
        return out[: min(n.value, cap) * CONTACT_DOUBLES].reshape(-1, CONTACT_DOUBLES)

    def contacts_noalloc(self, e1: int, e2: int, cap: int = 64) -> np.ndarray:
        """rp_contacts through the no-allocation entry point (static device scratch)."""
        out = np.zeros(max(cap, 1) * 9)
        n = _u()
        self._check(self.lib.rp_contacts_noalloc(self.h, e1, e2, _dp(out), cap, C.byref(n)))
        return out[: min(n.value, cap) * 9].reshape(-1, 9)

    def last_contacts(self, scene: int = 0):
        """(pairs (k,2), constraints (k,11)) of the last substep of the last simulate call."""
        cap = 1 << 16
        pairs = np.zeros(2 * cap, dtype=np.int32)
        out = np.zeros(11 * cap)
        n = _u()
        self._check(self.lib.rp_last_contacts(self.h, scene, pairs.ctypes.data_as(_P(_i)), _dp(out), cap, C.byref(n)))
        k = min(n.value, cap)
        return pairs[: 2 * k].reshape(-1, 2), out[: 11 * k].reshape(-1, 11)

    def adjoint(self, frames: int, loss_entity, target, checkpoint_every: int = 10, dt=None, substeps=None, pos_iters=None,
                collisions=None):
        """Loss |x_e(T) - target|^2 per scene after `frames` frames and its gradient with respect to
        initial velocities, masses and static / dynamic friction (rp_adjoint_trajectory). Step
        arguments default to the loaded scene's."""
        s = self.scene
        dt = s.dt if dt is None else dt
        substeps = s.substeps if substeps is None else substeps
        pos_iters = s.pos_iters if pos_iters is None else pos_iters
        collisions = bool(s.collisions) if collisions is None else bool(collisions)
        le = np.ascontiguousarray(np.atleast_1d(loss_entity), dtype=np.int32)
        tg = np.ascontiguousarray(np.reshape(target, (-1, 3)), dtype=np.float64)
        n = self.num_entities()
        loss = np.zeros(len(le))
        gv, gw, gm, gf = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n), np.zeros((n, 2))
        self._check(self.lib.rp_adjoint_trajectory(self.h, float(dt), int(substeps), int(pos_iters), int(collisions), int(frames),
                                                   int(checkpoint_every), le.ctypes.data_as(_P(_i)), _dp(tg), _dp(loss),
                                                   _dp(gv), _dp(gw), _dp(gm), _dp(gf)))
        return {"loss": loss, "grad_v": gv, "grad_w": gw, "grad_mass": gm, "grad_friction": gf}

    def adjoint_profile(self) -> dict:
        """Time split of the last adjoint's slowest scene (rp_adjoint_profile)."""
        out = np.zeros(6)
        self._check(self.lib.rp_adjoint_profile(self.h, _dp(out)))
        return {"forward_ms": out[0], "recompute_ms": out[1], "taped_ms": out[2], "reverse_ms": out[3],
                "max_tape_entries": int(out[4]), "tape_entries": int(out[5])}

    MODES = {"auto": 0, "persistent": 1, "phased": 2}

    def set_mode(self, mode: str):
        """Launch mode of a frame: "phased" (one kernel per phase, CUDA graph), "persistent" (one
        kernel per frame) or "auto"."""
        self._check(self.lib.rp_world_set_mode(self.h, self.MODES[mode]))

    def degenerate_info(self):
        """The first degenerate condition met since the last query (rp_degenerate_info): None, or
        {"bits": [names], "scene", "pair": (e1, e2), "substep"}."""
        out = np.zeros(5, dtype=np.int64)
        self._check(self.lib.rp_degenerate_info(self.h, out.ctypes.data_as(_P(C.c_int64))))
        if out[0] == 0:
            return None
        return {"bits": [v for k, v in STATUS_BITS.items() if int(out[0]) & k], "scene": int(out[1]),
                "pair": (int(out[2]), int(out[3])), "substep": int(out[4])}

    SWEEP_ORDERS = {"reference": 0, "coloured": 1}

    def transformed_hulls(self):
        """(vertices (nv, 3), normals (nf, 3)) of every hull collider at the current poses, entity by
        entity (rp_transformed_hulls: colliders_update computed on the device in FP64)."""
        nv, nn = _u64(), _u64()
        self._check(self.lib.rp_transformed_hulls_size(self.h, C.byref(nv), C.byref(nn)))
        v, n = np.zeros((max(nv.value, 1), 3)), np.zeros((max(nn.value, 1), 3))
        self._check(self.lib.rp_transformed_hulls(self.h, _dp(v), _dp(n)))
        return v[: nv.value], n[: nn.value]

    def last_schedule(self, scene: int = 0, which: int = 0):
        """(levels (n,), bodies (n, 2)) of the last substep's position (which=0) or velocity (1)
        sweep schedule: per solver node its level / colour (-1: no-op) and its dynamic entities."""
        n = _u()
        self._check(self.lib.rp_last_schedule(self.h, scene, which, None, None, 0, C.byref(n)))
        lev = np.zeros(max(n.value, 1), dtype=np.int32)
        bod = np.zeros(2 * max(n.value, 1), dtype=np.int32)
        self._check(self.lib.rp_last_schedule(self.h, scene, which, lev.ctypes.data_as(_P(_i)), bod.ctypes.data_as(_P(_i)),
                                              n.value, C.byref(n)))
        return lev[: n.value], bod[: 2 * n.value].reshape(-1, 2)

    def set_sweep_order(self, order: str):
        """Gauss-Seidel order of the sweeps: "reference" (the reference's serial order, the default)
        or "coloured" (graph-coloured; results differ from the reference's by the reordering)."""
        self._check(self.lib.rp_world_set_sweep_order(self.h, self.SWEEP_ORDERS[order]))

    def set_sweep_assignment(self, cta: int):
        """Scenes per warp or CTA in a batch's sweeps: 0 one warp per scene (default), 1 one CTA per
        scene, n >= 2 a CTA for scenes of sweep cost n or more (a launch shape: FP64 results identical,
        FP32 equal to rounding)."""
        self._check(self.lib.rp_world_set_sweep_assignment(self.h, int(cta)))

    def set_wait_limit(self, microseconds: int):
        """Bound of every device-side wait (grid barriers); a wait that runs out undoes the call and
        raises RPError(RP_ERR_TIMEOUT)."""
        self._check(self.lib.rp_world_set_wait_limit(self.h, int(microseconds)))

    def autotune(self, frames: int = 3) -> dict:
        """Pick the fastest launch configuration for the loaded scenes (the same schedule under every
        configuration: FP64 results identical, FP32 equal to rounding); returns the choice."""
        s = self.scene
        out = (_i * 4)()
        self._check(self.lib.rp_autotune(self.h, float(s.dt), int(s.substeps), int(s.pos_iters), int(bool(s.collisions)),
                                         int(frames), out))
        modes = {v: k for k, v in self.MODES.items()}
        return {"mode": modes.get(out[0], out[0]), "transform_threads": out[1],
                "batch_sweep_assignment": {0: "warp per scene", 1: "CTA per scene"}.get(out[2], "CTA for scenes of cost >= %d" % out[2]),
                "solo_level_nodes": out[3]}

    def counters(self):
        out = (C.c_uint64 * 24)()
        self._check(self.lib.rp_counters(self.h, out))
        return list(out)

    def kernel_launches(self) -> int:
        return int(self.lib.rp_kernel_launches(self.h))

    PHASES = ("broad", "islands", "schedule", "predict", "transform", "narrow", "solve", "velocity", "vsolve", "gjk", "epa",
              "manifold")

    def phase_times(self) -> dict:
        out = (C.c_double * len(self.PHASES))()
        self._check(self.lib.rp_phase_times(self.h, out))
        return dict(zip(self.PHASES, out[:]))

    def transfer_bytes(self):
        out = (C.c_uint64 * 2)()
        self._check(self.lib.rp_transfer_bytes(self.h, out))
        return list(out)

    def set_timing(self, on: bool):
        self._check(self.lib.rp_set_timing(self.h, int(on)))

    def last_step_ms(self) -> float:
        v = _d()
        self._check(self.lib.rp_last_step_ms(self.h, C.byref(v)))
        return v.value

    def set_stream(self, stream_ptr: int):
        self._check(self.lib.rp_world_set_stream(self.h, C.c_void_p(stream_ptr)))
