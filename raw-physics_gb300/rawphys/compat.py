"""The reference's caller-side data, for driving the C++-mangled pbd_simulate drop-in from Python.

raw-physics callers hold their scene as `Entity` structs (src/entity.h:17-47) with `Collider` light
arrays (src/physics/collider.h:5-44), `Physics_Force` light arrays (entity.h:11-15) and a
`Constraint` light array (src/physics/pbd.h:22-91), and pass `Entity**` to
pbd_simulate_with_constraints (pbd.h:93-94). This module restates those layouts in ctypes (the same
layouts include/rp_compat.h declares for C++ callers) and builds them for a rawphys.scenes.Scene, so
tests and bench.py call the drop-in exactly as a reference caller would.

Light arrays are the reference's: a {size_t capacity; size_t length;} header directly before the
first element (include/light_array.h:68-71).
"""
from __future__ import annotations

import ctypes as C

import numpy as np


class Vec3(C.Structure):
    _pack_ = 1
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class Quat(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double), ("w", C.c_double)]


class Mat3(C.Structure):
    _pack_ = 1
    _fields_ = [("data", C.c_double * 9)]


class Force(C.Structure):
    _fields_ = [("position", Vec3), ("force", Vec3), ("local_coords", C.c_int32)]


class HullFace(C.Structure):
    _fields_ = [("elements", C.c_void_p), ("normal", Vec3)]


class Hull(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("transformed_vertices", C.c_void_p), ("faces", C.c_void_p),
                ("transformed_faces", C.c_void_p), ("vertex_to_faces", C.c_void_p), ("vertex_to_neighbors", C.c_void_p),
                ("face_to_neighbors", C.c_void_p)]


class Sphere(C.Structure):
    _fields_ = [("radius", C.c_float), ("center", Vec3)]


class _ColliderShape(C.Union):
    _fields_ = [("convex_hull", Hull), ("sphere", Sphere)]


class Collider(C.Structure):
    _anonymous_ = ("u",)
    _fields_ = [("type", C.c_int32), ("u", _ColliderShape)]


class Entity(C.Structure):
    _fields_ = [("id", C.c_uint64), ("mesh", C.c_uint32 * 4), ("world_position", Vec3), ("world_rotation", Quat),
                ("world_scale", Vec3), ("color", C.c_double * 4), ("colliders", C.c_void_p),
                ("bounding_sphere_radius", C.c_double), ("forces", C.c_void_p), ("inverse_mass", C.c_double),
                ("inertia_tensor", Mat3), ("inverse_inertia_tensor", Mat3), ("angular_velocity", Vec3),
                ("linear_velocity", Vec3), ("fixed", C.c_int32), ("active", C.c_int32), ("deactivation_time", C.c_double),
                ("static_friction_coefficient", C.c_double), ("dynamic_friction_coefficient", C.c_double),
                ("restitution_coefficient", C.c_double), ("previous_world_position", Vec3), ("previous_world_rotation", Quat),
                ("previous_linear_velocity", Vec3), ("previous_angular_velocity", Vec3)]


class _Positional(C.Structure):
    _fields_ = [("r1_lc", Vec3), ("r2_lc", Vec3), ("compliance", C.c_double), ("lambda_", C.c_double),
                ("distance", Vec3)]


class _MutualOrientation(C.Structure):
    _fields_ = [("compliance", C.c_double), ("lambda_", C.c_double)]


class _Hinge(C.Structure):
    _fields_ = [("r1_lc", Vec3), ("r2_lc", Vec3), ("compliance", C.c_double), ("lambda_pos", C.c_double),
                ("e1_aligned_axis", C.c_int32), ("e2_aligned_axis", C.c_int32), ("lambda_aligned_axes", C.c_double),
                ("limited", C.c_int32), ("upper_limit", C.c_double), ("lower_limit", C.c_double),
                ("e1_limit_axis", C.c_int32), ("e2_limit_axis", C.c_int32), ("lambda_limit_axes", C.c_double)]


class _Spherical(C.Structure):
    _fields_ = [("r1_lc", Vec3), ("r2_lc", Vec3), ("lambda_pos", C.c_double), ("lambda_swing", C.c_double),
                ("swing_upper_limit", C.c_double), ("swing_lower_limit", C.c_double),
                ("e1_swing_axis", C.c_int32), ("e2_swing_axis", C.c_int32), ("lambda_twist", C.c_double),
                ("twist_upper_limit", C.c_double), ("twist_lower_limit", C.c_double),
                ("e1_twist_axis", C.c_int32), ("e2_twist_axis", C.c_int32)]


class _ConstraintBody(C.Union):
    _fields_ = [("positional_constraint", _Positional), ("mutual_orientation_constraint", _MutualOrientation),
                ("hinge_joint_constraint", _Hinge), ("spherical_joint_constraint", _Spherical),
                ("_size", C.c_ubyte * 120)]


class Constraint(C.Structure):
    _anonymous_ = ("u",)
    _fields_ = [("type", C.c_int32), ("e1_id", C.c_uint64), ("e2_id", C.c_uint64), ("u", _ConstraintBody)]


assert C.sizeof(Entity) == 504 and C.sizeof(Collider) == 64 and C.sizeof(Constraint) == 144

CONSTRAINT_TYPE = {"positional": 0, "mutual_orientation": 2, "hinge": 3, "spherical": 4}   # pbd.h:14-20


class LightArrays:
    """Allocates include/light_array.h arrays and keeps them alive."""

    def __init__(self):
        self.keep = []

    def make(self, ctype, values):
        n = len(values)
        buf = (C.c_ubyte * (16 + C.sizeof(ctype) * max(n, 1)))()
        self.keep.append(buf)
        hdr = (C.c_size_t * 2).from_buffer(buf)
        hdr[0] = max(n, 1)
        hdr[1] = n
        arr = (ctype * max(n, 1)).from_buffer(buf, 16)
        for i, v in enumerate(values):
            arr[i] = v
        return C.addressof(buf) + 16

    def ptrs(self, ptrs):
        a = (C.c_void_p * max(len(ptrs), 1))(*ptrs)
        self.keep.append(a)
        return C.addressof(a)


def hull_struct(la: LightArrays, verts, normals, tables) -> Hull:
    """A Collider_Convex_Hull (collider.h:15-24) from a hull's vertices, face normals and its four CSR
    tables (0 face loops, 1 vertex->faces, 2 vertex->neighbours, 3 face->neighbours)."""
    vtx = [Vec3(*v) for v in verts]
    fs, fd = tables[0]
    faces = [HullFace(la.make(C.c_uint32, [int(x) for x in fd[fs[f]:fs[f + 1]]]), Vec3(*normals[f]))
             for f in range(len(normals))]

    def rows(t):
        start, data = t
        return la.ptrs([la.make(C.c_uint32, [int(x) for x in data[start[r]:start[r + 1]]]) for r in range(len(start) - 1)])
    return Hull(la.make(Vec3, vtx), la.make(Vec3, vtx), la.make(HullFace, faces), la.make(HullFace, faces),
                rows(tables[1]), rows(tables[2]), rows(tables[3]))


class Callers:
    """A scene as a raw-physics caller holds it: `entities` (the Entity structs), `array` (the
    Entity** light array to pass), `constraints` (the Constraint light array, or None)."""

    def __init__(self, entities, array, constraints, la):
        self.entities = entities
        self.array = array
        self.constraints = constraints
        self._la = la

    def add_gravity(self, g: float = 10.0):
        """entity_add_force(e, 0, (0, -g / inverse_mass, 0)) on every entity, as the examples do before
        each step (src/examples/stack.cpp:93-96); the drop-in's caller then clears them (entity.cpp:193)."""
        for e in self.entities:
            f = -g * 1.0 / e.inverse_mass if e.inverse_mass else -np.inf
            e.forces = self._la.make(Force, [Force(Vec3(0.0, 0.0, 0.0), Vec3(0.0, f, 0.0), 0)])

    def clear_forces(self):
        for e in self.entities:
            e.forces = self._la.make(Force, [])

    def state(self) -> np.ndarray:
        """The entities' state in the rawphys state-record layout (28 doubles per entity)."""
        out = np.zeros((len(self.entities), 28))
        for i, e in enumerate(self.entities):
            out[i, 0:3] = (e.world_position.x, e.world_position.y, e.world_position.z)
            out[i, 3:7] = (e.world_rotation.x, e.world_rotation.y, e.world_rotation.z, e.world_rotation.w)
            out[i, 7:10] = (e.linear_velocity.x, e.linear_velocity.y, e.linear_velocity.z)
            out[i, 10:13] = (e.angular_velocity.x, e.angular_velocity.y, e.angular_velocity.z)
            out[i, 13:16] = (e.previous_world_position.x, e.previous_world_position.y, e.previous_world_position.z)
            out[i, 16:20] = (e.previous_world_rotation.x, e.previous_world_rotation.y, e.previous_world_rotation.z,
                             e.previous_world_rotation.w)
            out[i, 20:23] = (e.previous_linear_velocity.x, e.previous_linear_velocity.y, e.previous_linear_velocity.z)
            out[i, 23:26] = (e.previous_angular_velocity.x, e.previous_angular_velocity.y, e.previous_angular_velocity.z)
            out[i, 26] = float(e.active != 0)
            out[i, 27] = e.deactivation_time
        return out

    def set_state(self, st: np.ndarray):
        for i, e in enumerate(self.entities):
            o = st[i]
            e.world_position = Vec3(*o[0:3])
            e.world_rotation = Quat(*o[3:7])
            e.linear_velocity = Vec3(*o[7:10])
            e.angular_velocity = Vec3(*o[10:13])
            e.previous_world_position = Vec3(*o[13:16])
            e.previous_world_rotation = Quat(*o[16:20])
            e.previous_linear_velocity = Vec3(*o[20:23])
            e.previous_angular_velocity = Vec3(*o[23:26])
            e.active = int(o[26] != 0.0)
            e.deactivation_time = float(o[27])


def build_callers(scene, topology=None, mass_properties=None) -> Callers:
    """The Entity / Collider / Constraint arrays of a rawphys.scenes.Scene. Hull topology and mass
    properties come from `topology(entity, k) -> (verts, normals, tables)` and
    `mass_properties(entity) -> (inverse_mass, I, I_inv, radius)` when given (a test passes the
    oracle's), else from this library's host-side set-up (rp_hull_create, rp_entity_create on a
    host-only world), which reproduces the reference's collider_convex_hull_create and entity_create."""
    hw = None
    if topology is None or mass_properties is None:
        from . import World
        hw = World(-1, "fp64")
        hw.load(scene)
        hull_ids = {}
        for b in range(scene.num_bodies):
            for k, c in enumerate(scene.colliders[b]):
                if c.kind == "hull":
                    hull_ids[(b, k)] = hw._hulls[(id(scene.meshes[c.mesh]), tuple(c.scale))]
        if topology is None:
            topology = lambda b, k: hw.hull_topology(hull_ids[(b, k)])
        if mass_properties is None:
            mass_properties = hw.mass_properties
    la = LightArrays()
    ents = []
    for b in range(scene.num_bodies):
        cols = []
        for k, c in enumerate(scene.colliders[b]):
            if c.kind == "hull":
                col = Collider()
                col.type = 1
                col.convex_hull = hull_struct(la, *topology(b, k))
            else:
                col = Collider()
                col.type = 0
                col.sphere = Sphere(float(c.radius), Vec3(*scene.pos[b]))
            cols.append(col)
        invm, I, Ii, radius = mass_properties(b)
        e = Entity()
        e.id = 1000 + b
        e.world_position = Vec3(*scene.pos[b])
        e.world_rotation = Quat(*scene.rot[b])
        e.world_scale = Vec3(1.0, 1.0, 1.0)
        e.colliders = la.make(Collider, cols)
        e.bounding_sphere_radius = radius
        e.inverse_mass = invm
        e.inertia_tensor = Mat3((C.c_double * 9)(*np.asarray(I).reshape(9)))
        e.inverse_inertia_tensor = Mat3((C.c_double * 9)(*np.asarray(Ii).reshape(9)))
        e.linear_velocity = Vec3(*scene.vel[b])
        e.angular_velocity = Vec3(*scene.omega[b])
        e.fixed = int(scene.fixed[b])
        e.active = 1
        e.static_friction_coefficient = float(scene.mus[b])
        e.dynamic_friction_coefficient = float(scene.mud[b])
        e.restitution_coefficient = float(scene.rest[b])
        e.previous_world_rotation = Quat(0.0, 0.0, 0.0, 1.0)
        e.forces = la.make(Force, [])
        ents.append(e)
    array = la.make(C.POINTER(Entity), [C.pointer(x) for x in ents])
    cons = None
    if scene.constraints:
        rows = []
        for c in scene.constraints:
            x = Constraint()
            x.type = CONSTRAINT_TYPE[c.kind]
            x.e1_id = ents[c.e1].id
            x.e2_id = ents[c.e2].id
            if c.kind == "positional":
                x.positional_constraint = _Positional(Vec3(*c.r1), Vec3(*c.r2), c.compliance, 0.0, Vec3(*c.distance))
            elif c.kind == "mutual_orientation":
                x.mutual_orientation_constraint = _MutualOrientation(c.compliance, 0.0)
            elif c.kind == "hinge":
                x.hinge_joint_constraint = _Hinge(Vec3(*c.r1), Vec3(*c.r2), c.compliance, 0.0, c.axis1, c.axis2, 0.0,
                                                  int(c.limited), c.upper, c.lower, c.limit_axis1, c.limit_axis2, 0.0)
            else:
                x.spherical_joint_constraint = _Spherical(Vec3(*c.r1), Vec3(*c.r2), 0.0, 0.0, c.swing_upper,
                                                          c.swing_lower, c.swing_axis1, c.swing_axis2, 0.0,
                                                          c.twist_upper, c.twist_lower, c.twist_axis1, c.twist_axis2)
            rows.append(x)
        cons = la.make(Constraint, rows)
    if hw is not None:
        hw.close()
    return Callers(ents, array, cons, la)


def dropin(lib):
    """The two mangled entry points of the library (pbd_simulate, pbd_simulate_with_constraints)."""
    f = getattr(lib, "_Z12pbd_simulatedPP6Entityjji")
    f.argtypes = [C.c_double, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32]
    f.restype = None
    g = getattr(lib, "_Z29pbd_simulate_with_constraintsdPP6EntityP10Constraintjji")
    g.argtypes = [C.c_double, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32]
    g.restype = None
    return f, g
