"""Seeded synthetic scenes for raw-physics' rigid-body step.

A Scene is backend-neutral: meshes (the OBJ-loader form of rawphys.meshes), per-body colliders,
poses, masses, material coefficients, initial velocities and external constraints, plus the
per-frame call parameters of pbd_simulate (dt, substeps, position iterations, collisions) and the
gravity the caller applies as a force -g/inverse_mass (src/examples/stack.cpp:93-96).

Workloads (all seeded; none is a published dataset):
  stack_scene        10 unit cubes on a fixed 40x40 m floor, xz jitter U(-0.02, 0.02) m,
                     dt=1/60, 20 substeps, 1 iteration, friction 0.5/0.3, restitution 0
  large_scene        4096 bodies drawn uniformly from {cube, icosahedron, 32-segment cylinder,
                     42-vertex icosphere}, uniform scale U(0.5, 1.5), density 1, uniform random
                     orientation (Shoemake), v ~ N(0, 1) m/s, inside a fixed floor + 4 walls box
                     of 40x40x60 m; positions uniform in the box, rejection-sampled so no two
                     bounding spheres overlap at t=0
  tower_scene        a tower of unit cubes with alternating mass ratio
  chain_scene        cube links joined by hinge or spherical joints
  domino_scene       a row of 0.2x1x2 m dominoes and a thrown cube
  domino_batch       1024 domino rows of 16-64 with a thrown cube each (the differentiation workload)
  random_pile_scene  small mixed-shape piles for parity tests
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import meshes as M

# PBD_Axis_Type (src/physics/pbd.h:5-12)
POS_X, NEG_X, POS_Y, NEG_Y, POS_Z, NEG_Z = range(6)


@dataclass
class Collider:
    kind: str                    # "hull" or "sphere"
    mesh: int = -1               # index into Scene.meshes for hulls
    scale: tuple = (1.0, 1.0, 1.0)
    radius: float = 0.0          # spheres (stored as float32 by the reference)


@dataclass
class Constraint:
    kind: str                    # "positional" | "mutual_orientation" | "hinge" | "spherical"
    e1: int
    e2: int
    r1: tuple = (0.0, 0.0, 0.0)
    r2: tuple = (0.0, 0.0, 0.0)
    compliance: float = 0.0
    distance: tuple = (0.0, 0.0, 0.0)
    axis1: int = POS_X
    axis2: int = POS_X
    limited: bool = False
    limit_axis1: int = POS_Y
    limit_axis2: int = POS_Y
    lower: float = 0.0
    upper: float = 0.0
    swing_axis1: int = POS_X
    swing_axis2: int = POS_X
    twist_axis1: int = POS_Y
    twist_axis2: int = POS_Y
    swing_lower: float = 0.0
    swing_upper: float = 0.0
    twist_lower: float = 0.0
    twist_upper: float = 0.0


@dataclass
class Scene:
    name: str
    meshes: List[M.Mesh] = field(default_factory=list)
    colliders: List[List[Collider]] = field(default_factory=list)
    pos: Optional[np.ndarray] = None          # (N, 3) float64
    rot: Optional[np.ndarray] = None          # (N, 4) float64, (x, y, z, w)
    mass: Optional[np.ndarray] = None         # (N,) float64 (ignored for fixed bodies)
    fixed: Optional[np.ndarray] = None        # (N,) bool
    mus: Optional[np.ndarray] = None
    mud: Optional[np.ndarray] = None
    rest: Optional[np.ndarray] = None
    vel: Optional[np.ndarray] = None          # (N, 3)
    omega: Optional[np.ndarray] = None        # (N, 3)
    constraints: List[Constraint] = field(default_factory=list)
    dt: float = 1.0 / 60.0
    substeps: int = 20
    pos_iters: int = 1
    collisions: bool = True
    gravity: float = 10.0
    steps: int = 300

    @property
    def num_bodies(self) -> int:
        return 0 if self.pos is None else int(self.pos.shape[0])

    @property
    def num_dynamic(self) -> int:
        return int(np.count_nonzero(~self.fixed))


class _Builder:
    def __init__(self, name: str):
        self.scene = Scene(name)
        self._mesh_ids = {}
        self._cols, self._pos, self._rot, self._mass, self._fixed = [], [], [], [], []
        self._mus, self._mud, self._rest, self._v, self._w = [], [], [], [], []

    def mesh(self, name: str) -> int:
        if name not in self._mesh_ids:
            self._mesh_ids[name] = len(self.scene.meshes)
            self.scene.meshes.append(M.MESHES[name]())
        return self._mesh_ids[name]

    def body(self, colliders, pos, rot=(0.0, 0.0, 0.0, 1.0), mass=1.0, fixed=False, mus=0.5, mud=0.3, rest=0.0,
             v=(0.0, 0.0, 0.0), w=(0.0, 0.0, 0.0)) -> int:
        self._cols.append(list(colliders))
        self._pos.append(pos)
        self._rot.append(rot)
        self._mass.append(mass)
        self._fixed.append(bool(fixed))
        self._mus.append(mus)
        self._mud.append(mud)
        self._rest.append(rest)
        self._v.append(v)
        self._w.append(w)
        return len(self._pos) - 1

    def hull_body(self, mesh: str, scale, pos, **kw) -> int:
        return self.body([Collider("hull", self.mesh(mesh), tuple(float(s) for s in scale))], pos, **kw)

    def finish(self, **params) -> Scene:
        s = self.scene
        s.colliders = self._cols
        s.pos = np.asarray(self._pos, dtype=np.float64).reshape(-1, 3)
        s.rot = np.asarray(self._rot, dtype=np.float64).reshape(-1, 4)
        s.mass = np.asarray(self._mass, dtype=np.float64)
        s.fixed = np.asarray(self._fixed, dtype=bool)
        s.mus = np.asarray(self._mus, dtype=np.float64)
        s.mud = np.asarray(self._mud, dtype=np.float64)
        s.rest = np.asarray(self._rest, dtype=np.float64)
        s.vel = np.asarray(self._v, dtype=np.float64).reshape(-1, 3)
        s.omega = np.asarray(self._w, dtype=np.float64).reshape(-1, 3)
        for k, v in params.items():
            setattr(s, k, v)
        return s


def random_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random unit quaternions (Shoemake's subgroup algorithm), (x, y, z, w)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)
    return q


def _floor(b: _Builder, half=(20.0, 0.5, 20.0), y_top=0.0, mus=0.5, mud=0.3):
    return b.hull_body("cube", half, (0.0, y_top - half[1], 0.0), fixed=True, mus=mus, mud=mud)


def stack_scene(n: int = 10, seed: int = 0) -> Scene:
    """Cubes of edge 1 m (cube mesh scaled 0.5, density 1 -> mass 1) stacked on a 40x40 m floor."""
    rng = np.random.default_rng(seed)
    b = _Builder("stack%d" % n)
    _floor(b)
    for i in range(n):
        jx, jz = rng.uniform(-0.02, 0.02, size=2)
        b.hull_body("cube", (0.5, 0.5, 0.5), (float(jx), 0.5 + i * 1.001, float(jz)), mass=1.0)
    return b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=True, steps=300)


SHAPES = ("cube", "icosahedron", "cylinder32", "icosphere42")
_BASE_SCALE = 0.5   # all base meshes have radius ~1; scale 0.5 makes a unit-size body


def _mixed_body(b: _Builder, rng, shape: str, s: float, pos, rot, v, w=(0.0, 0.0, 0.0), mus=0.5, mud=0.3):
    sc = (_BASE_SCALE * s,) * 3
    mid = b.mesh(shape)
    mass = M.hull_volume(b.scene.meshes[mid], sc)
    return b.hull_body(shape, sc, pos, rot=rot, mass=mass, v=v, w=w, mus=mus, mud=mud)


def _box_walls(b: _Builder, half_x=20.0, half_z=20.0, height=60.0, t=0.5):
    _floor(b, (half_x, t, half_z))
    hy = height / 2.0
    b.hull_body("cube", (t, hy, half_z), (half_x + t, hy, 0.0), fixed=True)
    b.hull_body("cube", (t, hy, half_z), (-half_x - t, hy, 0.0), fixed=True)
    b.hull_body("cube", (half_x, hy, t), (0.0, hy, half_z + t), fixed=True)
    b.hull_body("cube", (half_x, hy, t), (0.0, hy, -half_z - t), fixed=True)


def large_scene(n: int = 4096, seed: int = 0, box=(40.0, 60.0, 40.0)) -> Scene:
    rng = np.random.default_rng(seed)
    b = _Builder("large%d" % n)
    _box_walls(b, box[0] / 2.0, box[2] / 2.0, box[1])
    shapes = rng.integers(0, len(SHAPES), size=n)
    scales = rng.uniform(0.5, 1.5, size=n)
    rots = random_quaternions(rng, n)
    vels = rng.normal(0.0, 1.0, size=(n, 3))
    # bounding radii of the base meshes (all 1) times the scale
    radii = _BASE_SCALE * scales
    placed = np.zeros((n, 3))
    placed_r = np.zeros(n)
    lo = np.array([-box[0] / 2.0, 0.0, -box[2] / 2.0])
    hi = np.array([box[0] / 2.0, box[1], box[2] / 2.0])
    for i in range(n):
        r = radii[i] * math.sqrt(3.0)   # cube corners reach sqrt(3) * half-edge
        for _ in range(10000):
            p = rng.uniform(lo + r, hi - r)
            if i == 0:
                break
            d = np.linalg.norm(placed[:i] - p, axis=1)
            if np.all(d > placed_r[:i] + r):
                break
        placed[i] = p
        placed_r[i] = r
    for i in range(n):
        _mixed_body(b, rng, SHAPES[shapes[i]], float(scales[i]), tuple(placed[i]), tuple(rots[i]), tuple(vels[i]))
    return b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=True, steps=600)


def tower_scene(n: int = 64, ratio: float = 100.0, seed: int = 0, substeps: int = 50) -> Scene:
    rng = np.random.default_rng(seed)
    b = _Builder("tower%d" % n)
    _floor(b)
    for i in range(n):
        jx, jz = rng.uniform(-0.005, 0.005, size=2)
        mass = 1.0 if i % 2 == 0 else ratio
        b.hull_body("cube", (0.5, 0.5, 0.5), (float(jx), 0.5 + i * 1.0005, float(jz)), mass=mass)
    return b.finish(dt=1.0 / 60.0, substeps=substeps, pos_iters=1, collisions=True, steps=10000)


def random_pile_scene(n: int = 12, seed: int = 0, shapes=SHAPES, spread: float = 1.6) -> Scene:
    """A small column of mixed shapes dropped on a floor, close enough to collide within a few frames."""
    rng = np.random.default_rng(seed)
    b = _Builder("pile%d_%d" % (n, seed))
    _floor(b, (8.0, 0.5, 8.0))
    for i in range(n):
        shape = shapes[int(rng.integers(0, len(shapes)))]
        s = float(rng.uniform(0.6, 1.2))
        p = (float(rng.uniform(-spread, spread)), 0.7 + 1.2 * i, float(rng.uniform(-spread, spread)))
        q = tuple(random_quaternions(rng, 1)[0])
        v = tuple(rng.normal(0.0, 0.5, size=3))
        w = tuple(rng.normal(0.0, 0.5, size=3))
        _mixed_body(b, rng, shape, s, p, q, v, w)
    return b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=True, steps=120)


def _axis_rotation(axis) -> tuple:
    """Unit quaternion mapping local +X onto the given unit vector (shortest arc)."""
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    x = np.array([1.0, 0.0, 0.0])
    c = float(np.dot(x, a))
    if c < -0.999999:
        return (0.0, 1.0, 0.0, 0.0)
    v = np.cross(x, a)
    q = np.array([v[0], v[1], v[2], 1.0 + c])
    q /= np.linalg.norm(q)
    return tuple(q)


def chain_scene(links: int = 8, joint: str = "spherical", seed: int = 0, collisions: bool = True,
                limited: bool = True) -> Scene:
    """Cube links (0.2 x 0.2 x 0.6 m boxes) hanging from a fixed anchor, joined end to end.

    Hinge chains align every link's local +X with one seeded random unit axis by rotating the
    links' initial orientation, since the reference's joints take body-frame axes only
    (PBD_Axis_Type, src/physics/pbd.h:5-12)."""
    rng = np.random.default_rng(seed)
    b = _Builder("chain%d_%s" % (links, joint))
    _floor(b, (10.0, 0.5, 10.0), y_top=-8.0 * links / 8.0 - 2.0)
    half = (0.1, 0.3, 0.1)
    axis = rng.normal(size=3)
    rot = _axis_rotation(axis) if joint == "hinge" else (0.0, 0.0, 0.0, 1.0)
    anchor = b.hull_body("cube", (0.1, 0.1, 0.1), (0.0, 1.0, 0.0), fixed=True, rot=rot)
    prev = anchor
    ids = []
    R = _rot_matrix(rot)
    down = R @ np.array([0.0, -1.0, 0.0])
    y0 = np.array([0.0, 1.0, 0.0])
    prev_off = R @ np.array([0.0, -0.1, 0.0])
    for i in range(links):
        centre = y0 + prev_off + down * 0.3 if i == 0 else np.asarray(b._pos[prev]) + down * 0.6
        mass = 8.0 * half[0] * half[1] * half[2]
        e = b.hull_body("cube", half, tuple(centre), rot=rot, mass=mass)
        ids.append(e)
        r1 = (0.0, -0.1, 0.0) if i == 0 else (0.0, -0.3, 0.0)
        r2 = (0.0, 0.3, 0.0)
        if joint == "hinge":
            c = Constraint("hinge", prev, e, r1, r2, 0.0, axis1=POS_X, axis2=POS_X, limited=limited,
                           limit_axis1=POS_Y, limit_axis2=POS_Y, lower=-0.5 * math.pi, upper=0.5 * math.pi)
        else:
            c = Constraint("spherical", prev, e, r1, r2, swing_axis1=POS_Y, swing_axis2=POS_Y,
                           twist_axis1=POS_X, twist_axis2=POS_X, swing_lower=-math.pi, swing_upper=math.pi,
                           twist_lower=-math.pi, twist_upper=math.pi)
        b.scene.constraints.append(c)
        prev = e
    # give the chain a kick so joints and limits work
    for k, e in enumerate(ids):
        b._v[e] = tuple(rng.normal(0.0, 1.0, size=3))
    return b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=collisions, steps=300)


def spring_scene(seed: int = 0) -> Scene:
    """Positional and mutual-orientation constraints, as the reference's spring example builds them
    (src/examples/spring.cpp:45-66): a unit cube (half extent 1, mass 1, friction 0.8) hung from a
    small fixed attachment by a positional constraint with compliance 0.001 and rest offset
    (0, -3, 0), over a floor (half extents 50 x 1 x 50 at y = -2). Beside it, seeded: a rope of four
    cubes joined by positional constraints (compliance 0, anchors at the faces, no offset), the top one
    to a second attachment with offset (0, -1, 0); two cubes locked together by a mutual-orientation
    constraint (compliance 0) and a second pair with compliance 0.01, which fall onto the floor and
    onto each other; every dynamic cube starts with a seeded rotation and velocity."""
    rng = np.random.default_rng(seed)
    b = _Builder("springs")
    b.hull_body("cube", (50.0, 1.0, 50.0), (0.0, -2.0, 0.0), fixed=True, mus=0.5, mud=0.5)
    q33 = tuple(_axis_angle((1.0, 1.0, 1.0), 33.0))
    att = b.hull_body("cube", (0.1, 0.1, 0.1), (0.0, 6.0, 0.0), rot=q33, fixed=True, mus=0.5, mud=0.5)
    cube = b.hull_body("cube", (1.0, 1.0, 1.0), (0.0, 2.0, 0.0), rot=q33, mass=1.0, mus=0.8, mud=0.8)
    b.scene.constraints.append(Constraint("positional", cube, att, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.001,
                                          distance=(0.0, -3.0, 0.0)))
    # a rope of cubes hanging from a second attachment
    att2 = b.hull_body("cube", (0.1, 0.1, 0.1), (5.0, 8.0, 0.0), fixed=True)
    prev, r_prev = att2, (0.0, -0.1, 0.0)
    for i in range(4):
        e = b.hull_body("cube", (0.3, 0.3, 0.3), (5.0 + 0.2 * rng.standard_normal(), 7.4 - 0.8 * i, 0.0),
                        rot=tuple(random_quaternions(rng, 1)[0]), mass=0.5, v=tuple(rng.normal(0.0, 0.5, 3)))
        dist = (0.0, -1.0, 0.0) if i == 0 else (0.0, 0.0, 0.0)
        b.scene.constraints.append(Constraint("positional", e, prev, (0.0, 0.3, 0.0), r_prev, 0.0, distance=dist))
        prev, r_prev = e, (0.0, -0.3, 0.0)
    # locked pairs falling onto the floor and onto each other
    for k, comp in enumerate((0.0, 0.01)):
        x = -5.0 - 3.0 * k
        e1 = b.hull_body("cube", (0.5, 0.5, 0.5), (x, 1.0 + k, 0.0), rot=tuple(random_quaternions(rng, 1)[0]),
                         mass=1.0, v=tuple(rng.normal(0.0, 1.0, 3)), w=tuple(rng.normal(0.0, 1.0, 3)))
        e2 = b.hull_body("cube", (0.4, 0.4, 0.4), (x + 0.3, 2.4 + k, 0.2), rot=tuple(random_quaternions(rng, 1)[0]),
                         mass=2.0, v=tuple(rng.normal(0.0, 1.0, 3)))
        b.scene.constraints.append(Constraint("mutual_orientation", e1, e2, compliance=comp))
    return b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=True, steps=300)


def _axis_angle(axis, degrees) -> np.ndarray:
    """quaternion_new (src/quaternion.cpp): rotation of `degrees` about the normalised axis, (x, y, z, w)."""
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    h = math.radians(degrees) / 2.0
    return np.concatenate([a * math.sin(h), [math.cos(h)]])


def _rot_matrix(q) -> np.ndarray:
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def domino_scene(n: int = 16, seed: int = 0) -> Scene:
    """Dominoes 0.2 x 1 x 2 m (cube scaled (0.1, 0.5, 1)... standing upright: height 2 m along y)
    spaced U(0.8, 1.2) m along x, plus a thrown unit cube with v ~ N(0, 2), w ~ N(0, 3)."""
    rng = np.random.default_rng(seed)
    b = _Builder("domino%d" % n)
    _floor(b, (max(10.0, 0.7 * n + 5.0), 0.5, 10.0))
    x = 0.0
    for i in range(n):
        x += float(rng.uniform(0.8, 1.2))
        b.hull_body("cube", (0.1, 1.0, 0.5), (x, 1.0, 0.0), mass=0.2 * 2.0 * 1.0)
    v = rng.normal(0.0, 2.0, size=3)
    v[0] = abs(v[0]) + 4.0
    w = rng.normal(0.0, 3.0, size=3)
    b.hull_body("cube", (0.5, 0.5, 0.5), (-1.0, 1.6, 0.0), mass=1.0, v=tuple(v), w=tuple(w))
    return b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=True, steps=120)


def sphere_scene(n: int = 6, seed: int = 0) -> Scene:
    """Analytic sphere colliders (collider_sphere_create) and a compound two-hull body."""
    rng = np.random.default_rng(seed)
    b = _Builder("spheres%d" % n)
    _floor(b, (6.0, 0.5, 6.0))
    for i in range(n):
        r = float(np.float32(rng.uniform(0.3, 0.6)))
        p = (float(rng.uniform(-0.6, 0.6)), 0.8 + 1.1 * i, float(rng.uniform(-0.6, 0.6)))
        b.body([Collider("sphere", radius=r)], p, mass=1.0, v=tuple(rng.normal(0, 0.3, size=3)))
    cm = b.mesh("cube")
    b.body([Collider("hull", cm, (0.3, 0.3, 0.3)), Collider("hull", cm, (0.6, 0.1, 0.1))], (0.3, 0.5 + 1.1 * n, 0.2),
           mass=2.0)
    return b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=True, steps=120)


# ---------------------------------------------------------------------------------------------
# Batches of many independent scenes
@dataclass
class SceneBatch:
    """Many independent scenes as flat per-body arrays (bodies of scene s are contiguous, scenes in
    order). Every body has one hull collider: mesh index into `meshes` and a scale vector."""
    name: str
    meshes: List[M.Mesh]
    scene: np.ndarray            # (N,) int32
    mesh: np.ndarray             # (N,) int32
    scale: np.ndarray            # (N, 3)
    pos: np.ndarray              # (N, 3)
    rot: np.ndarray              # (N, 4)
    mass: np.ndarray             # (N,)
    fixed: np.ndarray            # (N,) bool
    mus: np.ndarray
    mud: np.ndarray
    rest: np.ndarray
    vel: np.ndarray              # (N, 3)
    omega: np.ndarray            # (N, 3)
    constraints: List[Constraint] = field(default_factory=list)   # e1 / e2: global body indices
    num_scenes: int = 1
    dt: float = 1.0 / 60.0
    substeps: int = 20
    pos_iters: int = 1
    collisions: bool = True
    gravity: float = 10.0
    steps: int = 300

    @property
    def num_bodies(self) -> int:
        return int(self.pos.shape[0])

    @property
    def num_dynamic(self) -> int:
        return int(np.count_nonzero(~self.fixed))

    def scene_sizes(self) -> np.ndarray:
        """Dynamic bodies per scene."""
        return np.bincount(self.scene[~self.fixed], minlength=self.num_scenes)


def batched_scenes(num_scenes: int = 16384, seed: int = 0, min_bodies: int = 2, max_bodies: int = 512,
                   chain_fraction: float = 0.25, chain_links=(8, 64)) -> SceneBatch:
    """Independent scenes of uneven size for the batched form of the step.

    Per scene: N dynamic bodies, N log-uniform in [min_bodies, max_bodies], drawn uniformly from the
    large scene's shapes (cube, icosahedron, 32-segment cylinder, 42-vertex icosphere) with uniform
    scale U(0.5, 1.5) (quantised to 1/256 so that bodies of equal shape and scale share one hull),
    density 1, uniform random orientation, v ~ N(0, 1) m/s. Bodies sit one per cell of a jittered
    2.86 m grid (the large scene's 23.4 m^3 per body) inside a fixed floor-and-walls box sized to N
    (box dimensions quantised to 0.5 m). A `chain_fraction` of the scenes also hang a chain of
    8-64 cube links (0.2 x 0.2 x 0.6 m) from a fixed anchor, joined by spherical joints or by hinges
    whose axis is a seeded random unit vector, compliance 0, down the box's central column."""
    rng = np.random.default_rng(seed)
    meshes = [M.MESHES[n]() for n in SHAPES]
    CUBE = 0
    cell = 23.4 ** (1.0 / 3.0)
    rows = {k: [] for k in ("scene", "mesh", "scale", "pos", "rot", "mass", "fixed", "mus", "mud", "rest", "vel", "omega")}
    cons: List[Constraint] = []
    vol_cache = {}
    n_per = np.exp(rng.uniform(math.log(min_bodies), math.log(max_bodies + 1), size=num_scenes)).astype(int)
    n_per = np.clip(n_per, min_bodies, max_bodies)
    has_chain = rng.random(num_scenes) < chain_fraction
    count = 0

    def add(scene, mesh, scale, pos, rot=(0.0, 0.0, 0.0, 1.0), mass=1.0, fixed=False, v=(0.0, 0.0, 0.0), w=(0.0, 0.0, 0.0)):
        nonlocal count
        rows["scene"].append(scene)
        rows["mesh"].append(mesh)
        rows["scale"].append(scale)
        rows["pos"].append(pos)
        rows["rot"].append(rot)
        rows["mass"].append(mass)
        rows["fixed"].append(fixed)
        rows["mus"].append(0.5)
        rows["mud"].append(0.3)
        rows["rest"].append(0.0)
        rows["vel"].append(v)
        rows["omega"].append(w)
        count += 1
        return count - 1

    for s in range(num_scenes):
        n = int(n_per[s])
        links = int(rng.integers(chain_links[0], chain_links[1] + 1)) if has_chain[s] else 0
        # box: the large scene's 40 x 40 x 60 m for 4096 bodies, scaled to n, at least 3 cells wide
        f = (n / 4096.0) ** (1.0 / 3.0)
        half = max(1.5 * cell, math.ceil(20.0 * f * 2.0) / 2.0)
        nx = max(1, int(2 * half / cell))
        free_cells = nx * nx - (1 if links else 0)
        ny = max(1, math.ceil(n / max(free_cells, 1)))
        height = max(ny * cell, (0.6 * links + 3.0) if links else 0.0)
        height = math.ceil(height * 2.0) / 2.0
        t = 0.5
        add(s, CUBE, (half, t, half), (0.0, -t, 0.0), fixed=True)
        hy = height / 2.0
        add(s, CUBE, (t, hy, half), (half + t, hy, 0.0), fixed=True)
        add(s, CUBE, (t, hy, half), (-half - t, hy, 0.0), fixed=True)
        add(s, CUBE, (half, hy, t), (0.0, hy, half + t), fixed=True)
        add(s, CUBE, (half, hy, t), (0.0, hy, -half - t), fixed=True)
        # grid cells, the central column kept free for a chain
        cx = (np.arange(nx) + 0.5) * (2 * half / nx) - half
        cy = (np.arange(max(ny, int(height / cell))) + 0.5) * cell
        grid = np.stack(np.meshgrid(cx, cy, cx, indexing="ij"), axis=-1).reshape(-1, 3)
        if links:
            grid = grid[(np.abs(grid[:, 0]) > 0.7) | (np.abs(grid[:, 2]) > 0.7)]
        pick = rng.choice(len(grid), size=min(n, len(grid)), replace=False)
        shapes = rng.integers(0, len(SHAPES), size=len(pick))
        scales = 0.5 + np.round(rng.uniform(0.0, 1.0, size=len(pick)) * 256.0) / 256.0
        rots = random_quaternions(rng, len(pick))
        vels = rng.normal(0.0, 1.0, size=(len(pick), 3))
        jit = rng.uniform(-0.1, 0.1, size=(len(pick), 3))
        for i, g in enumerate(pick):
            sc = _BASE_SCALE * float(scales[i])
            key = (int(shapes[i]), sc)
            if key not in vol_cache:
                vol_cache[key] = M.hull_volume(meshes[key[0]], (sc, sc, sc))
            add(s, int(shapes[i]), (sc, sc, sc), tuple(grid[g] + jit[i]), rot=tuple(rots[i]), mass=vol_cache[key],
                v=tuple(vels[i]))
        if links:
            joint = "hinge" if rng.random() < 0.5 else "spherical"
            axis = rng.normal(size=3)
            rot = _axis_rotation(axis) if joint == "hinge" else (0.0, 0.0, 0.0, 1.0)
            R = _rot_matrix(rot)
            down = R @ np.array([0.0, -1.0, 0.0])
            top = np.array([0.0, height - 0.5, 0.0])
            anchor = add(s, CUBE, (0.1, 0.1, 0.1), tuple(top), rot=rot, fixed=True)
            prev, prev_c = anchor, top
            for i in range(links):
                centre = prev_c + R @ np.array([0.0, -0.1, 0.0]) + down * 0.3 if i == 0 else prev_c + down * 0.6
                e = add(s, CUBE, (0.1, 0.3, 0.1), tuple(centre), rot=rot, mass=8.0 * 0.1 * 0.3 * 0.1,
                        v=tuple(rng.normal(0.0, 0.5, size=3)))
                r1 = (0.0, -0.1, 0.0) if i == 0 else (0.0, -0.3, 0.0)
                if joint == "hinge":
                    cons.append(Constraint("hinge", prev, e, r1, (0.0, 0.3, 0.0), 0.0, axis1=POS_X, axis2=POS_X,
                                           limited=True, limit_axis1=POS_Y, limit_axis2=POS_Y,
                                           lower=-0.5 * math.pi, upper=0.5 * math.pi))
                else:
                    cons.append(Constraint("spherical", prev, e, r1, (0.0, 0.3, 0.0), swing_axis1=POS_Y,
                                           swing_axis2=POS_Y, twist_axis1=POS_X, twist_axis2=POS_X,
                                           swing_lower=-math.pi, swing_upper=math.pi, twist_lower=-math.pi,
                                           twist_upper=math.pi))
                prev, prev_c = e, centre
    f64 = lambda k, d: np.asarray(rows[k], dtype=np.float64).reshape(-1, d)
    return SceneBatch("batch%d" % num_scenes, meshes, np.asarray(rows["scene"], dtype=np.int32),
                      np.asarray(rows["mesh"], dtype=np.int32), f64("scale", 3), f64("pos", 3), f64("rot", 4),
                      np.asarray(rows["mass"], dtype=np.float64), np.asarray(rows["fixed"], dtype=bool),
                      np.asarray(rows["mus"]), np.asarray(rows["mud"]), np.asarray(rows["rest"]), f64("vel", 3),
                      f64("omega", 3), cons, num_scenes=num_scenes)


def batch_scene(batch: SceneBatch, s: int) -> Scene:
    """Scene s of a batch as a stand-alone Scene (entity indices local to it), for checks."""
    idx = np.nonzero(batch.scene == s)[0]
    b0 = int(idx[0])
    b = _Builder("%s_scene%d" % (batch.name, s))
    names = {id(m): n for n, m in zip(SHAPES, batch.meshes)}
    for i in idx:
        b.hull_body(names[id(batch.meshes[batch.mesh[i]])], tuple(batch.scale[i]), tuple(batch.pos[i]),
                    rot=tuple(batch.rot[i]), mass=float(batch.mass[i]), fixed=bool(batch.fixed[i]),
                    mus=float(batch.mus[i]), mud=float(batch.mud[i]), rest=float(batch.rest[i]),
                    v=tuple(batch.vel[i]), w=tuple(batch.omega[i]))
    for c in batch.constraints:
        if b0 <= c.e1 <= idx[-1]:
            d = Constraint(**{k: getattr(c, k) for k in c.__dataclass_fields__})
            d.e1, d.e2 = c.e1 - b0, c.e2 - b0
            b.scene.constraints.append(d)
    return b.finish(dt=batch.dt, substeps=batch.substeps, pos_iters=batch.pos_iters, collisions=batch.collisions,
                    steps=batch.steps)


def shard_batch(batch: SceneBatch, rank: int, world: int) -> SceneBatch:
    """Scenes of a batch for one of `world` ranks: contiguous scene ranges balanced by body count
    (scenes are independent, so ranks exchange nothing while stepping)."""
    sizes = np.bincount(batch.scene, minlength=batch.num_scenes).astype(np.float64)
    cum = np.concatenate([[0.0], np.cumsum(sizes)])
    bounds = [int(np.searchsorted(cum, cum[-1] * r / world, side="left")) for r in range(world + 1)]
    bounds[0], bounds[-1] = 0, batch.num_scenes
    s0, s1 = bounds[rank], max(bounds[rank], bounds[rank + 1])
    keep = (batch.scene >= s0) & (batch.scene < s1)
    idx = np.nonzero(keep)[0]
    remap = -np.ones(batch.num_bodies, dtype=np.int64)
    remap[idx] = np.arange(len(idx))
    cons = []
    for c in batch.constraints:
        if keep[c.e1]:
            d = Constraint(**{k: getattr(c, k) for k in c.__dataclass_fields__})
            d.e1, d.e2 = int(remap[c.e1]), int(remap[c.e2])
            cons.append(d)
    return SceneBatch("%s_rank%d" % (batch.name, rank), batch.meshes, (batch.scene[idx] - s0).astype(np.int32),
                      batch.mesh[idx], batch.scale[idx], batch.pos[idx], batch.rot[idx], batch.mass[idx],
                      batch.fixed[idx], batch.mus[idx], batch.mud[idx], batch.rest[idx], batch.vel[idx],
                      batch.omega[idx], cons, num_scenes=s1 - s0, dt=batch.dt, substeps=batch.substeps,
                      pos_iters=batch.pos_iters, collisions=batch.collisions, gravity=batch.gravity,
                      steps=batch.steps)


def domino_batch(num_scenes: int = 1024, seed: int = 0, min_dominoes: int = 16, max_dominoes: int = 64):
    """Differentiation workload: `num_scenes` independent scenes, each a row of n ~ U{16..64}
    dominoes (cube scaled (0.1, 1, 0.5): 0.2 x 2 x 1 m, density 1) spaced U(0.8, 1.2) m along x on
    its own fixed floor, plus a thrown unit cube with v ~ N(0, 2) m/s (x component made positive
    and raised by 4 so that it flies at the row) and w ~ N(0, 3) rad/s. dt 1/60, 20 substeps,
    120 steps. Returns the batch, the body index of each scene's last domino, and a seeded loss
    target per scene (the last domino's centre displaced by N(0, 0.5) m in x and z)."""
    rng = np.random.default_rng(seed)
    meshes = [M.MESHES[name]() for name in SHAPES]
    rows = {k: [] for k in ("scene", "scale", "pos", "mass", "fixed", "vel", "omega")}
    last, target = [], []
    for s in range(num_scenes):
        n = int(rng.integers(min_dominoes, max_dominoes + 1))
        half = max(10.0, 0.7 * n + 5.0)
        def add(scale, pos, mass, fixed, v=(0.0, 0.0, 0.0), w=(0.0, 0.0, 0.0)):
            rows["scene"].append(s); rows["scale"].append(scale); rows["pos"].append(pos)
            rows["mass"].append(mass); rows["fixed"].append(fixed); rows["vel"].append(v); rows["omega"].append(w)
            return len(rows["scene"]) - 1
        add((half, 0.5, 10.0), (0.0, -0.5, 0.0), 1.0, True)
        x = 0.0
        for i in range(n):
            x += float(rng.uniform(0.8, 1.2))
            e = add((0.1, 1.0, 0.5), (x, 1.0, 0.0), 0.2 * 2.0 * 1.0, False)
        last.append(e)
        target.append((x + rng.normal(0.0, 0.5), 1.0, rng.normal(0.0, 0.5)))
        v = rng.normal(0.0, 2.0, size=3)
        v[0] = abs(v[0]) + 4.0
        w = rng.normal(0.0, 3.0, size=3)
        add((0.5, 0.5, 0.5), (-1.0, 1.6, 0.0), 1.0, False, tuple(v), tuple(w))
    N = len(rows["scene"])
    batch = SceneBatch("dominoes%d" % num_scenes, meshes, np.asarray(rows["scene"], dtype=np.int32),
                       np.zeros(N, dtype=np.int32), np.asarray(rows["scale"], dtype=np.float64),
                       np.asarray(rows["pos"], dtype=np.float64), np.tile(np.array([0.0, 0.0, 0.0, 1.0]), (N, 1)),
                       np.asarray(rows["mass"], dtype=np.float64), np.asarray(rows["fixed"], dtype=bool),
                       np.full(N, 0.5), np.full(N, 0.3), np.zeros(N), np.asarray(rows["vel"], dtype=np.float64),
                       np.asarray(rows["omega"], dtype=np.float64), [], num_scenes=num_scenes, steps=120)
    return batch, np.asarray(last, dtype=np.int32), np.asarray(target, dtype=np.float64)


def tower_batch(num_towers: int = 2048, n: int = 64, ratio: float = 100.0, seed: int = 0, substeps: int = 50) -> SceneBatch:
    """Precision-stress batch: `num_towers` independent scenes, each a tower of n unit cubes on its
    own fixed floor, masses alternating 1 : ratio, xz jitter U(-0.005, 0.005) m, 50 substeps."""
    rng = np.random.default_rng(seed)
    meshes = [M.MESHES[name]() for name in SHAPES]
    N = num_towers * (n + 1)
    scene = np.repeat(np.arange(num_towers, dtype=np.int32), n + 1)
    mesh = np.zeros(N, dtype=np.int32)
    scale = np.tile(np.array([[20.0, 0.5, 20.0]] + [[0.5, 0.5, 0.5]] * n), (num_towers, 1))
    pos = np.zeros((N, 3))
    jit = rng.uniform(-0.005, 0.005, size=(num_towers, n, 2))
    for t in range(num_towers):
        base = t * (n + 1)
        pos[base] = (0.0, -0.5, 0.0)
        pos[base + 1:base + n + 1, 0] = jit[t, :, 0]
        pos[base + 1:base + n + 1, 1] = 0.5 + np.arange(n) * 1.0005
        pos[base + 1:base + n + 1, 2] = jit[t, :, 1]
    rot = np.tile(np.array([0.0, 0.0, 0.0, 1.0]), (N, 1))
    mass = np.tile(np.array([1.0] + [1.0 if i % 2 == 0 else ratio for i in range(n)]), num_towers)
    fixed = np.tile(np.array([True] + [False] * n), num_towers)
    z = np.zeros((N, 3))
    return SceneBatch("towers%d_%d" % (num_towers, n), meshes, scene, mesh, scale, pos, rot, mass, fixed,
                      np.full(N, 0.5), np.full(N, 0.3), np.zeros(N), z, z.copy(), [], num_scenes=num_towers,
                      substeps=substeps, steps=10000)
