"""CPU-side checks of the product: the C ABI library loads and exports every declared symbol; the
host set-up (hull topology, bounding radius, point-mass inertia) reproduces the reference exactly;
host-only worlds refuse GPU work loudly; argument validation; scene generators."""
from __future__ import annotations

import ctypes as C
import os
import re
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))

from conftest import ROOT, golden
from make_golden import SCENES


def declared_functions():
    names = []
    for h in ("rp.h", "rp_compat.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(rp_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(ext_built):
    lib = C.CDLL(ext_built.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the drop-in: C++-mangled exactly as the reference's pbd.cpp compiles them (pbd.h:93-94)
    for sym in ("_Z12pbd_simulatedPP6Entityjji", "_Z29pbd_simulate_with_constraintsdPP6EntityP10Constraintjji"):
        assert hasattr(lib, sym), sym
    # and the binding covers the whole C ABI of include/rp.h (the drop-in's own helpers are bound by
    # rawphys.compat's callers)
    assert set(n for n in names if not n.startswith("rp_compat_")) <= set(ext_built.SIGNATURES)


@pytest.mark.parametrize("name", ["stack10", "spheres6", "large1024", "chain8_hinge", "domino16"])
def test_host_mass_properties_match_reference(ext_built, name):
    g = golden(name)
    scene = SCENES[name][0]()
    w = ext_built.World(-1, "fp64")
    w.load(scene)
    for e in range(scene.num_bodies):
        invm, I, Ii, r = w.mass_properties(e)
        assert invm == g["invm"][e]
        assert r == g["radius"][e]
        if "inertia" in g:
            assert np.array_equal(I.reshape(9), g["inertia"][e])
            assert np.array_equal(Ii.reshape(9), g["inverse_inertia"][e])
    w.close()


def test_host_hull_topology_matches_oracle(ext_built, oracle_built):
    """Vertex order, faces, face normals, vertex->faces, vertex->neighbours, face->neighbours."""
    from rawphys import scenes as S
    scene = S.large_scene(40, seed=5)
    w = ext_built.World(-1, "fp32")
    w.load(scene)
    o = oracle_built("port").load(scene)
    for e in range(scene.num_bodies):
        c = scene.colliders[e][0]
        hid = w._hulls[(id(scene.meshes[c.mesh]), tuple(c.scale))]
        gv, gn, gt = w.hull_topology(hid)
        ov, on, ot = o.hull_topology(e)
        assert np.array_equal(gv, ov) and np.array_equal(gn, on)
        for k in range(4):
            assert np.array_equal(gt[k][0], ot[k][0]) and np.array_equal(gt[k][1], ot[k][1]), (e, k)
    w.close()


def test_cylinder_and_sphere_hull_shapes(ext_built):
    from rawphys import meshes as M
    w = ext_built.World(-1, "fp32")
    for mesh, nv, nf, maxval in ((M.cube(), 8, 6, 4), (M.icosahedron(), 12, 20, 3), (M.cylinder(32), 64, 34, 32),
                                 (M.icosphere(), 42, 80, 3)):
        h = w.hull(mesh.positions.astype(np.float64), mesh.indices)
        got_nv, faces = w.hull_faces(h)
        assert got_nv == nv and len(faces) == nf, mesh.name
        assert max(len(f[1]) for f in faces) == maxval
        # outward normals: every vertex lies behind every face plane
        v = w.hull_topology(h)[0]
        for n, el in faces:
            d = v @ np.asarray(n) - v[el[0]] @ np.asarray(n)
            assert np.all(d <= 1e-9), mesh.name
    w.close()


def test_host_only_world_refuses_gpu_work(ext_built):
    from rawphys import scenes as S
    w = ext_built.World(-1, "fp32")
    w.load(S.stack_scene(3))
    with pytest.raises(ext_built.RPError, match="RP_ERR_NO_DEVICE"):
        w.step(1)
    with pytest.raises(ext_built.RPError, match="RP_ERR_NO_DEVICE"):
        w.broad_pairs()
    st = w.get_state()             # snapshots still work on the host copy
    w.set_state(st)
    assert np.array_equal(w.get_state(), st)
    w.close()


def test_argument_validation(ext_built):
    rp = ext_built
    w = rp.World(-1, "fp32")
    cube = w.hull(np.array([[x, y, z] for x in (-1., 1.) for y in (-1., 1.) for z in (-1., 1.)]),
                  np.array([0, 1, 3], dtype=np.uint32))
    desc = [rp.ColliderDesc(rp.COLLIDER_HULL, cube, 0.0)]
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.entity(0, (0, 0, 0), (0, 0, 0, 1), -1.0, False, desc, 0.5, 0.3, 0.0)     # mass <= 0
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.entity(0, (0, 0, 0), (0, 0, 0, 1), 1.0, False, desc, 1.5, 0.3, 0.0)      # friction > 1
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.entity(0, (np.nan, 0, 0), (0, 0, 0, 1), 1.0, False, desc, 0.5, 0.3, 0.0)
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.entity(3, (0, 0, 0), (0, 0, 0, 1), 1.0, False, desc, 0.5, 0.3, 0.0)      # no such scene
    with pytest.raises(rp.RPError, match="RP_ERR_DEGENERATE"):
        w.hull(np.zeros((3, 3)), np.array([0, 1, 2], dtype=np.uint32))            # open, degenerate "hull"
    bad = [rp.ColliderDesc(rp.COLLIDER_SPHERE, -1, 0.5), rp.ColliderDesc(rp.COLLIDER_HULL, cube, 0.0)]
    with pytest.raises(rp.RPError, match="RP_ERR_DEGENERATE"):                    # reference asserts
        w.entity(0, (0, 0, 0), (0, 0, 0, 1), 1.0, False, bad, 0.5, 0.3, 0.0)
    e = w.entity(0, (0, 0, 0), (0, 0, 0, 1), 1.0, True, [rp.ColliderDesc(rp.COLLIDER_SPHERE, -1, 0.5)], 0.5, 0.3, 0.0)
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.set_state(np.full((1, rp.STATE_DOUBLES), np.inf))
    assert e == 0 and w.num_entities() == 1
    # launch-shape and order settings: accepted values only, no device needed
    for cta in (0, 1, 96):
        w.set_sweep_assignment(cta)
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.set_sweep_assignment(-1)
    w.set_sweep_order("coloured")
    w.set_sweep_order("reference")
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.set_wait_limit(61_000_000)                                              # above 60 s
    w.close()


def test_scene_generators_are_deterministic():
    from rawphys import scenes as S
    a, b = S.large_scene(256, seed=3), S.large_scene(256, seed=3)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.rot, b.rot) and np.array_equal(a.mass, b.mass)
    # no two bounding spheres overlap at t = 0, all bodies inside the walls
    dyn = ~a.fixed
    p = a.pos[dyn]
    assert np.all(np.abs(p[:, 0]) < 20) and np.all(np.abs(p[:, 2]) < 20) and np.all((p[:, 1] > 0) & (p[:, 1] < 60))
    q = np.linalg.norm(a.rot, axis=1)
    assert np.allclose(q, 1.0)


def test_adjoint_on_a_host_only_world_and_its_arguments(ext_built):
    """The adjoint's argument checks run on the host: a host-only world reports RP_ERR_NO_DEVICE,
    a loss entity outside its scene or a zero checkpoint spacing RP_ERR_INVALID."""
    from rawphys import scenes as S
    rp = ext_built
    w = rp.World(-1, "fp64")
    w.load(S.domino_scene(3, seed=0))
    with pytest.raises(rp.RPError, match="RP_ERR_NO_DEVICE"):
        w.adjoint(2, [1], np.zeros(3))
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.adjoint(2, [1], np.zeros(3), checkpoint_every=0)
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID"):
        w.adjoint(2, [17], np.zeros(3))                               # no such entity
    prof = w.adjoint_profile()
    assert prof["tape_entries"] == 0
    w.close()


def test_domino_batch_generator():
    from rawphys import scenes as S
    b, last, target = S.domino_batch(12, seed=4)
    assert b.num_scenes == 12 and len(last) == 12 and target.shape == (12, 3)
    sizes = np.bincount(b.scene, minlength=12)
    assert np.all((sizes >= 16 + 2) & (sizes <= 64 + 2))          # floor + dominoes + thrown cube
    for s in range(12):
        idx = np.nonzero(b.scene == s)[0]
        assert b.fixed[idx[0]] and not b.fixed[idx[1:]].any()        # the floor first
        assert idx[0] < last[s] < idx[-1]                             # the last domino precedes the cube
        assert np.allclose(b.scale[last[s]], (0.1, 1.0, 0.5))
        assert b.vel[idx[-1], 0] >= 4.0                               # the cube flies at the row
    b2, last2, target2 = S.domino_batch(12, seed=4)
    assert np.array_equal(b.pos, b2.pos) and np.array_equal(target, target2)


def _cube_obj(quads=False, negative=False):
    """A unit-half-extent cube as OBJ text: 8 positions, faces as triangles with v/vt/vn indices (or
    as quads), optionally with negative (relative) indices."""
    v = [(x, y, z) for x in (-1.0, 1.0) for y in (-1.0, 1.0) for z in (-1.0, 1.0)]
    quads_ccw = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    lines = ["# test cube"] + ["v %.6f %.6f %.6f" % p for p in v] + ["vt 0 0", "vn 0 0 1"]
    def ref(i):
        return str(i - 8) if negative else str(i + 1)
    tris = []
    for q in quads_ccw:
        if quads:
            lines.append("f " + " ".join(ref(i) for i in q))
        else:
            for t in ((q[0], q[1], q[2]), (q[0], q[2], q[3])):
                lines.append("f " + " ".join("%s/1/1" % ref(i) for i in t))
                tris.append(t)
    return "\n".join(lines) + "\n", np.asarray(v), tris


def test_hull_from_obj_and_binary_cache(ext_built, tmp_path):
    rp = ext_built
    w = rp.World(-1, "fp64")
    text, v, tris = _cube_obj()
    obj = tmp_path / "cube.obj"
    obj.write_text(text)
    scale = (0.5, 0.25, 2.0)
    h = w.hull_from_obj(str(obj), scale)
    # the per-corner arrays obj_parse hands to collider_convex_hull_create: FP32 positions scaled in FP64
    corners = np.array([v[i].astype(np.float32).astype(np.float64) * scale for t in tris for i in t])
    assert w.hull(corners, np.arange(len(corners), dtype=np.uint32)) == h      # identical input, shared hull
    nv, faces = w.hull_faces(h)
    assert nv == 8 and len(faces) == 6                                         # coplanar triangles merged
    # negative indices and quads (split as a fan) give the same solid
    obj2 = tmp_path / "cube_neg_quads.obj"
    obj2.write_text(_cube_obj(quads=True, negative=True)[0])
    h2 = w.hull_from_obj(str(obj2), scale)
    v2, n2, _ = w.hull_topology(h2)
    v1, n1, _ = w.hull_topology(h)
    assert sorted(map(tuple, v2)) == sorted(map(tuple, v1))
    # binary cache: the restored hull has the same geometry and tables
    cache = tmp_path / "cube.rphull"
    w.hull_save(h, str(cache))
    h3 = w.hull_load(str(cache))
    assert h3 != h
    a, b = w.hull_topology(h), w.hull_topology(h3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    for k in a[2]:
        assert np.array_equal(a[2][k][0], b[2][k][0]) and np.array_equal(a[2][k][1], b[2][k][1])
    # a damaged cache or a malformed OBJ is refused
    raw = bytearray(cache.read_bytes())
    raw[40] ^= 0xFF
    bad = tmp_path / "bad.rphull"
    bad.write_bytes(bytes(raw))
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID.*checksum"):
        w.hull_load(str(bad))
    bad_obj = tmp_path / "bad.obj"
    bad_obj.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 9\n")
    with pytest.raises(rp.RPError, match="RP_ERR_INVALID.*face index"):
        w.hull_from_obj(str(bad_obj))
    w.close()


def test_hull_from_obj_matches_the_reference_reader(ext_built, tmp_path):
    """rp_hull_from_obj hands the hull builder the same face corners, in the same order, as the
    reference's OBJ reader (obj_parse with its vendored tinyobj loader; fixtures made by
    tests/golden/make_obj_golden.py): triangle files with texture / normal indices, quads, hexagons
    and octagons (ear clipping), negative indices. Equal corners give the identical hull id."""
    rp = ext_built
    from conftest import GOLDEN
    g = np.load(os.path.join(GOLDEN, "obj_corners.npz"))
    names = sorted(k[: -len("_corners")] for k in g.files if k.endswith("_corners"))
    assert len(names) >= 5
    w = rp.World(-1, "fp64")
    scale = (0.7, 1.3, 0.9)
    for name in names:
        path = tmp_path / (name + ".obj")
        path.write_text(str(g[name + "_text"]))
        h = w.hull_from_obj(str(path), scale)
        ref = g[name + "_corners"].astype(np.float64) * np.asarray(scale)
        assert w.hull(ref, np.arange(len(ref), dtype=np.uint32)) == h, name
    w.close()


def test_hull_cache_format_is_stable(ext_built, tmp_path):
    """The hull cache format is fixed: the committed file (the triangulated cube of half-extent 0.5,
    written by rp_hull_save; tests/golden/make_obj_golden.py) loads into the hull the same cube's
    OBJ builds, and saving that hull again gives the same bytes."""
    rp = ext_built
    from conftest import GOLDEN
    import make_obj_golden as mk
    fixture = os.path.join(GOLDEN, "cube_half.rphull")
    w = rp.World(-1, "fp64")
    h = w.hull_load(fixture)
    obj = tmp_path / "tri_cube.obj"
    obj.write_text(mk._tri_cube())
    h2 = w.hull_from_obj(str(obj), (0.5, 0.5, 0.5))
    a, b = w.hull_topology(h), w.hull_topology(h2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    for k in a[2]:
        assert np.array_equal(a[2][k][0], b[2][k][0]) and np.array_equal(a[2][k][1], b[2][k][1])
    out = tmp_path / "again.rphull"
    w.hull_save(h2, str(out))
    assert out.read_bytes() == open(fixture, "rb").read()
    w.close()


def test_obj_fixtures_match_the_live_reference_reader(tmp_path):
    """Where the reference harness is built (the reference checkout is present), its OBJ reader still
    gives the committed corners."""
    from oracle.oracle import Oracle, reference_available
    if not reference_available():
        pytest.skip("reference harness not built (no reference checkout)")
    from conftest import GOLDEN
    import make_obj_golden as mk
    g = np.load(os.path.join(GOLDEN, "obj_corners.npz"))
    o = Oracle("ref")
    for name, text in mk.obj_cases().items():
        path = tmp_path / (name + ".obj")
        path.write_text(text)
        assert str(g[name + "_text"]) == text, name
        assert np.array_equal(o.obj_corners(str(path)), g[name + "_corners"]), name


def test_bench_roofline_inputs():
    """bench.py's roofline inputs: the peak (MEASURED_PEAKS.json, or the stated fallback) and the
    position sweep's DRAM traffic per launch from its committed ncu summary (a missing summary or
    line is reported with its reason, never silently)."""
    sys.path.insert(0, ROOT)
    import bench
    peak, kind = bench.measured_peak_hbm()
    assert peak > 1000.0 and kind in ("measured", "fallback")
    traffic, src = bench.profile_traffic("pipeline_large4096.md", "k_sweep_grid (position sweep, cooperative grid)")
    assert traffic is not None and traffic > 0.0, src
    none, why = bench.profile_traffic("no_such_summary.md", "k")
    assert none is None and "missing" in why
    assert bench.SWEEP_CONTACT_B > 0 and bench.SWEEP_NODE_B > 0


def test_bench_sample_and_step_error():
    """The bench's size-stratified scene sample keeps the batch's size range, and the per-step error
    summary measures positions in metres and rotations as angles."""
    sys.path.insert(0, ROOT)
    import bench
    from rawphys import scenes as S
    from rawphys.precision import rotation_angle, step_error
    batch = S.batched_scenes(256, seed=0)
    picks = bench.stratified_scenes(batch, 32)
    sizes = np.bincount(batch.scene, minlength=batch.num_scenes)
    assert len(picks) >= 30 and sizes[picks].min() == sizes.min() and sizes[picks].max() == sizes.max()
    q = np.array([[0.0, 0.0, 0.0, 1.0]])
    half = 0.5e-4
    r = np.array([[np.sin(half), 0.0, 0.0, np.cos(half)]])
    assert abs(rotation_angle(q, r)[0] - 1e-4) < 1e-12
    assert abs(rotation_angle(q, -r)[0] - 1e-4) < 1e-12      # q and -q are the same rotation
    a = np.zeros((3, 28))
    a[:, 6] = 1.0
    b = a.copy()
    b[0, 0] = 3e-5
    b[1, 1] = 2e-4
    e = step_error(b, a, np.array([True, True, False]))
    assert e["bodies"] == 2 and abs(e["pos_m"]["max"] - 2e-4) < 1e-15 and e["within_1e-4"] == 0.5
    # the second body's 2e-4 m is within three times a reference that itself moves 1e-4 m under noise
    e = bench.with_spread(e, b, a, np.array([True, True, False]), np.array([0.0, 1e-4, 0.0]))
    assert e["within_1e-4_or_3x_spread"] == 1.0 and e["reference_spread_m"]["max"] == 1e-4
