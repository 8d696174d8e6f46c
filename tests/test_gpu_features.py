"""GPU behaviour beyond single-scene parity: batched scenes, edge cases the reference defines
(dt <= 0, collisions off, empty and all-fixed worlds, forces), sleeping islands, scratch
overflow and regrowth, device status, and the C++-mangled pbd_simulate drop-in."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batched_scenes_equal_separate_runs(ext_built, oracle_built):
    """Several independent scenes in one world, one launch per frame: each equals its own oracle run."""
    from rawphys import scenes as S
    parts = [S.stack_scene(6, seed=1), S.chain_scene(6, "spherical", seed=2), S.random_pile_scene(8, seed=3),
             S.sphere_scene(4, seed=1)]
    w = ext_built.World(0, "fp64")
    firsts = []
    for i, sc in enumerate(parts):
        sid = 0 if i == 0 else w.new_scene()
        firsts.append(w.load(sc, scene_id=sid))
    w.simulate(1.0 / 60.0, 20, 1, True, 25)
    got = w.get_state()
    for sc, f in zip(parts, firsts):
        o = oracle_built("port").load(sc)
        o.step(25)
        assert np.array_equal(got[f:f + sc.num_bodies], o.get_state()), sc.name
    w.close()


def test_dt_nonpositive_is_noop_and_collisions_off(ext_built, oracle_built):
    from rawphys import scenes as S
    sc = S.random_pile_scene(6, seed=2)
    w = ext_built.World(0, "fp64")
    w.load(sc)
    w.step(3)
    before = w.get_state()
    w.simulate(0.0, 20, 1, True, 1)
    w.simulate(-1.0, 20, 1, True, 1)
    assert np.array_equal(before, w.get_state())
    o = oracle_built("port").load(sc)
    o.set_state(before)
    o.step(4, collisions=False)
    w.simulate(sc.dt, sc.substeps, 1, False, 4)
    assert np.array_equal(w.get_state(), o.get_state())
    w.close()


def test_forces_match_oracle(ext_built, oracle_built):
    """entity_add_force in world and local frames, cleared after the frame (entity.cpp:176-195)."""
    from rawphys import scenes as S
    sc = S.random_pile_scene(5, seed=7)
    o = oracle_built("port").load(sc)
    w = ext_built.World(0, "fp64")
    w.load(sc)
    for frame in range(3):
        for tgt in (o, w):
            tgt.add_force(2, (0.1, 0.2, 0.0), (3.0, 0.0, -1.0 - frame), False)
            tgt.add_force(3, (0.0, 0.3, 0.1), (0.0, 5.0, 2.0), True)
        o.step(1)
        w.step(1)
        assert np.array_equal(w.get_state(), o.get_state()), frame
    o.step(2)          # forces were cleared after each frame on both sides
    w.step(2)
    assert np.array_equal(w.get_state(), o.get_state())
    w.close()


def test_empty_and_all_fixed_worlds(ext_built):
    rp = ext_built
    w = rp.World(0, "fp32")
    w.simulate(1.0 / 60.0, 20, 1, True, 3)          # no entities: no-op
    assert w.num_entities() == 0
    from rawphys import meshes as M
    cube = M.cube()
    h = w.hull(cube.positions.astype(np.float64) * 0.5, cube.indices)
    for x in range(3):
        w.entity(0, (x * 0.9, 0.0, 0.0), (0, 0, 0, 1), 0.0, True, [rp.ColliderDesc(rp.COLLIDER_HULL, h, 0.0)], 0.5, 0.3, 0.0)
    st = w.get_state()
    w.set_gravity(10.0)
    w.simulate(1.0 / 60.0, 20, 1, True, 5)
    after = w.get_state()
    assert np.array_equal(after[:, 0:7], st[:, 0:7])
    assert w.broad_pairs().shape == (3, 2)          # fixed-fixed pairs are listed, then skipped
    w.close()


def test_sleeping_islands_match_oracle(ext_built, oracle_built):
    """A settled stack goes to sleep after 1 s of slow motion, island by island (pbd.cpp:477-506)."""
    from rawphys import scenes as S
    sc = S.stack_scene(4, seed=5)
    o = oracle_built("port").load(sc)
    w = ext_built.World(0, "fp64")
    w.load(sc)
    o.step(150)
    w.step(150)
    a, b = o.get_state(), w.get_state()
    assert np.array_equal(a, b)
    assert a[1:, 26].min() == 0.0, "the stack should be asleep by now"
    w.close()


def test_scratch_overflow_regrows_and_redoes(ext_built, oracle_built, monkeypatch):
    from rawphys import scenes as S
    sc = S.random_pile_scene(10, seed=8)
    monkeypatch.setenv("RP_SCRATCH_SCALE", "0.0001")
    w = ext_built.World(0, "fp64")
    w.load(sc)
    w.step(60)
    o = oracle_built("port").load(sc)
    o.step(60)
    assert np.array_equal(w.get_state(), o.get_state())
    w.close()


def test_gjk_cycle_exit_keeps_reference_results(ext_built, oracle_built):
    """A settled pile of curved hulls (32-segment cylinders, icospheres) resting on the floor and
    walls: GJK runs that repeat a state stop early instead of running to the 100-iteration cap.
    Every pair's contacts stay bit-identical to the reference's in the FP64 build, and the early
    exit is exercised."""
    from rawphys import scenes as S
    sc = S.large_scene(1024, seed=0)
    w = ext_built.World(0, "fp64")
    w.load(sc)
    w.step(60)
    st = w.get_state()
    o = oracle_built("port").load(sc)
    o.set_state(st)
    pairs = o.broad_pairs()
    w.set_state(st)
    assert np.array_equal(w.broad_pairs(), pairs)
    c0 = w.counters()
    for a, b in pairs:
        assert np.array_equal(w.contacts(int(a), int(b)), o.contacts(int(a), int(b))), (a, b)
    c1 = w.counters()
    assert c1[18] > c0[18], "no GJK run ended on a repeated state"
    w.close()


def test_deep_overlap_and_status(ext_built):
    """Bodies spawned inside each other (EPA from deep penetration) run without fault; the device
    reports informational status only."""
    from rawphys import scenes as S
    sc = S.random_pile_scene(12, seed=9, spread=0.2)
    sc.pos[1:, 1] = 0.6 + 0.3 * np.arange(sc.num_bodies - 1)
    w = ext_built.World(0, "fp32")
    w.load(sc)
    w.step(30)
    st = w.get_state()
    assert np.all(np.isfinite(st))
    assert (w.status() & ~(1 << 8)) == 0
    w.close()


# ---------------------------------------------------------------------------------------------
# The pbd_simulate drop-in, driven through the reference's own data layout (rawphys.compat)

def oracle_callers(o, scene):
    """The scene as a reference caller holds it, with hull topology and mass properties taken from
    the oracle (the reference's own set-up, independent of this library's)."""
    from rawphys import compat
    topo = lambda b, k: o.hull_topology(b, k)

    def mass(b):
        I, Ii = o.inertia(b)
        return o.inverse_mass(b), I, Ii, o.radius(b)
    return compat.build_callers(scene, topology=topo, mass_properties=mass)


def _rot(q):
    x, y, z, w_ = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w_ * z), 2 * (x * z + w_ * y)],
                     [2 * (x * y + w_ * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w_ * x)],
                     [2 * (x * z - w_ * y), 2 * (y * z + w_ * x), 1 - 2 * (x * x + y * y)]])


def _check_transformed(ents):
    """Every hull's transformed vertices and normals follow the entity's final pose."""
    from rawphys import compat
    for ent in ents:
        col = compat.Collider.from_address(ent.colliders)
        if col.type != 1:
            continue
        h = col.convex_hull
        nv = C.c_size_t.from_address(h.vertices - 8).value
        v = (compat.Vec3 * nv).from_address(h.vertices)
        tv = (compat.Vec3 * nv).from_address(h.transformed_vertices)
        R = _rot([ent.world_rotation.x, ent.world_rotation.y, ent.world_rotation.z, ent.world_rotation.w])
        p = np.array([ent.world_position.x, ent.world_position.y, ent.world_position.z])
        for i in range(nv):
            assert np.allclose([tv[i].x, tv[i].y, tv[i].z], R @ np.array([v[i].x, v[i].y, v[i].z]) + p, atol=1e-12)
        nf = C.c_size_t.from_address(h.faces - 8).value
        fs = (compat.HullFace * nf).from_address(h.faces)
        tf = (compat.HullFace * nf).from_address(h.transformed_faces)
        for f in range(nf):
            n = R @ np.array([fs[f].normal.x, fs[f].normal.y, fs[f].normal.z])
            assert np.allclose([tf[f].normal.x, tf[f].normal.y, tf[f].normal.z], n / np.linalg.norm(n), atol=1e-12)


def test_pbd_simulate_dropin(ext_built, oracle_built, monkeypatch):
    """A caller holding the reference's Entity / Collider / Physics_Force structs calls the mangled
    pbd_simulate, adding gravity before each frame and clearing it after, as the examples do; with
    the FP64 kernels the result equals the oracle bit for bit, the transformed hulls follow the final
    poses, and steady frames upload nothing (state unchanged, gravity kept on the device)."""
    from rawphys import compat, scenes as S
    monkeypatch.setenv("RP_SHIM_PRECISION", "fp64")
    lib = C.CDLL(ext_built.LIB_PATH)
    lib.rp_compat_reset()
    lib.rp_compat_world.restype = C.c_void_p
    sim, _ = compat.dropin(lib)
    sc = S.stack_scene(5, seed=2)
    o = oracle_built("port").load(sc)
    callers = oracle_callers(o, sc)
    h2d = []
    for frame in range(4):
        callers.add_gravity(sc.gravity)
        sim(sc.dt, callers.array, 20, 1, 1)
        callers.clear_forces()
        o.step(1)
        assert np.array_equal(callers.state(), o.get_state()), frame
        tb = (C.c_uint64 * 2)()
        assert ext_built.load_library().rp_transfer_bytes(C.c_void_p(lib.rp_compat_world()), tb) == 0
        h2d.append(tb[0])
    assert h2d[3] == h2d[1], "steady frames must upload nothing: %s" % h2d
    _check_transformed(callers.entities)
    lib.rp_compat_reset()


@pytest.mark.parametrize("name", ["springs", "chain8_hinge", "chain8_spherical"])
def test_pbd_simulate_with_constraints_dropin(ext_built, oracle_built, monkeypatch, name):
    """The mangled pbd_simulate_with_constraints over the reference's Constraint light array
    (positional with rest offsets, mutual orientation, hinge and spherical joints with limits): FP64
    bit-exact to the oracle over several frames, and the caller's constraints are never written."""
    from rawphys import compat
    from make_golden import SCENES
    monkeypatch.setenv("RP_SHIM_PRECISION", "fp64")
    lib = C.CDLL(ext_built.LIB_PATH)
    lib.rp_compat_reset()
    _, simc = compat.dropin(lib)
    sc = SCENES[name][0]()
    o = oracle_built("port").load(sc)
    callers = oracle_callers(o, sc)
    nc = len(sc.constraints)
    before = bytes((C.c_ubyte * (144 * nc)).from_address(callers.constraints))
    for frame in range(6):
        callers.add_gravity(sc.gravity)
        simc(sc.dt, callers.array, callers.constraints, sc.substeps, 1, int(sc.collisions))
        callers.clear_forces()
        o.step(1)
        assert np.array_equal(callers.state(), o.get_state()), (name, frame)
    assert bytes((C.c_ubyte * (144 * nc)).from_address(callers.constraints)) == before
    lib.rp_compat_reset()


def test_pbd_simulate_dropin_fp32_default(ext_built, oracle_built, monkeypatch):
    """The drop-in in its default FP32 mode: per-frame position error from identical states against
    the oracle within 1e-4 m at the median on a pile and the spring scene, transformed hulls exact at
    the final pose (computed on the device in FP64 in either mode)."""
    from rawphys import compat, scenes as S
    from rawphys.precision import step_error
    from make_golden import SCENES
    monkeypatch.delenv("RP_SHIM_PRECISION", raising=False)
    lib = C.CDLL(ext_built.LIB_PATH)
    _, simc = compat.dropin(lib)
    for sc in (S.random_pile_scene(12, seed=1), SCENES["springs"][0]()):
        lib.rp_compat_reset()
        o = oracle_built("port").load(sc)
        callers = oracle_callers(o, sc)
        o.step(30)
        for frame in range(3):
            st = o.get_state()
            callers.set_state(st)
            callers.add_gravity(sc.gravity)
            simc(sc.dt, callers.array, callers.constraints or None, sc.substeps, 1, 1)
            callers.clear_forces()
            o.step(1)
            err = step_error(callers.state(), o.get_state(), ~sc.fixed)
            assert err["pos_m"]["median"] <= 1e-4, (sc.name, frame, err)
        _check_transformed(callers.entities)
    lib.rp_compat_reset()


def test_batched_form_matches_oracle_per_scene(ext_built, oracle_built):
    """The batched form (many scenes of uneven size, a quarter with hinge or spherical chains) in one
    world: every scene's trajectory equals the oracle's run of that scene alone, bit for bit in the
    FP64 build, in both launch modes."""
    from rawphys import scenes as S
    batch = S.batched_scenes(12, seed=5, min_bodies=2, max_bodies=40, chain_fraction=0.5, chain_links=(8, 12))
    frames = 8
    got = {}
    for mode in ("phased", "persistent"):
        w = ext_built.World(0, "fp64")
        w.set_mode(mode)
        first = w.load_batch(batch)
        w.simulate(batch.dt, batch.substeps, batch.pos_iters, batch.collisions, frames)
        got[mode] = w.get_state()[first:]
        assert (w.status() & ~(1 << 8)) == 0
        w.close()
    assert np.array_equal(got["phased"], got["persistent"])
    for s in range(batch.num_scenes):
        idx = np.nonzero(batch.scene == s)[0]
        o = oracle_built("port").load(S.batch_scene(batch, s))
        o.step(frames)
        assert np.array_equal(got["phased"][idx], o.get_state()), "scene %d" % s


def test_fp32_persistent_and_phased_forms_agree(ext_built):
    """The FP32 build in its two launch modes (one persistent kernel per frame; the phase-major
    pipeline) runs the same substep on contact scenes: from the same state, one frame of a batch of
    piles agrees to rounding for most bodies (median <= 1e-6 m, 95th percentile <= 1e-4 m), and
    within the FP32 build's per-step spread where a contact's sign test flips (<= 5e-2 m). (Joint
    chains are left out: their links meet face to face, and the phase-major form redoes such
    FP32-degenerate pairs in FP64 while the persistent form keeps the FP32 result.)"""
    from rawphys import scenes as S
    batch = S.batched_scenes(16, seed=11, min_bodies=2, max_bodies=48, chain_fraction=0.0)
    got, start = {}, None
    for mode in ("phased", "persistent"):
        w = ext_built.World(0, "fp32")
        w.set_mode(mode)
        first = w.load_batch(batch)
        if start is None:
            w.simulate(batch.dt, batch.substeps, batch.pos_iters, batch.collisions, 3)
            start = w.get_state()
        w.set_state(start)
        w.simulate(batch.dt, batch.substeps, batch.pos_iters, batch.collisions, 1)
        got[mode] = w.get_state()[first:]
        assert (w.status() & ~(1 << 8)) == 0
        w.close()
    d = np.linalg.norm(got["phased"][:, 0:3] - got["persistent"][:, 0:3], axis=1)
    assert np.median(d) <= 1e-6 and np.percentile(d, 95) <= 1e-4 and d.max() <= 5e-2, \
        (np.median(d), np.percentile(d, 95), d.max())


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batched_sweep_assignments_agree(ext_built, precision):
    """The batched sweeps' scene assignment is a launch shape only: one warp per scene, one CTA per
    scene and the hybrid (a CTA for the costlier scenes) give bit-identical trajectories in the FP64
    build (compiled without FMA contraction), so the schedule is the same. In the FP32 build the
    compiler may contract a multiply-add differently in each kernel instantiation; one frame from the
    same state then differs at rounding level for most bodies (median <= 1e-6 m), and by at most the
    FP32 build's own per-step spread where a contact's sign test flips (<= 1e-2 m; the FP32-vs-FP64
    per-step maximum on the batched workload is of that order)."""
    from rawphys import scenes as S
    batch = S.batched_scenes(24, seed=7, min_bodies=2, max_bodies=60, chain_fraction=0.5, chain_links=(8, 16))
    frames = 6 if precision == "fp64" else 1
    start = None
    got = {}
    for cta in (0, 1, 24):
        w = ext_built.World(0, precision)
        w.set_sweep_assignment(cta)
        first = w.load_batch(batch)
        if start is None:
            w.simulate(batch.dt, batch.substeps, batch.pos_iters, batch.collisions, 3)
            start = w.get_state()
        w.set_state(start)
        w.simulate(batch.dt, batch.substeps, batch.pos_iters, batch.collisions, frames)
        got[cta] = w.get_state()[first:]
        assert (w.status() & ~(1 << 8)) == 0
        w.close()
    for cta in (1, 24):
        if precision == "fp64":
            assert np.array_equal(got[0], got[cta]), cta
        else:
            d = np.linalg.norm(got[0][:, 0:3] - got[cta][:, 0:3], axis=1)
            assert np.median(d) <= 1e-6 and d.max() <= 1e-2, (cta, np.median(d), d.max())
    with pytest.raises(ext_built.RPError):
        w = ext_built.World(0, precision)
        try:
            w.set_sweep_assignment(-1)
        finally:
            w.close()


def test_batched_form_fp32_per_step_error(ext_built, oracle_built):
    """FP32 batched form: per-step position error from identical states against the oracle, per
    scene of a mixed batch (contacts and joints)."""
    from rawphys import scenes as S
    batch = S.batched_scenes(8, seed=6, min_bodies=4, max_bodies=30, chain_fraction=0.25, chain_links=(8, 10))
    w = ext_built.World(0, "fp32")
    first = w.load_batch(batch)
    w.simulate(batch.dt, batch.substeps, 1, True, 30)
    st = w.get_state()[first:]
    w.simulate(batch.dt, batch.substeps, 1, True, 1)
    nxt = w.get_state()[first:]
    errs = []
    for s in range(batch.num_scenes):
        idx = np.nonzero(batch.scene == s)[0]
        o = oracle_built("port").load(S.batch_scene(batch, s))
        o.set_state(st[idx])
        o.step(1)
        errs.append(float(np.max(np.abs(o.get_state()[:, 0:3] - nxt[idx, 0:3]))))
    assert np.median(errs) <= 1e-4, errs
    w.close()


def test_autotune_keeps_results_and_state(ext_built, oracle_built):
    """rp_autotune times every launch configuration from the current state, restores it, and the
    chosen configuration gives the oracle's results bit for bit (FP64 build)."""
    from rawphys import scenes as S
    for sc in (S.random_pile_scene(10, seed=12), S.large_scene(1024, seed=1)):
        w = ext_built.World(0, "fp64")
        w.load(sc)
        w.step(2)
        st = w.get_state()
        choice = w.autotune(frames=2)
        assert choice["mode"] in ("phased", "persistent")
        assert np.array_equal(w.get_state(), st)
        w.step(3)
        o = oracle_built("port").load(sc)
        o.set_state(st)
        o.step(3)
        assert np.array_equal(w.get_state(), o.get_state()), (sc.name, choice)
        w.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sorted_broad_phase_grid_wide_sort(ext_built, oracle_built, precision):
    """A single scene above one CTA's sort size (16384 bodies) takes the grid-wide radix passes of
    the sort-based broad phase: 17000 small cubes on a jittered grid over a floor, about five pairs a
    body plus the floor's row of 17000. Same pairs, same order as the reference."""
    from rawphys import scenes as S
    rng = np.random.default_rng(3)
    b = S._Builder("grid17k")
    S._floor(b, (60.0, 0.5, 60.0))
    for i in range(17000):
        x, z = i % 130, i // 130
        p = (x * 0.45 - 29.0 + rng.uniform(-0.05, 0.05), 0.2 + rng.uniform(0.0, 0.3), z * 0.45 - 29.0 + rng.uniform(-0.05, 0.05))
        b.hull_body("cube", (0.2, 0.2, 0.2), p, mass=0.064)
    sc = b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=True, steps=1)
    o = oracle_built("port").load(sc)
    w = ext_built.World(0, precision)
    w.load(sc)
    pairs = w.broad_pairs()
    ref = o.broad_pairs()
    assert len(ref) > 17000 * 3
    assert np.array_equal(pairs, ref)
    w.close()


@pytest.mark.parametrize("mode", ["phased", "persistent"])
def test_wait_limit_runs_out_undoes_the_call_and_world_recovers(ext_built, oracle_built, mode):
    """Failure detection without a GPU fault: with the wait limit at 0 every grid barrier of the
    cooperative launches gives up at its first incomplete check. The frame is abandoned (each CTA
    leaves the launch, later kernels return at once), rp_simulate restores the starting state and
    returns RP_ERR_TIMEOUT; with the default limit back the world steps exactly as the oracle."""
    from rawphys import scenes as S
    sc = S.large_scene(1024, seed=1)          # one scene of >= 256 bodies: the cooperative grid path
    w = ext_built.World(0, "fp64")
    w.set_mode(mode)
    w.load(sc)
    w.step(2)
    start = w.get_state()
    w.set_wait_limit(0)
    with pytest.raises(ext_built.RPError, match="RP_ERR_TIMEOUT"):
        w.step(1)
    assert np.array_equal(w.get_state(), start), "a timed-out call must leave the state as it found it"
    w.set_wait_limit(1_000_000)
    w.step(1)
    w.sync()
    o = oracle_built("port").load(sc)
    o.set_state(start)
    o.step(1)
    assert np.array_equal(w.get_state(), o.get_state())
    w.close()


def _check_schedule(lev, bod, ne, which, order):
    """The properties a sweep schedule must have: velocity sweeps hold no external constraint; in
    reference order every active node's level is one more than the latest earlier active node on
    either of its bodies (so shared-body nodes keep constraint order and levels are as short as that
    allows); in coloured order no two active nodes of one colour share a dynamic body."""
    act = lev >= 0
    if which == 1:
        assert not act[:ne].any(), "an external constraint in the velocity sweep"
    if order == "reference":
        last = {}
        for k in np.nonzero(act)[0]:
            bs = [int(b) for b in bod[k] if b >= 0]
            expect = 1 + max([last.get(b, -1) for b in bs] + [-1])
            assert lev[k] == expect, (k, lev[k], expect)
            for b in bs:
                last[b] = int(lev[k])
    else:
        for c in np.unique(lev[act]):
            bs = bod[(lev == c)].ravel()
            bs = bs[bs >= 0]
            assert len(bs) == len(np.unique(bs)), "colour %d: two constraints share a body" % c
    return int(lev.max()) + 1 if act.any() else 0


@pytest.mark.parametrize("order", ["reference", "coloured"])
def test_sweep_schedules_are_valid(ext_built, order):
    """The per-substep sweep schedules (built after each substep's narrowphase from the constraints
    that act in it) of a pile and of a hinge chain, in both Gauss-Seidel orders."""
    from rawphys import scenes as S
    parts = [S.random_pile_scene(16, seed=4), S.chain_scene(24, "hinge", seed=2)]
    w = ext_built.World(0, "fp32")
    w.set_sweep_order(order)
    for i, sc in enumerate(parts):
        w.load(sc, scene_id=0 if i == 0 else w.new_scene())
    w.simulate(1.0 / 60.0, 20, 1, True, 12)
    depth = {}
    for s, sc in enumerate(parts):
        for which in (0, 1):
            lev, bod = w.last_schedule(s, which)
            depth[(s, which)] = _check_schedule(lev, bod, len(sc.constraints), which, order)
    assert depth[(0, 0)] > 0 and depth[(1, 0)] > 0
    if order == "coloured":
        assert depth[(1, 0)] <= 6, "a chain needs a few colours, not one per link"
    else:
        assert depth[(1, 0)] >= 23, "reference order keeps one step per chain link"
    w.close()
