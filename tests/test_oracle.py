"""The oracle is pinned before it is trusted.

The oracle port (oracle/port/oracle.c) must reproduce, bit for bit, the fixtures generated from the
reference's own physics sources (tests/golden/make_golden.py): trajectories, broad-phase pair
lists, contact manifolds of every pair of a penetrating state, derived mass properties. Where the
reference build is present (this container), the port is also compared live against it.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, scene_fingerprint_ok
from make_golden import SCENES

SMALL = [n for n in SCENES if not n.startswith("large")]
# entity_create_ex leaves previous_world_position / _rotation unset (src/entity.cpp:24-65); they are
# defined from the first substep on, so frame 0 compares every other field
DEFINED_AT_FRAME0 = np.r_[0:13, 20:28]


@pytest.mark.parametrize("name", SMALL)
def test_port_trajectory_bitexact(oracle_built, name):
    g = golden(name)
    scene = SCENES[name][0]()
    assert scene_fingerprint_ok(scene, g), "scene generator differs from the fixture's"
    o = oracle_built("port").load(scene)
    done = 0
    for k, expect in zip(g["steps"], g["states"]):
        o.step(int(k) - done)
        done = int(k)
        got = o.get_state()
        cols = DEFINED_AT_FRAME0 if k == 0 else slice(None)
        assert np.array_equal(got[:, cols], expect[:, cols]), "%s differs from the reference after %d frames (max %.3g)" % (
            name, k, np.max(np.abs(got[:, cols] - expect[:, cols])))


@pytest.mark.parametrize("name", SMALL + ["large1024"])
def test_port_pairs_and_mass_properties(oracle_built, name):
    g = golden(name)
    scene = SCENES[name][0]()
    o = oracle_built("port").load(scene)
    assert np.array_equal(o.broad_pairs(), g["pairs0"])
    n = scene.num_bodies
    assert np.array_equal(np.array([o.inverse_mass(e) for e in range(n)]), g["invm"])
    assert np.array_equal(np.array([o.radius(e) for e in range(n)]), g["radius"])
    if "inertia" in g:
        for e in range(n):
            I, Ii = o.inertia(e)
            assert np.array_equal(I.reshape(9), g["inertia"][e])
            assert np.array_equal(Ii.reshape(9), g["inverse_inertia"][e])


@pytest.mark.parametrize("name", SMALL)
def test_port_contacts_known_answers(oracle_built, name):
    g = golden(name)
    o = oracle_built("port").load(SCENES[name][0]())
    o.set_state(g["kat_state"])
    k = 0
    for (a, b), cnt in zip(g["kat_pairs"], g["kat_counts"]):
        c = o.contacts(int(a), int(b))
        assert len(c) == cnt
        assert np.array_equal(c, g["kat_contacts"][k:k + cnt])
        k += cnt


@pytest.mark.parametrize("name", ["stack10", "chain8_hinge", "pile16"])
def test_port_manifold_for_given_normal(oracle_built, name):
    """clipping_get_contact_manifold with EPA's own normal reproduces colliders_get_contacts (single
    hull bodies), and with a tilted normal the port's manifold equals the reference's (live)."""
    from oracle.oracle import reference_available
    g = golden(name)
    scene = SCENES[name][0]()
    kinds = ["port"] + (["reference"] if reference_available() else [])
    outs = {}
    for kind in kinds:
        o = oracle_built(kind).load(scene)
        o.set_state(g["kat_state"])
        res = []
        k = 0
        for (a, b), cnt in zip(g["kat_pairs"], g["kat_counts"]):
            expect = g["kat_contacts"][k:k + cnt]
            k += cnt
            hit, e = o.gjk_epa(int(a), int(b))
            if hit != 1 or len(scene.colliders[a]) != 1 or len(scene.colliders[b]) != 1:
                continue
            assert np.array_equal(o.manifold(int(a), int(b), e[0:3], e[3]), expect), (kind, a, b)
            tilted = e[0:3] + np.array([1e-3, -2e-3, 1.5e-3])
            tilted /= np.linalg.norm(tilted)
            res.append(o.manifold(int(a), int(b), tilted, e[3]))
        outs[kind] = res
    if "reference" in outs:
        assert len(outs["port"]) == len(outs["reference"])
        for x, y in zip(outs["port"], outs["reference"]):
            assert np.array_equal(x, y)


def test_port_large_one_frame(oracle_built):
    g = golden("large1024")
    scene = SCENES["large1024"][0]()
    o = oracle_built("port").load(scene)
    o.step(1)
    assert np.array_equal(o.get_state()[:, 0:7], g["pos_rot_1"])


def test_port_matches_reference_live(oracle_built):
    from oracle.oracle import reference_available
    if not reference_available():
        pytest.skip("reference build not present (only where the reference checkout exists)")
    for name in ("stack10", "chain8_hinge", "spheres6", "springs"):
        scene = SCENES[name][0]()
        a = oracle_built("port").load(scene)
        a.step(40)
        sa = a.get_state()
        b = oracle_built("reference").load(scene)
        b.step(40)
        assert np.array_equal(sa, b.get_state())


def test_port_matches_reference_on_batched_scenes(oracle_built):
    """The port is the oracle of the batched workload's per-step error (bench.py), so it is also
    compared live with the reference on scenes of that generator: piles of the four hull shapes,
    hinge chains with +-pi/2 limits and spherical chains, a size-stratified handful, 12 frames each,
    bit for bit."""
    from oracle.oracle import reference_available
    from rawphys import scenes as S
    if not reference_available():
        pytest.skip("reference build not present (only where the reference checkout exists)")
    batch = S.batched_scenes(48, seed=0, max_bodies=256)
    sizes = np.bincount(batch.scene, minlength=batch.num_scenes)
    first_chain = {}
    for c in batch.constraints:
        first_chain.setdefault(c.kind, int(batch.scene[c.e2]))
    assert {"hinge", "spherical"} <= set(first_chain), first_chain
    picks = sorted(set([int(np.argmax(sizes)), int(np.argmin(sizes)), first_chain["hinge"], first_chain["spherical"]] +
                       [int(i) for i in np.argsort(sizes)[len(sizes) // 2:len(sizes) // 2 + 2]]))
    for s_ in picks:
        scene = S.batch_scene(batch, s_)
        a = oracle_built("port").load(scene)
        a.step(12)
        b = oracle_built("reference").load(scene)
        b.step(12)
        assert np.array_equal(a.get_state(), b.get_state()), "scene %d (%d bodies)" % (s_, sizes[s_])


def test_port_forces_and_edge_cases(oracle_built):
    """Extra forces (world and local frame), dt <= 0 no-op, collisions off: port == reference."""
    from oracle.oracle import reference_available
    from rawphys import scenes as S
    if not reference_available():
        pytest.skip("reference build not present")
    scene = S.random_pile_scene(6, seed=4)
    outs = []
    for kind in ("port", "reference"):
        o = oracle_built(kind).load(scene)
        o.add_force(2, (0.1, 0.2, 0.0), (3.0, 0.0, -1.0), local=False)
        o.add_force(3, (0.0, 0.3, 0.1), (0.0, 5.0, 2.0), local=True)
        o.step(1)
        before = o.get_state()
        o.step(1, dt=0.0)
        assert np.array_equal(before, o.get_state())
        o.step(3, collisions=False)
        outs.append(o.get_state())
    assert np.array_equal(outs[0], outs[1])


def test_port_speed_against_the_reference(oracle_built):
    """The port is the CPU baseline on machines without the reference checkout (the GPU host), so
    its speed relative to the reference's own build is recorded here: the same frames of the same
    scenes, same flags, same results. Printed (pytest -s) as body-substeps/s of each and their ratio;
    the assertion only keeps the comparison honest (equal results, both measured)."""
    import time
    from oracle.oracle import reference_available
    if not reference_available():
        pytest.skip("reference build not present (only where the reference checkout exists)")
    for name, settle, frames in (("stack10", 20, 20), ("large1024", 2, 3)):
        scene = SCENES[name][0]()
        rates, states = {}, {}
        for kind in ("port", "reference"):
            o = oracle_built(kind).load(scene)
            o.step(settle)
            t = time.perf_counter()
            o.step(frames)
            dt = time.perf_counter() - t
            rates[kind] = scene.num_dynamic * scene.substeps * frames / dt
            states[kind] = o.get_state()
        assert np.array_equal(states["port"], states["reference"]), name
        print("%s: port %.3g, reference %.3g body-substeps/s, port / reference %.2f"
              % (name, rates["port"], rates["reference"], rates["port"] / rates["reference"]))
