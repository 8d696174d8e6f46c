"""Generate the golden fixtures of tests/golden/ from the reference's own physics sources.

Runs oracle/_ref/libref_harness.so (raw-physics' src/physics/*.cpp, entity.cpp, quaternion.cpp and
util.cpp compiled headless by oracle/Makefile with -O2 -ffp-contract=off, asserts on) on seeded
scenes of raw-physics_gb300/rawphys/scenes.py and stores, per scene, in <scene>.npz:
  steps, states     full entity state (oracle/harness.h layout) after selected frame counts
  pairs0            broad_get_collision_pairs on the initial state
  kat_state, kat_pairs, kat_counts, kat_contacts
                    colliders_get_contacts on every broad-phase pair of one mid-run state
  invm, inertia, inverse_inertia, radius
                    entity_create's derived mass properties
plus meta.json (compiler, flags, machine). Regenerate with
    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import platform
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "raw-physics_gb300"))
sys.path.insert(0, ROOT)

from rawphys import scenes as S  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

# name -> (scene factory, frame counts to record, frame count of the contact known-answer state)
SCENES = {
    "stack10": (lambda: S.stack_scene(10, seed=0), [0, 1, 2, 5, 10, 30, 60, 100, 200, 300], 30),
    "pile12": (lambda: S.random_pile_scene(12, seed=1), [0, 1, 10, 40, 80, 120], 40),
    "pile16": (lambda: S.random_pile_scene(16, seed=2), [0, 1, 10, 40, 80, 120], 60),
    "chain8_hinge": (lambda: S.chain_scene(8, "hinge", seed=1), [0, 1, 10, 50, 100], 20),
    "chain8_spherical": (lambda: S.chain_scene(8, "spherical", seed=0), [0, 1, 10, 50, 100], 20),
    "chain6_hinge_free": (lambda: S.chain_scene(6, "hinge", seed=3, collisions=False), [0, 1, 10, 50], 10),
    "domino16": (lambda: S.domino_scene(16, seed=0), [0, 1, 10, 40, 80, 120], 40),
    "spheres6": (lambda: S.sphere_scene(6, seed=0), [0, 1, 10, 40, 60], 40),
    "tower12": (lambda: S.tower_scene(12, ratio=100.0, seed=0), [0, 1, 5, 20, 60], 20),
    "large1024": (lambda: S.large_scene(1024, seed=0), [0, 1], 0),
    "springs": (lambda: S.spring_scene(seed=0), [0, 1, 10, 40, 100, 200], 40),
}


def generate(name: str, ref: Oracle) -> dict:
    make, record, kat_at = SCENES[name]
    scene = make()
    ref.load(scene)
    n = scene.num_bodies
    out = {"invm": np.array([ref.inverse_mass(e) for e in range(n)]),
           "radius": np.array([ref.radius(e) for e in range(n)])}
    inert = [ref.inertia(e) for e in range(n)]
    out["inertia"] = np.array([I.reshape(9) for I, _ in inert])
    out["inverse_inertia"] = np.array([Ii.reshape(9) for _, Ii in inert])
    out["pairs0"] = ref.broad_pairs().astype(np.int32)
    states, done = [], 0
    for k in record:
        if kat_at == k and "kat_state" not in out:
            pass
        while done < k:
            if done == kat_at and "kat_state" not in out:
                out.update(kat(ref))
            ref.step(1)
            done += 1
        if done == kat_at and "kat_state" not in out:
            out.update(kat(ref))
        st = ref.get_state()
        states.append(st[:, 0:7] if name.startswith("large") and k > 0 else st)
    out["steps"] = np.array(record)
    if name.startswith("large"):
        out["states"] = states[0]
        out["pos_rot_1"] = states[1]
        for k in ("inertia", "inverse_inertia", "kat_state", "kat_pairs", "kat_counts", "kat_contacts"):
            out.pop(k, None)
    else:
        out["states"] = np.stack(states)
    return out


def kat(ref: Oracle) -> dict:
    """Contacts of every broad-phase pair after moving each dynamic body 2 mm down, so that
    resting contacts penetrate as they do inside a substep."""
    st = ref.get_state()
    moved = st.copy()
    dyn = np.array([ref.inverse_mass(e) > 0.0 for e in range(st.shape[0])])
    moved[dyn, 1] -= 0.002
    ref.set_state(moved)
    pairs = ref.broad_pairs()
    counts, conts = [], []
    for a, b in pairs:
        c = ref.contacts(int(a), int(b))
        counts.append(len(c))
        conts.append(c)
    ref.set_state(st)
    return {"kat_state": moved, "kat_pairs": pairs.astype(np.int32), "kat_counts": np.array(counts, dtype=np.int32),
            "kat_contacts": np.concatenate(conts) if conts else np.zeros((0, 9))}


def main(names=None) -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    ref = Oracle("reference")
    for name in names or SCENES:
        data = generate(name, ref)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, {k: getattr(v, "shape", None) for k, v in data.items()})
    cxx = subprocess.run(["g++", "--version"], capture_output=True, text=True).stdout.splitlines()[0]
    meta = {"generator": "oracle/_ref/libref_harness.so (reference physics sources, headless)",
            "flags": "-O2 -ffp-contract=off -fno-fast-math (asserts enabled)", "compiler": cxx,
            "machine": platform.machine(), "scenes": list(SCENES)}
    with open(os.path.join(HERE, "meta.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
