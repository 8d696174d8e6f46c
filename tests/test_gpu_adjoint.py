"""Adjoint of the collision-free step (rp_adjoint_trajectory): its forward pass reproduces the FP64
build's trajectory bit for bit, and its gradients with respect to initial velocities and masses
match FP64 central finite differences of the FP64 build. A torch.autograd.Function built on it (test
harness only) returns the same gradients through loss.backward().

Horizons: spherical chains over 24 frames of 20 substeps (h = 1e-6 relative). Hinge chains whose axes
are all parallel keep their axis misalignment theta small (of order g h^2 / L, about 1e-5 rad), and the hinge
alignment divides by |a1 x a2| (src/physics/pbd.cpp:251-262,
src/physics/pbd_base_constraints.cpp:133-148), so the loss has curvature of order
1/theta that compounds over substeps: the central difference itself stops converging after ~15
substeps (at 20 substeps h = 1e-6 gives -3.4 where h = 1e-8 gives -8.61 and the adjoint -8.587).
Hinges are therefore checked over 12 substeps with h = 1e-7, where every step size from 1e-7 to 1e-8
agrees to 1e-5."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FRAMES = 24


def _scene(kind):
    from rawphys import scenes as S
    sc = S.chain_scene(5, kind, seed=4, collisions=False)
    return sc


def _loss(rp, sc, state, run, masses=None, entity=None, target=None):
    w = rp.World(0, "fp64")
    w.load(sc)
    if masses is not None:
        for e, m in masses.items():
            invm, I, Ii, r = w.mass_properties(e)
            m0 = 1.0 / invm
            w.set_mass_properties(e, 1.0 / m, I * (m / m0), Ii * (m0 / m), r)
    w.set_state(state)
    dt, substeps, frames = run
    w.simulate(dt, substeps, sc.pos_iters, False, frames)
    x = w.get_state()[entity, 0:3]
    w.close()
    return float(np.sum((x - target) ** 2))


# (joint, frames, dt, substeps per frame, relative FD step)
RUNS = [("spherical", FRAMES, 1.0 / 60.0, 20, 1e-6), ("hinge", 12, 1.0 / 1200.0, 1, 1e-7)]


@pytest.mark.parametrize("kind,frames,dt,substeps,hrel", RUNS)
def test_adjoint_forward_matches_fp64_step_and_fd(ext_built, kind, frames, dt, substeps, hrel):
    rp = ext_built
    sc = _scene(kind)
    run = (dt, substeps, frames)
    entity = sc.num_bodies - 1
    target = np.array([0.3, -2.0, 0.4])
    w = rp.World(0, "fp64")
    w.load(sc)
    w.simulate(sc.dt, sc.substeps, sc.pos_iters, False, 3)     # swinging, every body awake
    state = w.get_state()
    res = w.adjoint(frames, [entity], target, checkpoint_every=5, dt=dt, substeps=substeps)
    # the adjoint's own forward pass is the FP64 step
    w.simulate(dt, substeps, sc.pos_iters, False, frames)
    x = w.get_state()[entity, 0:3]
    assert res["loss"][0] == float(np.sum((x - target) ** 2))
    w.close()
    rng = np.random.default_rng(7)
    dyn = np.nonzero(~sc.fixed)[0]
    checks = []
    for _ in range(4):
        e, k = int(rng.choice(dyn)), int(rng.integers(0, 6))
        col = 7 + k
        hstep = hrel * max(1.0, abs(state[e, col]))
        sp, sm = state.copy(), state.copy()
        sp[e, col] += hstep
        sm[e, col] -= hstep
        fd = (_loss(rp, sc, sp, run, entity=entity, target=target)
              - _loss(rp, sc, sm, run, entity=entity, target=target)) / (2 * hstep)
        ad = (res["grad_v"] if k < 3 else res["grad_w"])[e, k % 3]
        checks.append((e, k, fd, ad))
    w2 = rp.World(0, "fp64")
    w2.load(sc)
    masses0 = {int(e): 1.0 / w2.mass_properties(int(e))[0] for e in dyn[:2]}
    w2.close()
    for e, m in masses0.items():
        hstep = hrel * m
        fd = (_loss(rp, sc, state, run, {e: m + hstep}, entity, target)
              - _loss(rp, sc, state, run, {e: m - hstep}, entity, target)) / (2 * hstep)
        checks.append((e, "mass", fd, res["grad_mass"][e]))
    scale = max(abs(c[2]) for c in checks)
    for e, k, fd, ad in checks:
        assert abs(ad - fd) <= 1e-3 * max(abs(fd), 1e-3 * scale), (kind, e, k, fd, ad)
    assert np.all(res["grad_friction"] == 0.0)


def test_adjoint_through_torch_autograd(ext_built):
    torch = pytest.importorskip("torch")
    rp = ext_built
    sc = _scene("hinge")
    entity = sc.num_bodies - 1
    target = np.array([0.0, -1.5, 0.0])
    w = rp.World(0, "fp64")
    w.load(sc)
    w.simulate(sc.dt, sc.substeps, sc.pos_iters, False, 2)
    state = w.get_state()

    class Rollout(torch.autograd.Function):
        @staticmethod
        def forward(ctx, v0):
            st = state.copy()
            st[:, 7:10] = v0.detach().cpu().numpy()
            w.set_state(st)
            res = w.adjoint(FRAMES, [entity], target, checkpoint_every=4)
            ctx.save_for_backward(torch.from_numpy(res["grad_v"]))
            return torch.tensor(res["loss"][0], dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            (gv,) = ctx.saved_tensors
            return g * gv

    v0 = torch.tensor(state[:, 7:10], dtype=torch.float64, requires_grad=True)
    loss = Rollout.apply(v0)
    loss.backward()
    w.set_state(state)
    ref = w.adjoint(FRAMES, [entity], target, checkpoint_every=8)     # another checkpoint spacing
    assert np.allclose(v0.grad.numpy(), ref["grad_v"], rtol=1e-12, atol=1e-15)
    w.close()


# ---------------------------------------------------------------------------------------------
# Contacts: a unit cube sliding on the floor (dynamic friction acting the whole time) and a thrown
# cube reaching a domino row. Over these horizons the contact set does not change within the FD
# steps, so the loss is smooth there and FP64 central differences converge (h = 1e-6 relative).

def _slide_scene():
    from rawphys import scenes as S
    b = S._Builder("slide")
    S._floor(b, (10.0, 0.5, 10.0))
    b.hull_body("cube", (0.5, 0.5, 0.5), (0.0, 0.5, 0.0), mass=1.0, v=(2.0, 0.0, 0.5))
    return b.finish(dt=1.0 / 60.0, substeps=20, pos_iters=1, collisions=True, steps=60)


def _contact_loss(rp, sc, state, frames, entity, target, masses=None):
    w = rp.World(0, "fp64")
    w.load(sc)
    for e, m in (masses or {}).items():
        invm, I, Ii, r = w.mass_properties(e)
        m0 = 1.0 / invm
        w.set_mass_properties(e, 1.0 / m, I * (m / m0), Ii * (m0 / m), r)
    w.set_state(state)
    w.simulate(sc.dt, sc.substeps, sc.pos_iters, True, frames)
    x = w.get_state()[entity, 0:3]
    w.close()
    return float(np.sum((x - target) ** 2))


def _contact_case(name):
    from rawphys import scenes as S
    if name == "slide":
        sc = _slide_scene()
        return sc, 20, 1, np.array([1.0, 0.5, 0.3]), [(1, 7), (1, 8), (1, 9), (1, 10)], [1], [(1, 1), (0, 1), (1, 0)]
    sc = S.domino_scene(4, seed=1)
    n = sc.num_bodies
    return sc, 15, n - 1, np.array([1.0, 1.5, 0.2]), [(n - 1, 7), (n - 1, 9), (n - 1, 10), (n - 1, 12)], [n - 1], [(n - 1, 1)]


@pytest.mark.parametrize("name", ["slide", "domino"])
def test_adjoint_contacts_match_fd(ext_built, name):
    rp = ext_built
    sc, frames, entity, target, comps, masses, fric = _contact_case(name)
    w = rp.World(0, "fp64")
    w.load(sc)
    state = w.get_state()
    res = w.adjoint(frames, [entity], target, checkpoint_every=4)
    w.simulate(sc.dt, sc.substeps, sc.pos_iters, True, frames)
    x = w.get_state()[entity, 0:3]
    assert res["loss"][0] == float(np.sum((x - target) ** 2))     # the forward pass is the FP64 step
    w.close()
    checks = []
    for e, col in comps:
        h = 1e-6 * max(1.0, abs(state[e, col]))
        sp, sm = state.copy(), state.copy()
        sp[e, col] += h
        sm[e, col] -= h
        fd = (_contact_loss(rp, sc, sp, frames, entity, target) - _contact_loss(rp, sc, sm, frames, entity, target)) / (2 * h)
        ad = (res["grad_v"] if col < 10 else res["grad_w"])[e, (col - 7) % 3]
        checks.append((e, col, fd, ad))
    for e in masses:
        w = rp.World(0, "fp64")
        w.load(sc)
        m = 1.0 / w.mass_properties(e)[0]
        w.close()
        h = 1e-6 * m
        fd = (_contact_loss(rp, sc, state, frames, entity, target, {e: m + h})
              - _contact_loss(rp, sc, state, frames, entity, target, {e: m - h})) / (2 * h)
        checks.append((e, "mass", fd, res["grad_mass"][e]))
    for e, k in fric:
        arr = sc.mus if k == 0 else sc.mud
        old = arr[e]
        vals = []
        for sgn in (1.0, -1.0):
            arr[e] = old + sgn * 1e-6
            vals.append(_contact_loss(rp, sc, state, frames, entity, target))
        arr[e] = old
        checks.append((e, "friction%d" % k, (vals[0] - vals[1]) / 2e-6, res["grad_friction"][e, k]))
    scale = max(abs(c[2]) for c in checks)
    for e, k, fd, ad in checks:
        assert abs(ad - fd) <= 1e-3 * max(abs(fd), 1e-3 * scale), (name, e, k, fd, ad)
    assert np.all(res["grad_friction"][:, 0] == 0.0)     # static friction acts through a comparison only


def test_adjoint_batched_dominoes_equal_single_scenes(ext_built):
    from rawphys import scenes as S
    rp = ext_built
    batch, last, target = S.domino_batch(3, seed=5, min_dominoes=3, max_dominoes=6)
    frames = 10
    w = rp.World(0, "fp64")
    w.load_batch(batch)
    res = w.adjoint(frames, last, target, checkpoint_every=3)
    w.close()
    for s in range(batch.num_scenes):
        sc = S.batch_scene(batch, s)
        idx = np.nonzero(batch.scene == s)[0]
        b0 = int(idx[0])
        w1 = rp.World(0, "fp64")
        w1.load(sc)
        r1 = w1.adjoint(frames, [int(last[s]) - b0], target[s], checkpoint_every=5)
        w1.close()
        assert res["loss"][s] == r1["loss"][0]
        assert np.array_equal(res["grad_v"][idx], r1["grad_v"])
        assert np.array_equal(res["grad_w"][idx], r1["grad_w"])
        assert np.array_equal(res["grad_mass"][idx], r1["grad_mass"])
        assert np.array_equal(res["grad_friction"][idx], r1["grad_friction"])
