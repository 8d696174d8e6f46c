"""GPU parity: the CUDA step against the oracle, through the C ABI.

  * all-FP64 build: bit-identical to the oracle (itself pinned bit-exactly to the reference) over
    whole trajectories, pair lists and contact manifolds;
  * FP32 build: per-step position / orientation error from identical states within 1e-4 m / rad,
    except where the reference itself is ill-conditioned (a resting stack of exactly parallel faces:
    FP64-rounding-size input perturbations already move the reference's next frame by more than
    1e-4 m); there the bound is 3x the reference's own sensitivity, measured live.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, scene_fingerprint_ok
from make_golden import SCENES

pytestmark = pytest.mark.gpu

SMALL = [n for n in SCENES if not n.startswith("large")]
PREV_POSE = np.r_[13:20]          # undefined in the reference before the first substep
DEFINED = np.r_[0:13, 20:28]


def world(rp, scene, precision):
    w = rp.World(0, precision)
    w.load(scene)
    return w


@pytest.mark.parametrize("name", SMALL)
def test_fp64_trajectory_bitexact(ext_built, oracle_built, name):
    scene = SCENES[name][0]()
    o = oracle_built("port").load(scene)
    w = world(ext_built, scene, "fp64")
    w.set_state(o.get_state())
    g = golden(name)
    use_golden = scene_fingerprint_ok(scene, g)
    done = 0
    for k, expect in zip(g["steps"], g["states"]):
        k = int(k)
        o.step(k - done)
        w.step(k - done)
        done = k
        got, ref = w.get_state(), o.get_state()
        cols = DEFINED if k == 0 else slice(None)
        assert np.array_equal(got[:, cols], ref[:, cols]), "%s frame %d: max |diff| %.3g" % (
            name, k, np.max(np.abs(got[:, cols] - ref[:, cols])))
        if use_golden:
            assert np.array_equal(got[:, cols], expect[:, cols])
    assert w.status() & ~(1 << 8) == 0
    assert w.kernel_launches() >= g["steps"][-1]
    w.close()


def reference_sensitivity(o, state, rel=1e-12, trials=4, seed=0):
    """How far the reference's next frame moves when its input pose is perturbed at FP64-rounding
    scale: the floor below which no implementation that rounds differently can agree."""
    rng = np.random.default_rng(seed)
    o.set_state(state)
    o.step(1)
    base = o.get_state()
    worst = 0.0
    for _ in range(trials):
        p = state.copy()
        p[:, 0:7] *= 1.0 + rel * rng.standard_normal(p[:, 0:7].shape)
        o.set_state(p)
        o.step(1)
        worst = max(worst, float(np.max(np.abs(o.get_state()[:, 0:3] - base[:, 0:3]))))
    return worst


def contact_sets_agree(po, co, pg, cg, tol=1e-5, touch=1e-6):
    """Same collision constraints per pair (order-insensitive, within tol on r1, r2, normal);
    constraints whose two anchors coincide to `touch` may be present on one side only."""
    keys = set(map(tuple, po.tolist())) | set(map(tuple, pg.tolist()))
    for k in keys:
        a = co[(po == k).all(axis=1)]
        b = cg[(pg == k).all(axis=1)]
        if not _match_sets(a[:, 0:9], b[:, 0:9], tol, touch=touch, anchors=True):
            return False
    return True


@pytest.mark.parametrize("name", SMALL)
def test_fp32_substep_agreement(ext_built, oracle_built, name):
    """One substep at a time from identical states. Whenever the FP32 build generates the same
    contact set as the FP64 reference, positions and orientations agree within 1e-4 (in practice
    ~1e-6). Substeps where the two contact sets differ are discrete events the reference decides
    below FP32 resolution (a reference-face choice between faces parallel to ~1e-8, a contact
    touching at rounding level, a GJK/EPA that runs out of iterations on a curved hull); they must
    stay a minority."""
    scene = SCENES[name][0]()
    o = oracle_built("port").load(scene)
    o.step(SCENES[name][2] or 10)
    w = world(ext_built, scene, "fp32")
    h = scene.dt / scene.substeps
    agree_err, events, n = [], 0, 60
    for k in range(n):
        st = o.get_state()
        w.set_state(st)
        o.step(1, dt=h, substeps=1)
        w.simulate(h, 1, scene.pos_iters, scene.collisions, 1)
        a, b = o.get_state(), w.get_state()
        pe = float(np.max(np.abs(a[:, 0:3] - b[:, 0:3])))
        re = float(np.max(np.abs(a[:, 3:7] - b[:, 3:7])))
        same = True
        if scene.collisions:
            same = contact_sets_agree(*o.last_contacts(), *w.last_contacts())
        if same:
            assert pe <= 1e-4 and re <= 1e-4, "%s substep %d: %.3g m, %.3g rad with identical contacts" % (name, k, pe, re)
            agree_err.append(max(pe, re))
        else:
            events += 1
    assert events <= n // 4, "%s: %d of %d substeps diverge in their contact sets" % (name, events, n)
    assert np.median(agree_err) <= 1e-5, (name, np.median(agree_err))
    w.close()


@pytest.mark.parametrize("name", SMALL)
def test_fp32_frame_error(ext_built, oracle_built, name):
    """Whole frames (20 substeps) from identical states: the median error over 12 frames is within
    1e-4 m / rad, or within the reference's own response to an FP32-rounding-sized (1e-7 relative)
    perturbation of its input where the scene is ill-conditioned (resting stacks of parallel faces,
    hinge limits at +-90 degrees)."""
    scene = SCENES[name][0]()
    o = oracle_built("port").load(scene)
    o.step(SCENES[name][2] or 10)
    start = o.get_state()
    sens = reference_sensitivity(oracle_built("port").load(scene), start, rel=1e-7)
    o = oracle_built("port").load(scene)
    o.set_state(start)
    w = world(ext_built, scene, "fp32")
    errs = []
    for k in range(12):
        st = o.get_state()
        w.set_state(st)
        w.step(1)
        o.step(1)
        a, b = o.get_state(), w.get_state()
        errs.append(max(float(np.max(np.abs(a[:, 0:3] - b[:, 0:3]))), float(np.max(np.abs(a[:, 3:7] - b[:, 3:7])))))
    bound = max(1e-4, sens)
    assert np.median(errs) <= bound, "%s: median frame error %.3g > %.3g (sensitivity %.3g)" % (name, np.median(errs), bound, sens)
    assert max(errs) <= 5e-2, (name, errs)
    w.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", SMALL + ["large1024"])
def test_pairs_bitexact(ext_built, oracle_built, name, precision):
    """broad_get_collision_pairs: same pairs, same order, on identical inputs (both builds)."""
    scene = SCENES[name][0]()
    o = oracle_built("port").load(scene)
    w = world(ext_built, scene, precision)
    states = [o.get_state()]
    g = golden(name)
    if "kat_state" in g and scene_fingerprint_ok(scene, g):
        states.append(g["kat_state"])
    for st in states:
        o.set_state(st)
        w.set_state(st)
        assert np.array_equal(w.broad_pairs(), o.broad_pairs())
    w.close()


def _match_sets(a, b, tol, touch=1e-6, anchors=False):
    """True when contact lists a and b hold the same contacts up to order (within tol). A contact
    whose two points are within `touch` of each other (penetration at rounding level: the
    reference keeps it when its FP64 penetration is below zero) may be present on one side only.
    anchors=True: rows are constraint anchors r1_lc, r2_lc (body frames), compared as such and
    never treated as touching."""
    def touching(r):
        return (not anchors) and np.max(np.abs(r[0:3] - r[3:6])) <= touch
    used = np.zeros(len(b), dtype=bool)
    for row in a:
        d = np.max(np.abs(b - row), axis=1) if len(b) else np.zeros(0)
        d[used] = np.inf
        j = int(np.argmin(d)) if len(d) else -1
        if j >= 0 and d[j] <= tol:
            used[j] = True
        elif not touching(row):
            return False
    return all(touching(r) for r in b[~used])


@pytest.mark.parametrize("name", [n for n in SMALL])
def test_contacts_known_answers(ext_built, oracle_built, name):
    """colliders_get_contacts on every pair of a penetrating state: exact in FP64; the same
    contacts (order may differ where parallel faces tie) within 2e-5 in FP32."""
    g = golden(name)
    scene = SCENES[name][0]()
    if not scene_fingerprint_ok(scene, g):
        pytest.skip("scene generator differs from the fixture's")
    for precision in ("fp64", "fp32"):
        w = world(ext_built, scene, precision)
        w.set_state(g["kat_state"])
        k = 0
        for (a, b), cnt in zip(g["kat_pairs"], g["kat_counts"]):
            c = w.contacts(int(a), int(b))
            expect = g["kat_contacts"][k:k + cnt]
            k += cnt
            if precision == "fp64":
                assert np.array_equal(c, expect), (name, a, b)
            else:
                assert _match_sets(c, expect, 2e-5), (name, a, b, c, expect)
        w.close()


def test_large_scene_one_frame(ext_built, oracle_built):
    name = "large1024"
    scene = SCENES[name][0]()
    o = oracle_built("port").load(scene)
    o.step(1)
    ref = o.get_state()
    w = world(ext_built, scene, "fp64")
    w.step(1)
    assert np.array_equal(w.get_state()[:, 0:7], ref[:, 0:7])
    w.close()
    w = world(ext_built, scene, "fp32")
    w.step(1)
    got = w.get_state()
    err = np.max(np.abs(got[:, 0:3] - ref[:, 0:3]), axis=1)
    assert np.median(err) <= 1e-5 and np.max(err) <= 1e-4, np.sort(err)[-5:]
    w.close()


def test_large_4096_pairs_and_frame(ext_built, oracle_built):
    """The bench workload (4096 bodies): pair list bit-exact, first frame within tolerance."""
    from rawphys import scenes as S
    scene = S.large_scene(4096, seed=0)
    o = oracle_built("port").load(scene)
    w = world(ext_built, scene, "fp32")
    assert np.array_equal(w.broad_pairs(), o.broad_pairs())
    o.step(1)
    w.step(1)
    err = np.max(np.abs(w.get_state()[:, 0:3] - o.get_state()[:, 0:3]), axis=1)
    assert np.max(err) <= 1e-4, np.sort(err)[-5:]
    w.close()
