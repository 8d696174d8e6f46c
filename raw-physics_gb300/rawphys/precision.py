"""Precision report of the FP32 build (FP32 arithmetic, FP64 pose accumulation) against the all-FP64
build on the same GPU: per-step position / orientation error from identical states, short-horizon
trajectory divergence, tower drift and energy drift, on any scene batch (normally
scenes.tower_batch: towers of unit cubes with alternating mass ratio 1:100, 50 substeps)."""
from __future__ import annotations

import numpy as np


def _rot(q):
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], -2)


def energies(batch, state, inertia_local, gravity):
    """Kinetic + potential energy per scene: sum of m v^2 / 2 + w^T I_w w / 2 + m g y."""
    dyn = ~batch.fixed
    m = batch.mass
    v, w, y = state[:, 7:10], state[:, 10:13], state[:, 1]
    Rm = _rot(state[:, 3:7])
    Iw = Rm @ inertia_local @ np.transpose(Rm, (0, 2, 1))
    e = 0.5 * m * np.sum(v * v, 1) + 0.5 * np.einsum("bi,bij,bj->b", w, Iw, w) + m * gravity * y
    return np.bincount(batch.scene[dyn], weights=e[dyn], minlength=batch.num_scenes)


def pose_error(a, b):
    return float(np.max(np.abs(a[:, 0:3] - b[:, 0:3]))), float(np.max(np.abs(a[:, 3:7] - b[:, 3:7])))


def precision_report(rawphys, batch, frames: int = 300, sample_every: int = 50, device: int = 0):
    """Runs the batch in FP64 and FP32 side by side. Returns the per-step errors of FP32 frames taken
    from the FP64 trajectory's states, the FP32-FP64 trajectory divergence at the end, the top
    bodies' horizontal drift, and the energy drift of each precision."""
    worlds = {}
    for prec in ("fp64", "fp32"):
        w = rawphys.World(device, prec)
        first = w.load_batch(batch)
        assert first == 0
        worlds[prec] = w
    w64, w32 = worlds["fp64"], worlds["fp32"]
    inertia = np.stack([w64.mass_properties(e)[1] for e in range(batch.num_bodies)])
    g = batch.gravity
    s0 = w64.get_state()
    e0 = {p: energies(batch, s0, inertia, g) for p in worlds}
    top = np.array([np.max(np.nonzero(batch.scene == s)[0]) for s in range(batch.num_scenes)])
    rng = np.random.default_rng(0)
    step_pos, step_rot, spread, at, done = [], [], [], [], 0
    while done < frames:
        if done % sample_every == 0:
            at.append(done)
            st = w64.get_state()
            # the FP64 build's own response to FP32-scale noise (1e-7 m, 1e-7 relative) on this
            # frame's input: the floor below which no FP32 implementation can agree
            sp = 0.0
            w64.step(1)
            ref = w64.get_state()
            for _ in range(2):
                p = st.copy()
                p[:, 0:3] += 1e-7 * rng.standard_normal(p[:, 0:3].shape)
                p[:, 3:7] *= 1.0 + 1e-7 * rng.standard_normal(p[:, 3:7].shape)
                w64.set_state(p)
                w64.step(1)
                sp = max(sp, max(pose_error(w64.get_state(), ref)))
            spread.append(sp)
            # one FP32 frame from the FP64 trajectory's state, against the FP64 frame
            w32.set_state(st)
            w32.step(1)
            w64.set_state(ref)
            pe, re = pose_error(w32.get_state(), ref)
            step_pos.append(pe)
            step_rot.append(re)
            done += 1
        else:
            k = min(sample_every - done % sample_every, frames - done)
            w64.step(k)
            done += k
    end64 = w64.get_state()
    # the FP32 trajectory over the same horizon, from the same initial state
    w32.set_state(s0)
    w32.step(frames)
    end32 = w32.get_state()
    dyn = ~batch.fixed
    div = np.abs(end32[dyn, 0:3] - end64[dyn, 0:3])
    e_end = {"fp64": energies(batch, end64, inertia, g), "fp32": energies(batch, end32, inertia, g)}
    drift = {p: float(np.median(np.abs(e_end[p] - e0[p]) / np.maximum(np.abs(e0[p]), 1e-12))) for p in worlds}
    tower_drift = {p: float(np.median(np.linalg.norm((end64 if p == "fp64" else end32)[top][:, [0, 2]] - s0[top][:, [0, 2]],
                                                     axis=1))) for p in worlds}
    for w in worlds.values():
        w.close()
    return {"frames": frames, "scenes": batch.num_scenes, "bodies": int(dyn.sum()), "substeps": batch.substeps,
            "step_pos_err_fp32_vs_fp64": {"median": float(np.median(step_pos)), "max": float(np.max(step_pos))},
            "step_rot_err_fp32_vs_fp64": {"median": float(np.median(step_rot)), "max": float(np.max(step_rot))},
            "step_err_by_frame": [[f, p, r, n] for f, p, r, n in zip(at, step_pos, step_rot, spread)],
            "step_err_by_frame_columns": ["frame", "pos err m", "rot err", "FP64 spread under 1e-7 input noise"],
            "trajectory_divergence_m": {"median": float(np.median(div)), "max": float(np.max(div))},
            "top_body_horizontal_drift_m": tower_drift,
            "relative_energy_drift": drift,
            "samples": len(step_pos)}


def rotation_angle(qa, qb):
    """Angle (rad) of the rotation between unit quaternions, per row: 4 asin(|qa - s qb| / 2) with s
    the sign of their dot product (accurate for small angles, unlike 2 acos(|qa . qb|))."""
    s = np.where(np.sum(qa * qb, axis=1) < 0.0, -1.0, 1.0)[:, None]
    return 4.0 * np.arcsin(np.minimum(1.0, 0.5 * np.linalg.norm(qa - s * qb, axis=1)))


def step_error(got, expected, dynamic):
    """Per-step error of one frame from identical states: position error |x - x_ref| (m) and rotation
    angle between orientations (rad) over the dynamic bodies, as median, 99th percentile and max."""
    pe = np.linalg.norm(got[dynamic, 0:3] - expected[dynamic, 0:3], axis=1)
    re = rotation_angle(got[dynamic, 3:7], expected[dynamic, 3:7])

    def summary(x):
        if x.size == 0:
            return {"median": 0.0, "p99": 0.0, "max": 0.0}
        return {"median": float(np.median(x)), "p99": float(np.quantile(x, 0.99)), "max": float(np.max(x))}
    return {"pos_m": summary(pe), "rot_rad": summary(re), "bodies": int(pe.size),
            "within_1e-4": float(np.mean((pe <= 1e-4) & (re <= 1e-4))) if pe.size else 1.0}
