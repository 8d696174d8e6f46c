"""Precision stress (towers of 64 unit cubes, masses alternating 1:100, 50 substeps): the all-FP64 GPU
build follows the oracle bit for bit; the FP32 build's per-step error from identical states stays
within 1e-4 m / rad or within the reference's own spread under FP32-scale input noise; the report of
rawphys.precision (used by bench.py) is complete and finite."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tower_fp64_bitexact_and_fp32_step_error(ext_built, oracle_built):
    from rawphys import scenes as S
    from test_gpu_parity import perturb, pose_dev
    batch = S.tower_batch(2, n=64, seed=3)
    w64 = ext_built.World(0, "fp64")
    w64.load_batch(batch)
    w32 = ext_built.World(0, "fp32")
    w32.load_batch(batch)
    rng = np.random.default_rng(4)
    # FP64 trajectories of both towers against the oracle, 30 frames
    w64.step(30)
    got = w64.get_state()
    errs, spreads = [], []
    for s in range(batch.num_scenes):
        idx = np.nonzero(batch.scene == s)[0]
        sc = S.batch_scene(batch, s)
        o = oracle_built("port").load(sc)
        o.step(30)
        assert np.array_equal(got[idx], o.get_state()), "tower %d" % s
        # FP32 frames from identical states, against the reference and its FP32-noise spread
        noisy = oracle_built("port").load(sc)
        for k in range(4):
            st = o.get_state()
            full = w32.get_state()
            full[idx] = st
            w32.set_state(full)
            w32.step(1)
            o.step(1)
            ref = o.get_state()
            errs.append(pose_dev(w32.get_state()[idx], ref))
            spread = 0.0
            for _ in range(3):
                noisy.set_state(perturb(st, rng))
                noisy.step(1)
                spread = max(spread, pose_dev(noisy.get_state(), ref))
            spreads.append(spread)
    assert np.median(errs) <= max(1e-4, float(np.median(spreads))), (errs, spreads)
    w64.close()
    w32.close()


def test_precision_report(ext_built):
    from rawphys import scenes as S
    from rawphys.precision import precision_report
    rep = precision_report(ext_built, S.tower_batch(8, n=16, seed=1), frames=40, sample_every=10)
    assert rep["samples"] == 4 and rep["scenes"] == 8
    for k in ("step_pos_err_fp32_vs_fp64", "step_rot_err_fp32_vs_fp64", "trajectory_divergence_m"):
        assert np.isfinite(rep[k]["max"])
    assert all(np.isfinite(v) for v in rep["relative_energy_drift"].values())
