"""Benchmark of the GB300 rigid-body step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload batched|large4096|stack10]

Headline workload (default, "batched"): 16384 independent scenes in one world, dynamic bodies per scene
log-uniform in [2, 512] (about 1.65 M in all), shapes drawn from cube / icosahedron / 32-segment cylinder
/ 42-vertex icosphere with scale U(0.5, 1.5), a quarter of the scenes with 8-64-link hinge or spherical
chains; dt = 1/60, 20 substeps, 1 position iteration, FP32 arithmetic with FP64 poses; every frame is
one replay of the captured phase-major CUDA graph. Seeded synthetic data. The batch is first advanced
`--batched-settle` frames (untimed), then W warm-up frames, then K timed frames. A "step" is one
pbd_simulate frame of every scene.

Printed JSON line (rank 0):
  value     body-substeps/s = dynamic bodies x substeps x K / summed device time of the K frames
            (CUDA events on the world's stream; L2 flushed with a 256 MiB write before every frame)
  e2e       the same metric through the C ABI with host buffers: every frame uploads the whole batch's
            state from pinned host memory (rp_state_set), steps, and downloads it (rp_state_get); the
            copies are inside the timer, the same L2 flush before every frame
  step_err  per-step error of the first timed frame against the oracle (the FP64 restatement of the
            reference, bit-exact to it) run from the same state, on a size-stratified sample of scenes:
            position (m) and rotation angle (rad), median / p99 / max over the sampled dynamic bodies
  roofline  the dominant kernel of the frame (from CUDA events around each phase) against the
            measured HBM copy bandwidth: its algorithmic bytes per launch over its average duration
  fp32_pipe FP32-pipe utilisation of GJK and EPA: algorithmic flops (device-counted support calls,
            iterations and faces times the per-operation flop model) over time x nominal FP32 peak
  cpu_baseline  the oracle port on one host core, on a bounded sample of the same workload
  plain     the plain single-scene form beside it (4096 bodies, FP32 and the all-FP64 build), with its
            own per-step error; vs_plain_gpu = batched / plain FP32
  precision the precision-stress report: 128 towers of 64 cubes (masses 1:100, 50 substeps) run in the
            FP32 and the all-FP64 builds side by side
  adjoint   grad/s of the adjoint (scene-gradients per second) on a bounded sample of the
            differentiation workload
--workload large4096 / stack10 measure the plain form of that scene as the line's value.
--impl reference times the reference's CPU algorithm (the oracle port, a bit-exact plain-C restatement
of the reference) on every host core, on the same workload: a size-stratified sample of the batch's
scenes, one process per core (the reference is single-threaded and keeps process-global state).
Multi-GPU (torchrun): the batch shards by scene, every rank steps its own batch (weak scaling); the
single scene does not shard ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "raw-physics_gb300"))
sys.path.insert(0, ROOT)

METRIC = "body-substeps/s batched vs plain GPU at ≤1e-4 m pos err vs FP64 CPU; grad/s"
UNIT = "body-substeps/s"
# Algorithmic bytes of one position sweep: every contact record read (48 B) and its two lambdas
# written back (8 B); per solved pair node, both bodies' pose read and written (2 x 64 B) and their
# inverse mass and inertia read (2 x 28 B).
SWEEP_CONTACT_B, SWEEP_NODE_B = 56, 2 * (64 + 64 + 28)
# Algorithmic FP32 flops of the narrowphase (per device-counted operation): a support call is one dot
# product and a compare per hull vertex (6 V); a GJK iteration's simplex update ~60; an EPA iteration
# ~40 per new face plus 6 per face scanned.
FLOP_SUPPORT_PER_VERT, FLOP_GJK_ITER, FLOP_EPA_ITER = 6, 60, 40 * 6 + 6 * 24
NOMINAL_FP32_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12   # 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz
BATCHED_WORKLOAD = ("batched16384: 16384 independent scenes, dynamic bodies per scene log-uniform in [2,512], "
                    "cube/icosahedron/cylinder32/icosphere42 hulls at scale U(0.5,1.5), 25% of scenes with "
                    "8-64-link hinge or spherical chains, dt=1/60, 20 substeps, 1 position iteration")
PLAIN_WORKLOAD = ("large4096: one scene of 4096 dynamic bodies (cube/icosahedron/cylinder32/icosphere42, scale "
                  "U(0.5,1.5)) in a 40x40x60 m box, dt=1/60, 20 substeps, 1 position iteration")


def make_scene(name):
    from rawphys import scenes as S
    if name == "stack10":
        return S.stack_scene(10, seed=0)
    return S.large_scene(4096, seed=0)


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clock / throttle samples every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r.split(", ") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(summary, kernel):
    """DRAM bytes per launch of `kernel` from a committed ncu summary (a line
    `traffic_bytes_per_launch[<kernel>]: <bytes>`), or None with the reason."""
    rel = "profiles/" + summary
    key = "traffic_bytes_per_launch[%s]:" % kernel
    try:
        for line in open(os.path.join(ROOT, rel)):
            if line.startswith(key):
                return float(line.split(":", 1)[1]), rel
    except OSError:
        return None, "missing " + rel
    return None, "no %s line in %s" % (key, rel)


# ---------------------------------------------------------------------------------------------
# Sampling of the batch for the CPU legs and the per-step error
def stratified_scenes(batch, count):
    """`count` scenes spread evenly over the batch's scenes sorted by body count (the sample has the
    batch's size distribution, so its body-substeps/s stands for the whole batch's)."""
    sizes = np.bincount(batch.scene, minlength=batch.num_scenes)
    order = np.argsort(sizes, kind="stable")
    pick = order[np.linspace(0, batch.num_scenes - 1, min(count, batch.num_scenes)).round().astype(int)]
    return sorted(set(int(s) for s in pick))


def oracle_frames(scene, state, frames, noise_seed=None):
    """The oracle port: `frames` frames of `scene` from `state`; returns (end state, seconds, error bits,
    spread). With noise_seed, also the same frames from the state with FP32-scale noise (1e-7 m on
    positions, 1e-7 relative on orientations): spread is each body's position change under it, the
    reference's own sensitivity on this frame."""
    from oracle.oracle import Oracle
    o = Oracle("port").load(scene)
    o.set_state(state)
    t = time.perf_counter()
    o.step(frames)
    secs = time.perf_counter() - t
    end, bits = o.get_state(), o.error_bits()
    spread = None
    if noise_seed is not None:
        rng = np.random.default_rng(noise_seed)
        p = state.copy()
        p[:, 0:3] += 1e-7 * rng.standard_normal(p[:, 0:3].shape)
        p[:, 3:7] *= 1.0 + 1e-7 * rng.standard_normal(p[:, 3:7].shape)
        o.set_state(p)
        o.step(frames)
        spread = np.linalg.norm(o.get_state()[:, 0:3] - end[:, 0:3], axis=1)
    return end, secs, bits, spread


def with_spread(err, got, exp, dyn, spread):
    """Adds to a step_error summary the reference's own position change under FP32-scale input noise
    (median / p99 / max over the same bodies) and the fraction of bodies within 1e-4 m or within
    three times that change (where the reference is ill-conditioned, no FP32 result can agree closer)."""
    pe = np.linalg.norm(got[dyn, 0:3] - exp[dyn, 0:3], axis=1)
    sp = spread[dyn]
    err["reference_spread_m"] = {"median": float(np.median(sp)), "p99": float(np.quantile(sp, 0.99)),
                                 "max": float(np.max(sp))} if sp.size else None
    err["within_1e-4_or_3x_spread"] = float(np.mean((pe <= 1e-4) | (pe <= 3.0 * sp))) if sp.size else 1.0
    return err


# ---------------------------------------------------------------------------------------------
# Reference arm: the reference's CPU algorithm on every host core
_WORKER = {}


def _ref_pin(barrier):
    """Pool initializer: every task below waits at this barrier once, so each of the pool's
    processes takes exactly one task per map and keeps its own slice of the sample."""
    _WORKER["barrier"] = barrier


def _ref_load(job):
    """Pool worker: keep its scenes of the batch sample and settle them on the CPU."""
    sys.path.insert(0, os.path.join(ROOT, "raw-physics_gb300"))
    sys.path.insert(0, ROOT)
    from oracle.oracle import Oracle, build
    build(ref=False)
    scenes, settle = job
    _WORKER["scenes"] = scenes
    _WORKER["states"] = []
    for _, sc in scenes:
        o = Oracle("port").load(sc)
        o.step(settle)
        _WORKER["states"].append(o.get_state())
    _WORKER["barrier"].wait()
    return [s for s, _ in scenes]


def _ref_frame(_):
    """Pool worker: one frame of each of its own scenes from their settled states; returns
    (body-substeps, seconds, its scene ids)."""
    from oracle.oracle import Oracle
    work, secs = 0, 0.0
    for (_, sc), st in zip(_WORKER["scenes"], _WORKER["states"]):
        o = Oracle("port").load(sc)
        o.set_state(st)
        t = time.perf_counter()
        o.step(1)
        secs += time.perf_counter() - t
        work += sc.num_dynamic * sc.substeps
    _WORKER["barrier"].wait()
    return work, secs, [s for s, _ in _WORKER["scenes"]]


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle.oracle import build
    from rawphys import scenes as S
    build(ref=False)
    cores = os.cpu_count() or 1
    if args.workload != "batched":
        return run_reference_plain(args, cores)
    batch = S.batched_scenes(args.batched_scenes, seed=0)
    picks = stratified_scenes(batch, args.ref_scenes)
    sizes = np.bincount(batch.scene[~batch.fixed], minlength=batch.num_scenes)
    # every core owns a fixed slice of the sample (balanced by bodies), settles it, then times frames
    order = sorted(picks, key=lambda s: -int(sizes[s]))
    slices = [[] for _ in range(cores)]
    load = [0] * cores
    for s in order:
        k = int(np.argmin(load))
        slices[k].append(s)
        load[k] += int(sizes[s])
    slices = [sl for sl in slices if sl]
    ctx = mp.get_context("spawn")
    jobs = [([(x, S.batch_scene(batch, x)) for x in sl], args.batched_settle) for sl in slices]
    n = len(jobs)
    barrier = ctx.Barrier(n)
    with ctx.Pool(n, initializer=_ref_pin, initargs=(barrier,)) as pool:
        owned = pool.map(_ref_load, jobs, chunksize=1)
        assert sorted(x for o in owned for x in o) == sorted(picks)
        for _ in range(args.warmup):
            pool.map(_ref_frame, range(n), chunksize=1)
        total, wall = 0, 0.0
        for _ in range(args.steps):
            res = pool.map(_ref_frame, range(n), chunksize=1)
            assert sorted(x for _, _, o in res for x in o) == sorted(picks), "a process ran another's slice"
            total += sum(b for b, _, _ in res)
            # a step lasts as long as its slowest process spent inside the step calls (re-loading a
            # scene into the single-scene harness between frames is not part of the reference's step)
            wall += max(t for _, t, _ in res)
    value = total / wall
    nd_sample = int(sum(sizes[s] for s in picks))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene generator)",
            "config": {"workload": BATCHED_WORKLOAD},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": n, "kind": "port",
                             "sample": "%d of the %d scenes, evenly spaced in body-count order (%d of %d dynamic "
                                       "bodies), each settled %d frames on the CPU, then one frame of all of them per "
                                       "step over %d processes (a step lasts as long as the slowest process's step "
                                       "calls); oracle port, a bit-exact plain-C restatement of the reference "
                                       "(-O2 -ffp-contract=off); the whole batch takes sum(N*S) / value per frame"
                                       % (len(picks), batch.num_scenes, nd_sample, batch.num_dynamic,
                                          args.batched_settle, n)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _plain_init(name, state):
    sys.path.insert(0, os.path.join(ROOT, "raw-physics_gb300"))
    sys.path.insert(0, ROOT)
    from oracle.oracle import Oracle
    scene = make_scene(name)
    _WORKER["scene"] = scene
    _WORKER["oracle"] = Oracle("port").load(scene)
    _WORKER["state"] = state


def _plain_frame(frames):
    o, scene = _WORKER["oracle"], _WORKER["scene"]
    o.set_state(_WORKER["state"])
    t = time.perf_counter()
    o.step(frames)
    return scene.num_dynamic * scene.substeps * frames, time.perf_counter() - t


def run_reference_plain(args, cores):
    import multiprocessing as mp
    from oracle.oracle import Oracle
    scene = make_scene(args.workload)
    o = Oracle("port").load(scene)
    o.step(args.settle)
    state = o.get_state()
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_plain_init, initargs=(args.workload, state)) as pool:
        for _ in range(args.warmup):
            pool.map(_plain_frame, [1] * cores)
        t = time.perf_counter()
        total = 0
        for _ in range(args.steps):
            total += sum(b for b, _ in pool.map(_plain_frame, [1] * cores))
        wall = time.perf_counter() - t
    value = total / wall
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene generator)",
            "config": {"workload": PLAIN_WORKLOAD if args.workload == "large4096" else args.workload},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d replicas x 1 frame per step, frame %d after a %d-frame settle, oracle port"
                                       % (cores, args.settle + 1, args.settle)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# GPU arm
def timed_frames(w, stream, flush, frames, clocks_gpu=None):
    """Device time (ms) of each of `frames` frames, L2 flushed before each; optional clock samples."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(frames)]
    clk = ClockSampler(clocks_gpu) if clocks_gpu is not None else None
    torch.cuda.synchronize()
    if clk:
        clk.__enter__()
    for k in range(frames):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xff)              # evict L2 (129 MB) before each timed frame
        ev[k][0].record(stream)
        w.step(1)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    if clk:
        clk.__exit__()
    return [a.elapsed_time(b) for a, b in ev], (clk.summary() if clk else None)


def phase_pass(w, start_state, frames):
    """Per-phase ms per frame of `frames` frames from start_state (events after every phase)."""
    w.set_state(start_state)
    w.sync()
    p0 = w.phase_times()
    w.set_timing(True)
    w.step(frames)
    w.sync()
    w.set_timing(False)
    p1 = w.phase_times()
    return {k: round((p1[k] - p0[k]) / frames, 4) for k in p0}


def e2e_frames(w, stream, flush, start_state, frames):
    """End to end through the C ABI with host buffers: per frame the whole state from pinned host
    memory (rp_state_set), one step, the whole state back (rp_state_get); copies inside the timer."""
    import torch
    st = start_state
    w.set_state(st)
    w.step(1)
    w.get_state()
    b0 = w.transfer_bytes()
    torch.cuda.synchronize()
    wall = 0.0
    buf = np.array(st, dtype=np.float64, order="C")    # the caller's state array, reused every frame
    for k in range(frames):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        t = time.perf_counter()
        w.set_state(buf)
        w.step(1)
        w.get_state(out=buf)
        wall += time.perf_counter() - t
    b1 = w.transfer_bytes()
    return wall, (b1[0] - b0[0]) // frames, (b1[1] - b0[1]) // frames


def narrow_flops(c0, c1, frames, verts_avg):
    """Algorithmic FP32 flops per frame of GJK and of EPA from the device counters."""
    gjk_iters = (c1[0] - c0[0]) / frames
    epa_iters = (c1[1] - c0[1]) / frames
    # every GJK iteration and every EPA iteration makes one Minkowski support call (two hull scans)
    gjk = gjk_iters * (FLOP_GJK_ITER + 2 * FLOP_SUPPORT_PER_VERT * verts_avg)
    epa = epa_iters * (FLOP_EPA_ITER + 2 * FLOP_SUPPORT_PER_VERT * verts_avg)
    return gjk, epa


def fp32_pipe(c0, c1, frames, phase, verts_avg):
    gjk, epa = narrow_flops(c0, c1, frames, verts_avg)
    out = {"peak_tflops": NOMINAL_FP32_TFLOPS, "peak_kind": "nominal (152 SMs x 128 FP32 lanes x 2 x 2.07 GHz)",
           "model": "support call 6 flop per hull vertex per hull, GJK 60 flop per iteration, EPA ~400 flop per "
                    "iteration; counts from the device counters"}
    for name, flops, key in (("k_gjk", gjk, "gjk"), ("k_epa", epa, "epa")):
        ms = phase.get(key, 0.0)
        ach = flops / (ms / 1e3) / 1e12 if ms > 0 else 0.0
        out[name] = {"gflop_per_frame": flops / 1e9, "ms_per_frame": ms, "achieved_tflops": ach,
                     "frac": ach / NOMINAL_FP32_TFLOPS}
    return out


def roofline_of(phase, c0, c1, frames, substeps, pos_iters, kernels, summary):
    """Roofline object of the dominant kernel. The position sweep (one launch per substep and
    iteration) has the HBM byte model above; other phases are reported with their share only."""
    peak, peak_kind = measured_peak_hbm()
    sweeps = substeps * pos_iters
    alg_bytes = ((c1[5] - c0[5]) / frames * SWEEP_CONTACT_B + (c1[2] - c0[2]) / frames * SWEEP_NODE_B) / substeps
    launch_ms = phase["solve"] / sweeps if sweeps else 0.0
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9 if launch_ms > 0 else 0.0
    traffic, src = profile_traffic(summary, kernels["solve"])
    frame_ms = sum(phase.values())
    shares = {k: (v / frame_ms if frame_ms else 0.0) for k, v in phase.items()}
    dom = max(phase, key=lambda k: phase[k])
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak if peak else 0.0,
            "peak_kind": peak_kind, "traffic": traffic, "traffic_source": src, "kernel": kernels["solve"],
            "alg_bytes_per_launch": alg_bytes, "launch_ms": launch_ms,
            "kernel_share_of_frame": shares.get("solve", 0.0), "dominant_phase": dom,
            "phase_share": {k: round(v, 4) for k, v in shares.items()}}


def measure_batched(args, dev, rank, world_size, with_oracle):
    """The headline: the batched form (rawphys.scenes.batched_scenes), every frame one replay of the
    captured phase-major graph. Weak scaling: every rank steps its own batch (seed = rank)."""
    import torch
    import rawphys
    from rawphys import scenes as S
    from rawphys.precision import step_error
    batch = S.batched_scenes(args.batched_scenes, seed=rank)
    stream = torch.cuda.Stream(dev)
    w = rawphys.World(dev, "fp32")
    w.set_stream(stream.cuda_stream)
    w.set_sweep_order(args.sweep_order)
    w.load_batch(batch)
    w.step(args.batched_settle)
    tuned = w.autotune(frames=2) if args.autotune else None
    w.step(args.warmup)
    w.sync()
    nd = batch.num_dynamic
    start_state = w.get_state()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    w.degenerate_info()                       # clear: count what the timed frames meet
    c0 = w.counters()
    l0 = w.kernel_launches()
    if world_size > 1:
        torch.distributed.barrier()
    ms, clocks = timed_frames(w, stream, flush, args.steps, clocks_gpu=dev)
    if world_size > 1:
        torch.distributed.barrier()
    total_ms = float(sum(ms))
    c1 = w.counters()
    launches = w.kernel_launches() - l0
    status = w.status()
    degenerate = w.degenerate_info()
    if world_size > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = nd * batch.substeps * args.steps * world_size / (total_ms / 1e3)
    phase = phase_pass(w, start_state, 2)
    # the first timed frame again, from its start state: the GPU's answer for the per-step error
    w.set_state(start_state)
    w.step(1)
    first = w.get_state()
    e2e_wall, h2d, d2h = e2e_frames(w, stream, flush, start_state, args.e2e_frames)
    e2e = {"value": nd * batch.substeps * args.e2e_frames * world_size / e2e_wall, "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    w.close()
    verts = np.array([m.positions.shape[0] for m in batch.meshes], dtype=np.float64)
    verts_avg = float(np.mean(verts[batch.mesh]))
    out = {"value": value, "total_ms": total_ms, "ms": ms, "clocks": clocks, "launches": launches, "status": status,
           "degenerate_first": degenerate, "phase": phase, "e2e": e2e, "tuned": tuned, "nd": nd,
           "roofline": roofline_of(phase, c0, c1, args.steps, batch.substeps, batch.pos_iters,
                                   {"solve": "k_sweep_warp (position sweep, one warp per scene)"}, "pipeline_batched16384.md"),
           "fp32_pipe": fp32_pipe(c0, c1, args.steps, phase, verts_avg),
           "pairs_per_step": (c1[6] - c0[6]) / args.steps, "contacts_per_step": (c1[5] - c0[5]) / args.steps}
    if with_oracle:
        # the oracle on a size-stratified sample of scenes, one frame from the same start state:
        # the per-step error of the GPU's frame, and the 1-core CPU baseline of the same work
        picks = stratified_scenes(batch, args.err_scenes)
        got, exp, dyn, spr = [], [], [], []
        cpu_work, cpu_secs, bits = 0, 0.0, 0
        for s in picks:
            idx = np.nonzero(batch.scene == s)[0]
            sc = S.batch_scene(batch, s)
            end, secs, eb, sp = oracle_frames(sc, start_state[idx], 1, noise_seed=s)
            got.append(first[idx])
            exp.append(end)
            dyn.append(~batch.fixed[idx])
            spr.append(sp)
            cpu_work += sc.num_dynamic * sc.substeps
            cpu_secs += secs
            bits |= eb
        G, E, D = np.concatenate(got), np.concatenate(exp), np.concatenate(dyn)
        out["step_err"] = with_spread(step_error(G, E, D), G, E, D, np.concatenate(spr))
        out["step_err"]["scenes"] = len(picks)
        out["step_err"]["oracle_assert_bits"] = bits
        out["cpu_baseline"] = {"value": cpu_work / cpu_secs, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": "%d of the %d scenes, stratified by body count, one frame each from the state "
                                         "the timed GPU frames start from; oracle port (bit-exact plain-C restatement "
                                         "of the reference), %.1f s" % (len(picks), batch.num_scenes, cpu_secs)}
    sizes = batch.scene_sizes()
    out["workload_detail"] = ("%d scenes, dynamic bodies per scene mean %.1f max %d (%d in all), %d scenes with chains "
                              "(%d joints); frames %d-%d after a %d-frame settle and %d warm-up frames"
                              % (batch.num_scenes, sizes.mean(), sizes.max(), nd,
                                 len({int(batch.scene[c.e1]) for c in batch.constraints}), len(batch.constraints),
                                 args.batched_settle + args.warmup, args.batched_settle + args.warmup + args.steps,
                                 args.batched_settle, args.warmup))
    return out


def measure_plain(args, dev, precision, steps, start_from=None, with_oracle=False):
    """The plain form: one large scene (the cooperative grid path). Returns its device-timed rate, phase
    split, roofline, e2e and (with_oracle) the per-step error of its first timed frame."""
    import torch
    import rawphys
    from rawphys.precision import step_error
    scene = make_scene(args.workload if args.workload != "batched" else "large4096")
    stream = torch.cuda.Stream(dev)
    w = rawphys.World(dev, precision)
    w.set_stream(stream.cuda_stream)
    if precision == "fp32":
        w.set_sweep_order(args.sweep_order)
    w.load(scene)
    if start_from is not None:
        w.set_state(start_from)
    elif args.settle:
        w.step(args.settle)
    tuned = w.autotune(frames=3) if args.autotune else None
    w.step(args.warmup)
    w.sync()
    start_state = w.get_state()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    c0 = w.counters()
    l0 = w.kernel_launches()
    ms, clocks = timed_frames(w, stream, flush, steps, clocks_gpu=dev)
    launches = w.kernel_launches() - l0
    c1 = w.counters()
    total_ms = float(sum(ms))
    value = scene.num_dynamic * scene.substeps * steps / (total_ms / 1e3)
    phase = phase_pass(w, start_state, min(steps, 5))
    w.set_state(start_state)
    w.step(1)
    first = w.get_state()
    e2e_wall, h2d, d2h = e2e_frames(w, stream, flush, start_state, max(3, steps // 2))
    status = w.status()
    w.close()
    dropin = dropin_e2e(args, scene, start_state, flush, max(3, steps // 2)) if precision == "fp32" else None
    out = {"value": value, "unit": UNIT, "precision": precision, "e2e_dropin": dropin, "ms_per_step": total_ms / steps, "steps": steps,
           "clocks": clocks, "gpu_launches": launches, "device_status": status, "phase_ms_per_step": phase,
           "autotuned": tuned, "start_state": start_state,
           "e2e": {"value": scene.num_dynamic * scene.substeps * max(3, steps // 2) / e2e_wall, "unit": UNIT,
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "roofline": roofline_of(phase, c0, c1, steps, scene.substeps, scene.pos_iters,
                                   {"solve": "k_sweep_grid (position sweep, cooperative grid)"}, "pipeline_large4096.md"),
           "pairs_per_step": (c1[6] - c0[6]) / steps, "contacts_per_step": (c1[5] - c0[5]) / steps,
           "levels_per_step": (c1[7] - c0[7]) / steps}
    if with_oracle:
        end, secs, bits, sp = oracle_frames(scene, start_state, 1, noise_seed=0)
        out["step_err"] = with_spread(step_error(first, end, ~scene.fixed), first, end, ~scene.fixed, sp)
        out["step_err"]["oracle_assert_bits"] = bits
        out["cpu_baseline"] = {"value": scene.num_dynamic * scene.substeps / secs, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": "1 frame of the scene from the state the timed GPU frames start from, oracle "
                                         "port, %.1f s" % secs}
    return out


def dropin_e2e(args, scene, start_state, flush, frames):
    """The same metric through the reference's own entry point: the C++-mangled pbd_simulate over
    Entity** (rawphys.compat builds the caller's structs), as a reference caller runs a frame: add
    gravity with entity_add_force semantics, call pbd_simulate (FP32 default), clear the forces. Each
    call writes every entity's state and transformed hulls back into the caller's structs; the L2 is
    flushed before every call; only the call is timed."""
    import ctypes as C
    import torch
    import rawphys
    from rawphys import compat
    lib = C.CDLL(rawphys.LIB_PATH)
    lib.rp_compat_reset()
    lib.rp_compat_world.restype = C.c_void_p
    sim, _ = compat.dropin(lib)
    callers = compat.build_callers(scene)
    callers.set_state(start_state)
    for _ in range(2):
        callers.add_gravity(scene.gravity)
        sim(scene.dt, callers.array, scene.substeps, scene.pos_iters, int(scene.collisions))
        callers.clear_forces()
    tb0 = (C.c_uint64 * 2)()
    rawphys.load_library().rp_transfer_bytes(C.c_void_p(lib.rp_compat_world()), tb0)
    wall = 0.0
    for k in range(frames):
        callers.add_gravity(scene.gravity)
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        t = time.perf_counter()
        sim(scene.dt, callers.array, scene.substeps, scene.pos_iters, int(scene.collisions))
        wall += time.perf_counter() - t
        callers.clear_forces()
    tb1 = (C.c_uint64 * 2)()
    rawphys.load_library().rp_transfer_bytes(C.c_void_p(lib.rp_compat_world()), tb1)
    lib.rp_compat_reset()
    return {"value": scene.num_dynamic * scene.substeps * frames / wall, "unit": UNIT,
            "h2d_bytes_per_step": (tb1[0] - tb0[0]) // frames, "d2h_bytes_per_step": (tb1[1] - tb0[1]) // frames,
            "call": "pbd_simulate(dt, Entity**, 20, 1, true), C++-mangled, FP32 default; state written back and "
                    "transformed hulls refreshed every call"}


def measure_adjoint(args, dev):
    """grad/s of the adjoint on a bounded sample of the differentiation workload (1024 domino rows of
    16-64 with a thrown cube, loss |x_last - target|^2 after 120 steps, gradients with respect to
    initial v / w, masses and friction, checkpoints every 10 steps): the first `adjoint_scenes` scenes
    of the same generator over `adjoint_frames` frames."""
    import torch
    import rawphys
    from rawphys import scenes as S
    batch, last, target = S.domino_batch(1024, seed=0)
    keep = batch.scene < args.adjoint_scenes
    idx = np.nonzero(keep)[0]
    remap = -np.ones(batch.num_bodies, dtype=np.int64)
    remap[idx] = np.arange(len(idx))
    sub = S.SceneBatch(batch.name, batch.meshes, batch.scene[keep], batch.mesh[keep], batch.scale[keep], batch.pos[keep],
                       batch.rot[keep], batch.mass[keep], batch.fixed[keep], batch.mus[keep], batch.mud[keep],
                       batch.rest[keep], batch.vel[keep], batch.omega[keep], [], num_scenes=args.adjoint_scenes, steps=120)
    w = rawphys.World(dev, "fp64")
    w.load_batch(sub)
    le = remap[last[:args.adjoint_scenes]].astype(np.int32)
    K = min(10, args.adjoint_frames)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res = w.adjoint(args.adjoint_frames, le, target[:args.adjoint_scenes], checkpoint_every=K)
    secs = time.perf_counter() - t0
    prof = w.adjoint_profile()
    w.close()
    n = args.adjoint_scenes
    return {"value": n / secs, "unit": "scene-gradients/s", "scenes": n, "frames": args.adjoint_frames,
            "seconds": secs, "scene_frame_gradients_per_s": n * args.adjoint_frames / secs,
            "workload": "bounded sample of the differentiation workload: the first %d of 1024 domino scenes (16-64 "
                        "dominoes and a thrown cube each), %d of its 120 frames, dt=1/60, 20 substeps, collisions on, "
                        "checkpoints every %d frames; loss |x_last_domino - target|^2, gradients with respect to every "
                        "body's initial v, w, mass and static / dynamic friction; FP64 adjoint" % (n, args.adjoint_frames, K),
            "full_workload_estimate_s": secs * (1024.0 / n) * (120.0 / args.adjoint_frames),
            "slowest_scene_profile": prof, "loss_mean": float(np.mean(res["loss"])),
            "gradient_check": "FP64 central differences, tests/test_gpu_adjoint.py (relative error <= 1e-3)"}


def run_ours(args):
    import torch
    import rawphys
    rank, world_size, local = dist_info()
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = local
    torch.cuda.set_device(dev)
    if args.workload != "batched":
        run_plain_only(args, dev, rank, world_size)
        return
    b = measure_batched(args, dev, rank, world_size, with_oracle=(rank == 0))
    plain = {}
    if rank == 0 and args.plain:
        p32 = measure_plain(args, dev, "fp32", args.plain_steps, with_oracle=True)
        p64 = measure_plain(args, dev, "fp64", max(3, args.plain_steps // 3), start_from=p32["start_state"])
        for p in (p32, p64):
            p.pop("start_state")
        plain = {"workload": PLAIN_WORKLOAD + "; frames after a %d-frame settle" % args.settle,
                 "fp32": p32, "fp64": p64, "fp32_over_fp64": p32["value"] / p64["value"]}
    adjoint = measure_adjoint(args, dev) if args.adjoint_scenes > 0 and rank == 0 else None
    precision = None
    if args.precision_towers > 0 and rank == 0:
        from rawphys import scenes as S
        from rawphys.precision import precision_report
        precision = precision_report(rawphys, S.tower_batch(args.precision_towers, n=64, seed=0),
                                     frames=args.precision_frames, sample_every=max(1, args.precision_frames // 6),
                                     device=dev)
        precision["workload"] = ("%d towers of 64 unit cubes, masses alternating 1:100, 50 substeps, dt=1/60; FP32 build "
                                 "against the all-FP64 build (bit-identical to the FP64 CPU oracle, tests/test_gpu_precision.py)"
                                 % args.precision_towers)
    if rank == 0:
        line = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": b["total_ms"] / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
                "config": {"workload": BATCHED_WORKLOAD},
                "details": {"batch": b["workload_detail"], "sweep_order": args.sweep_order, "l2": "flushed (256 MiB write) before every timed frame",
                            "parallelism": "scenes sharded by rank (own batch per rank)" if world_size > 1 else "one GPU",
                            "pairs_per_step": b["pairs_per_step"], "contacts_per_step": b["contacts_per_step"],
                            "phase_ms_per_step": b["phase"], "autotuned": b["tuned"],
                            "frame_ms": [round(x, 3) for x in b["ms"]]},
                "gpu_launches": b["launches"],
                "step_err": b.get("step_err"),
                "roofline": b["roofline"],
                "fp32_pipe": b["fp32_pipe"],
                "cpu_baseline": b.get("cpu_baseline"),
                "e2e": b["e2e"], "clocks": b["clocks"], "device_status": b["status"],
                "degenerate_first": b["degenerate_first"],
                "vs_plain_gpu": b["value"] / plain["fp32"]["value"] if plain else None,
                "plain": plain or None, "adjoint": adjoint, "precision": precision}
        print(json.dumps(line), flush=True)
    if world_size > 1:
        torch.distributed.destroy_process_group()


def run_plain_only(args, dev, rank, world_size):
    """--workload large4096 / stack10: the plain form as the line's value (replicas under torchrun)."""
    import torch
    p = measure_plain(args, dev, "fp32", args.steps, with_oracle=(rank == 0))
    total_ms = p["ms_per_step"] * args.steps
    if world_size > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    scene = make_scene(args.workload)
    value = scene.num_dynamic * scene.substeps * args.steps * world_size / (total_ms / 1e3)
    if rank == 0:
        p.pop("start_state")
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
                "config": {"workload": PLAIN_WORKLOAD if args.workload == "large4096" else args.workload},
                "details": {"parallelism": "replicas only" if world_size > 1 else "single scene, one GPU",
                            "l2": "flushed (256 MiB write) before every timed frame",
                            "phase_ms_per_step": p["phase_ms_per_step"], "autotuned": p["autotuned"],
                            "pairs_per_step": p["pairs_per_step"], "contacts_per_step": p["contacts_per_step"],
                            "levels_per_step": p["levels_per_step"]},
                "gpu_launches": p["gpu_launches"], "step_err": p.get("step_err"), "roofline": p["roofline"],
                "cpu_baseline": p.get("cpu_baseline"), "e2e": p["e2e"], "clocks": p["clocks"],
                "device_status": p["device_status"]}
        print(json.dumps(line), flush=True)
    if world_size > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--settle", type=int, default=120, help="untimed frames before the plain form's timed frames")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched", choices=["batched", "large4096", "stack10"])
    ap.add_argument("--batched-scenes", type=int, default=16384)
    ap.add_argument("--batched-settle", type=int, default=20)
    ap.add_argument("--e2e-frames", type=int, default=3)
    ap.add_argument("--err-scenes", type=int, default=128, help="scenes of the batch the oracle checks")
    ap.add_argument("--ref-scenes", type=int, default=256, help="scenes of the batch the reference arm runs")
    ap.add_argument("--no-plain", dest="plain", action="store_false", help="skip the plain single-scene form")
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--precision-towers", type=int, default=128, help="0 skips the precision-stress report")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false", help="keep the default launch configuration")
    ap.add_argument("--sweep-order", default="reference", choices=["reference", "coloured"],
                    help="Gauss-Seidel order of the constraint sweeps")
    ap.add_argument("--precision-frames", type=int, default=300)
    ap.add_argument("--adjoint-scenes", type=int, default=152, help="0 skips the adjoint grad/s measurement")
    ap.add_argument("--adjoint-frames", type=int, default=4)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
