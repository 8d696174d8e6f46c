"""Benchmark of the GB300 rigid-body step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload large4096|stack10|batched]

Workload (default): the single large scene — 4096 convex bodies (cube / icosahedron / 32-segment
cylinder / 42-vertex icosphere, scale U(0.5,1.5), density 1) in a fixed 40x40x60 m box, dt=1/60,
20 substeps, 1 position iteration, FP32 build with FP64 poses; seeded synthetic data. The scene is
first advanced `--settle` frames (untimed) so the timed frames see the falling / colliding regime,
then W warm-up frames, then K timed frames. A "step" is one pbd_simulate frame.

Printed JSON line (rank 0):
  value     body-substeps/s = dynamic bodies x substeps x K / summed device time of the K frames
            (CUDA events on the world's stream; L2 flushed with a 256 MiB write before every frame)
  e2e       the same metric through the C ABI with host buffers: every frame uploads the full body
            state (rp_state_set), steps, and downloads it (rp_state_get), copies inside the timer
  roofline  the dominant kernel (the position sweep, one launch per substep): its algorithmic
            bytes per launch / its average duration from CUDA events around each phase, against
            the measured HBM copy bandwidth
  cpu_baseline  the oracle port (plain-C restatement of the reference, bit-exact to it) on one host
            core, on a bounded sample of the same workload
  batched   the batched form beside it: 16384 independent scenes of 2-512 bodies (a quarter with
            hinge / spherical chains) in one world, one CUDA-graph replay per frame
  precision the precision-stress report: 128 towers of 64 cubes (masses 1:100, 50 substeps) run
            in the FP32 and the all-FP64 builds side by side for 300 frames (per-step error from
            identical states, trajectory divergence, tower drift, energy drift)
  adjoint   grad/s of the adjoint (scene-gradients per second) on a bounded sample of the
            differentiation workload: 152 of its 1024 domino scenes over 4 of its 120 frames
--workload batched measures the batched form alone (its value becomes the line's value).
--impl reference times that CPU implementation on every host core instead (one replica of the
workload per core; the reference is single-threaded and keeps process-global state).
Multi-GPU (torchrun): the single scene does not shard, so every rank steps its own replica
("replicas only"); value is the sum over ranks of body-substeps over the slowest rank's time. The
batched form shards by scene: every rank steps its own batch.
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
# Algorithmic bytes of the plain form (per substep): body state read + written, the pair list, and
# every contact record written once and read by the position and velocity solves.
STATE_READ_B, STATE_WRITE_B, PAIR_B, CONTACT_B = 160, 84, 16, 156
# Algorithmic bytes of one position sweep (the dominant kernel): every contact record read (48 B)
# and its two lambdas written back (8 B); per solved pair node, both bodies' pose read and written
# (2 x 64 B) and their inverse mass and inertia read (2 x 28 B).
SWEEP_CONTACT_B, SWEEP_NODE_B = 56, 2 * (64 + 64 + 28)


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


def profile_traffic():
    """DRAM bytes per position-sweep launch from the committed ncu summary, if one exists."""
    path = os.path.join(ROOT, "profiles", "pipeline_large4096.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def cpu_baseline_sample(scene, state, frames=3):
    """The oracle port on one core: body-substeps/s over `frames` frames of the workload, started
    from the state the timed GPU frames started from."""
    from oracle.oracle import Oracle, build
    build(ref=False)
    o = Oracle("port").load(scene)
    o.set_state(state)
    t = time.perf_counter()
    o.step(frames)
    dt = time.perf_counter() - t
    return scene.num_dynamic * scene.substeps * frames / dt, dt


_WORKER = {}


def _ref_init(name, state):
    sys.path.insert(0, os.path.join(ROOT, "raw-physics_gb300"))
    sys.path.insert(0, ROOT)
    from oracle.oracle import Oracle
    scene = make_scene(name)
    _WORKER["scene"] = scene
    _WORKER["oracle"] = Oracle("port").load(scene)
    _WORKER["state"] = state


def _ref_frame(frames):
    o, scene = _WORKER["oracle"], _WORKER["scene"]
    o.set_state(_WORKER["state"])
    t = time.perf_counter()
    o.step(frames)
    return scene.num_dynamic * scene.substeps * frames, time.perf_counter() - t


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle.oracle import Oracle, build
    build(ref=False)
    cores = os.cpu_count() or 1
    scene = make_scene(args.workload)
    # the same settled frames the GPU arm times, settled by the CPU implementation itself
    o = Oracle("port").load(scene)
    o.step(args.settle)
    state = o.get_state()
    frames = 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_ref_init, initargs=(args.workload, state)) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_frame, [frames] * cores)
        t = time.perf_counter()
        total = 0
        for _ in range(args.steps):
            total += sum(b for b, _ in pool.map(_ref_frame, [frames] * cores))
        wall = time.perf_counter() - t
    value = total / wall
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene generator)",
            "config": {"workload": "%s: %d dynamic bodies, %d substeps, dt=1/60, 1 position iteration; frame %d "
                                   "(after a %d-frame settle), one frame per core per step"
                                   % (args.workload, scene.num_dynamic, scene.substeps, args.settle + 1, args.settle)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d replicas x %d frame(s) per step of the workload, oracle port (bit-exact "
                                       "restatement of the reference, -O2 -ffp-contract=off)" % (cores, frames)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
    if args.workload == "batched":
        run_batched_only(args, dev, rank, world_size)
        return
    stream = torch.cuda.Stream(dev)          # a capturable stream: frames replay from a CUDA graph
    scene = make_scene(args.workload)
    w = rawphys.World(dev, "fp32")
    w.set_stream(stream.cuda_stream)
    w.load(scene)
    nd = scene.num_dynamic
    # untimed: settle into the colliding regime, pick the launch configuration, then warm up
    if args.settle:
        w.step(args.settle)
    tuned = w.autotune(frames=3) if args.autotune else None
    w.step(args.warmup)
    w.sync()
    start_state = w.get_state()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    c0 = w.counters()
    l0 = w.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)              # evict L2 (129 MB) before each timed frame
            ev[k][0].record(stream)
            w.step(1)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    if world_size > 1:
        torch.distributed.barrier()
    ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = float(sum(ms))
    launches = w.kernel_launches() - l0
    c1 = w.counters()
    # phase breakdown: the same frames again, untimed by the bench, with an event after every phase
    w.set_state(start_state)
    w.sync()
    p0 = w.phase_times()
    w.set_timing(True)
    w.step(args.steps)
    w.sync()
    w.set_timing(False)
    p1 = w.phase_times()
    phase_ms = {k: round((p1[k] - p0[k]) / args.steps, 4) for k in p0}
    # slowest rank
    if world_size > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = nd * scene.substeps * args.steps * world_size / (total_ms / 1e3)
    status = w.status()

    # roofline of the dominant kernel, the position sweep (one launch per substep): algorithmic bytes
    # per launch over its duration, both from the phase pass (CUDA events around each phase)
    pairs_per_step = (c1[6] - c0[6]) / args.steps
    contacts_per_step = (c1[5] - c0[5]) / args.steps
    manifolds_per_step = (c1[2] - c0[2]) / args.steps
    sweeps = scene.substeps * scene.pos_iters
    alg_bytes = (contacts_per_step * SWEEP_CONTACT_B + manifolds_per_step * SWEEP_NODE_B) / scene.substeps
    launch_ms = phase_ms["solve"] / sweeps
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic = profile_traffic()

    # end to end through the C ABI with host buffers, over the same frames the device-timed loop ran
    # (from its start state; two untimed frames first)
    st = start_state
    for _ in range(2):
        w.set_state(st)
        w.step(1)
        w.get_state()
    st = start_state
    b0 = w.transfer_bytes()
    torch.cuda.synchronize()
    t = time.perf_counter()
    e2e_steps = max(3, args.steps // 2)
    for _ in range(e2e_steps):
        w.set_state(st)
        w.step(1)
        st = w.get_state()
    e2e_wall = time.perf_counter() - t
    b1 = w.transfer_bytes()
    e2e = {"value": nd * scene.substeps * e2e_steps * world_size / e2e_wall, "unit": UNIT,
           "h2d_bytes_per_step": (b1[0] - b0[0]) // e2e_steps, "d2h_bytes_per_step": (b1[1] - b0[1]) // e2e_steps}

    w.close()
    batched = measure_batched(args, dev, rank, world_size, value) if args.batched_scenes > 0 else None
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
        cpu_v, cpu_t = cpu_baseline_sample(scene, start_state, frames=args.cpu_frames)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
                "config": {"workload": "large single scene: %d dynamic bodies (cube/icosahedron/cylinder32/icosphere42, "
                                       "scale U(0.5,1.5)) in a 40x40x60 m box, dt=1/60, %d substeps, 1 position iteration, "
                                       "FP32 with FP64 poses; frames %d-%d after a %d-frame settle"
                                       % (nd, scene.substeps, args.settle + args.warmup,
                                          args.settle + args.warmup + args.steps, args.settle),
                           "l2": "flushed (256 MiB write) before every timed frame",
                           "parallelism": "replicas only" if world_size > 1 else "single scene, one GPU",
                           "pairs_per_step": pairs_per_step, "contacts_per_step": contacts_per_step,
                           "levels_per_step": (c1[7] - c0[7]) / args.steps,
                           "gjk_iters_per_step": (c1[0] - c0[0]) / args.steps,
                           "epa_calls_per_step": (c1[2] - c0[2]) / args.steps,
                           "epa_iters_per_step": (c1[1] - c0[1]) / args.steps,
                           "gjk_cap_hits_per_step": (c1[8] - c0[8]) / args.steps,
                           "gjk_cycles_detected_per_step": (c1[18] - c0[18]) / args.steps,
                           "epa_cap_hits_per_step": (c1[9] - c0[9]) / args.steps,
                           "pair_cycles_max": c1[10],
                           "pair_cycles_mean": (c1[11] - c0[11]) / max(1, c1[12] - c0[12]),
                           "pairs_narrowphased_per_step": (c1[12] - c0[12]) / args.steps,
                           "pairs_bounds_apart_per_step": (c1[13] - c0[13]) / args.steps,
                           "gjk_epa_manifold_support_cycles_per_step": [(c1[k] - c0[k]) / args.steps for k in (14, 15, 16, 17)],
                           "phase_ms_per_step": phase_ms, "autotuned": tuned},
                "gpu_launches": launches,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                             "peak_kind": peak_kind, "traffic": traffic, "kernel": "k_sweep_grid (position sweep)",
                             "alg_bytes_per_launch": alg_bytes, "launch_ms": launch_ms},
                "batched": batched,
                "adjoint": adjoint,
                "precision": precision,
                "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": 1, "kind": "port",
                                 "sample": "%d frames of the same scene from the state the timed GPU frames start "
                                           "from, oracle port (bit-exact restatement of the reference), %.1f s"
                                           % (args.cpu_frames, cpu_t)},
                "e2e": e2e, "clocks": clk.summary(), "device_status": status}
        print(json.dumps(line), flush=True)
    if world_size > 1:
        torch.distributed.destroy_process_group()


def measure_batched(args, dev, rank, world_size, plain_value):
    """The batched form: many independent scenes of uneven size in one world (rawphys.scenes.
    batched_scenes), every frame one replay of the captured phase-major graph. Weak scaling: every
    rank steps its own batch (seed = rank)."""
    import torch
    import rawphys
    from rawphys import scenes as S
    batch = S.batched_scenes(args.batched_scenes, seed=rank)
    stream = torch.cuda.Stream(dev)
    w = rawphys.World(dev, "fp32")
    w.set_stream(stream.cuda_stream)
    w.load_batch(batch)
    w.step(args.batched_settle)
    tuned = w.autotune(frames=2) if args.autotune else None
    w.step(3)
    w.sync()
    nd = batch.num_dynamic
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    c0 = w.counters()
    l0 = w.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.batched_steps)]
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for k in range(args.batched_steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)
            ev[k][0].record(stream)
            w.step(1)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    total_ms = float(sum(a.elapsed_time(b) for a, b in ev))
    c1 = w.counters()
    launches = w.kernel_launches() - l0
    if world_size > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    p0 = w.phase_times()
    w.set_timing(True)
    w.step(2)
    w.sync()
    w.set_timing(False)
    p1 = w.phase_times()
    # end to end through the C ABI with host buffers: every frame uploads the whole batch's state,
    # steps, and downloads it
    st = w.get_state()
    w.set_state(st)
    w.step(1)
    st = w.get_state()
    b0 = w.transfer_bytes()
    e2e_frames = 3
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(e2e_frames):
        w.set_state(st)
        w.step(1)
        st = w.get_state()
    e2e_wall = time.perf_counter() - t
    b1 = w.transfer_bytes()
    e2e = {"value": nd * batch.substeps * e2e_frames * world_size / e2e_wall, "unit": UNIT,
           "h2d_bytes_per_step": (b1[0] - b0[0]) // e2e_frames, "d2h_bytes_per_step": (b1[1] - b0[1]) // e2e_frames}
    value = nd * batch.substeps * args.batched_steps * world_size / (total_ms / 1e3)
    sizes = batch.scene_sizes()
    # roofline of the batched form's dominant kernel, the position sweep (k_sweep_warp, one launch per
    # substep): the same algorithmic bytes per contact and per solved pair as the plain form's
    phase = {k: round((p1[k] - p0[k]) / 2, 3) for k in p0}
    steps = args.batched_steps
    alg_bytes = ((c1[5] - c0[5]) / steps * SWEEP_CONTACT_B + (c1[2] - c0[2]) / steps * SWEEP_NODE_B) / batch.substeps
    launch_ms = phase["solve"] / (batch.substeps * batch.pos_iters)
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9 if launch_ms > 0 else 0.0
    peak, peak_kind = measured_peak_hbm()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": peak_kind, "kernel": "k_sweep_warp (position sweep, one warp per scene)",
                "alg_bytes_per_launch": alg_bytes, "launch_ms": launch_ms}
    out = {"value": value, "unit": UNIT, "ms_per_step": total_ms / args.batched_steps, "steps": args.batched_steps,
           "vs_plain_gpu": value / plain_value if plain_value else None,
           "workload": "%d independent scenes, dynamic bodies per scene log-uniform in [2, 512] (mean %.1f, max %d; "
                       "%d dynamic bodies in all), large-scene shape mix, %d scenes with 8-64-link hinge or spherical "
                       "chains (%d joints), dt=1/60, %d substeps, FP32 with FP64 poses; frames %d-%d after a %d-frame "
                       "settle" % (batch.num_scenes, sizes.mean(), sizes.max(), nd,
                                   len({int(batch.scene[c.e1]) for c in batch.constraints}), len(batch.constraints),
                                   batch.substeps, args.batched_settle + 3, args.batched_settle + 3 + args.batched_steps,
                                   args.batched_settle),
           "l2": "flushed (256 MiB write) before every timed frame",
           "pairs_per_step": (c1[6] - c0[6]) / args.batched_steps,
           "contacts_per_step": (c1[5] - c0[5]) / args.batched_steps,
           "phase_ms_per_step": phase, "roofline": roofline,
           "e2e": e2e, "clocks": clk.summary(), "device_status": w.status(), "gpu_launches": launches,
           "autotuned": tuned}
    w.close()
    return out


def measure_adjoint(args, dev):
    """grad/s of the adjoint on a bounded sample of the differentiation workload (1024 domino rows of
    16-64 with a thrown cube, loss |x_last - target|^2 after 120 steps, gradients with respect to
    initial v / w, masses and friction, checkpoints every 10 steps): the first `adjoint_scenes` scenes
    of the same generator over `adjoint_frames` frames. The adjoint runs one scene per GPU thread in
    FP64; its time grows linearly with the frames and, above one scene per SM, with the scenes."""
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


def run_batched_only(args, dev, rank, world_size):
    """--workload batched: the batched form alone, as the line's own value."""
    import torch
    b = measure_batched(args, dev, rank, world_size, None)
    if rank == 0:
        line = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": world_size, "steps": b["steps"],
                "warmup": 3, "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
                "config": {"workload": b["workload"], "l2": b["l2"],
                           "parallelism": "scenes sharded by rank (own batch per rank)" if world_size > 1 else "one GPU",
                           "pairs_per_step": b["pairs_per_step"], "contacts_per_step": b["contacts_per_step"],
                           "phase_ms_per_step": b["phase_ms_per_step"]},
                "roofline": b["roofline"],
                "gpu_launches": b["gpu_launches"], "e2e": b["e2e"], "clocks": b["clocks"],
                "device_status": b["device_status"]}
        print(json.dumps(line), flush=True)
    if world_size > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--settle", type=int, default=120)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large4096", choices=["large4096", "stack10", "batched"])
    ap.add_argument("--cpu-frames", type=int, default=2)
    ap.add_argument("--batched-scenes", type=int, default=16384, help="0 skips the batched measurement")
    ap.add_argument("--batched-steps", type=int, default=10)
    ap.add_argument("--batched-settle", type=int, default=20)
    ap.add_argument("--precision-towers", type=int, default=128, help="0 skips the precision-stress report")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false", help="keep the default launch configuration")
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
