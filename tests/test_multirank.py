"""The multi-GPU path on CPU ranks (gloo, world_size 2): the batched form shards by scene with no
exchange while stepping; every rank builds its shard of the batch, the shards partition the batch,
each rank steps its shard (with the oracle port, the CPU stand-in for its GPU) and the gathered
states equal the unsharded batch's run, and the bench's timing reduction (max over ranks) and
throughput sum behave as on GPUs."""
from __future__ import annotations

import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, os.path.join(ROOT, "raw-physics_gb300"))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import rawphys
    from rawphys import scenes as S
    batch = S.batched_scenes(24, seed=11, min_bodies=2, max_bodies=40, chain_fraction=0.25, chain_links=(8, 10))
    shard = S.shard_batch(batch, rank, world)
    w = rawphys.World(-1, "fp32")          # host-only world: the shard's entities and joints load
    first = w.load_batch(shard)
    n = w.num_entities()
    w.close()
    # step the shard: every scene of it, 5 frames, with no exchange between ranks
    from oracle.oracle import Oracle, build
    build(ref=False)
    states = []
    for s in range(shard.num_scenes):
        o = Oracle("port").load(S.batch_scene(shard, s))
        o.step(5)
        states.append(o.get_state())
    mine = np.concatenate(states) if states else np.zeros((0, 28))
    every = [None] * world
    dist.all_gather_object(every, mine)
    if rank == 0:
        np.save(out + ".states.npy", np.concatenate(every))
    stats = torch.tensor([shard.num_scenes, shard.num_bodies, len(shard.constraints), first, n], dtype=torch.int64)
    gathered = [torch.zeros_like(stats) for _ in range(world)]
    dist.all_gather(gathered, stats)
    # the bench's reduction: slowest rank's time, throughput summed over ranks
    t = torch.tensor([1.0 + rank], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        np.save(out, np.stack([g.numpy() for g in gathered] + [np.array([t.item(), batch.num_scenes, batch.num_bodies,
                                                                         len(batch.constraints), 0])]))
    dist.barrier()
    dist.destroy_process_group()


def test_batched_form_shards_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "stats.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    res = np.load(out)
    shards, tail = res[:2], res[2]
    assert tail[0] == 2.0                                   # max over ranks
    assert shards[:, 0].sum() == tail[1]                    # scenes partitioned
    assert shards[:, 1].sum() == tail[2]                    # bodies partitioned
    assert shards[:, 2].sum() == tail[3]                    # joints stay with their scene
    assert np.all(shards[:, 0] > 0) and np.all(shards[:, 3] == 0) and np.all(shards[:, 4] == shards[:, 1])
    # the sharded run equals the unsharded batch's, scene by scene
    sys.path.insert(0, os.path.join(ROOT, "raw-physics_gb300"))
    sys.path.insert(0, ROOT)
    from oracle.oracle import Oracle, build
    from rawphys import scenes as S
    build(ref=False)
    batch = S.batched_scenes(24, seed=11, min_bodies=2, max_bodies=40, chain_fraction=0.25, chain_links=(8, 10))
    whole = []
    for s in range(batch.num_scenes):
        o = Oracle("port").load(S.batch_scene(batch, s))
        o.step(5)
        whole.append(o.get_state())
    assert np.array_equal(np.load(out + ".states.npy"), np.concatenate(whole))
