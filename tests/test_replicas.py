"""Replica (multi-GPU) host logic on CPU: two gloo ranks, as torchrun would start them.

Each rank steps its own contiguous shard of seeds with the oracle (the data path has no collective),
the per-rank timings are reduced with max over ranks, and the gathered shards equal a single-process
run over the whole batch.  Runs without a GPU; rendezvous on 127.0.0.1."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir, per_rank):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from exponax_gb300 import ic, replicas
    from oracle import exponax_np as o

    r, ws = replicas.init("gloo")
    assert (r, ws) == (rank, world)
    seeds = replicas.shard(per_rank, rank)
    st = o.KuramotoSivashinskyConservative(1, 100.0, 64, 0.1)
    gen = ic.RandomSineWaves1d(1, cutoff=5)
    mine = np.stack([o.repeat(st, 5)(gen(64, key=s)) for s in seeds])
    fake_ms = 10.0 + 7.0 * rank  # rank-dependent "timing"
    slowest = replicas.max_over_ranks(fake_ms)
    gathered = replicas.gather_to_rank0((list(seeds), mine))
    if rank == 0:
        seeds_all = [s for part in gathered for s in part[0]]
        states = np.concatenate([part[1] for part in gathered])
        np.savez(os.path.join(out_dir, "result.npz"), seeds=np.array(seeds_all), states=states,
                 slowest=np.array(slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_match_single_process(tmp_path):
    world, per_rank = 2, 3
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path), per_rank), nprocs=world,
                       join=True, start_method="spawn")
    res = np.load(tmp_path / "result.npz")
    assert list(res["seeds"]) == list(range(world * per_rank))  # disjoint, contiguous, complete shards
    assert float(res["slowest"]) == 17.0  # max over ranks
    from exponax_gb300 import ic
    from oracle import exponax_np as o

    st = o.KuramotoSivashinskyConservative(1, 100.0, 64, 0.1)
    gen = ic.RandomSineWaves1d(1, cutoff=5)
    want = np.stack([o.repeat(st, 5)(gen(64, key=s)) for s in range(world * per_rank)])
    np.testing.assert_array_equal(res["states"], want)


def test_aggregate_throughput_and_single_process_identity():
    from exponax_gb300 import replicas

    assert replicas.aggregate_throughput(1000, 4, 2.0) == 1000 * 4 / 2e-3
    assert replicas.max_over_ranks(3.5) == 3.5  # no process group: identity
    assert list(replicas.shard(4, 2, start=10)) == [18, 19, 20, 21]
    assert replicas.gather_to_rank0("x") == ["x"]
