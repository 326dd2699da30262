"""Query sharding across ranks (the multi-GPU layout of the KDE: every rank
holds the full training set and evaluates its contiguous query shard; no
data-path collective).  Run as two gloo ranks on the CPU with the oracle
standing in for the GPU kernel; checks the gathered result equals the
single-process evaluation."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_path: str):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    sys.path[:0] = [str(root / "flash-sd-kde_gb300"), str(root)]
    import torch

    from fsk.workloads import plain_kde_16d, shard
    from oracle import reference_numpy as R

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    x, q = plain_kde_16d(512, 301)
    lo, hi = shard(q.shape[0], world, rank)
    part = torch.from_numpy(R.kde_eval_nd_numpy(q[lo:hi], x, 0.8).astype(np.float32))
    sizes = [shard(q.shape[0], world, r)[1] - shard(q.shape[0], world, r)[0] for r in range(world)]
    # gloo all_gather needs equal sizes: pad to the largest shard
    pad = max(sizes)
    padded = torch.zeros(pad)
    padded[: part.numel()] = part
    gathered = [torch.empty(pad) for _ in range(world)]
    dist.all_gather(gathered, padded)
    if rank == 0:
        full = torch.cat([g[:s] for g, s in zip(gathered, sizes)]).numpy()
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_query_sharding(tmp_path):
    out = str(tmp_path / "full.npy")
    mp.spawn(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True)
    from fsk.workloads import plain_kde_16d
    from oracle import reference_numpy as R

    x, q = plain_kde_16d(512, 301)
    ref = R.kde_eval_nd_numpy(q, x, 0.8)
    np.testing.assert_array_equal(np.load(out), ref.astype(np.float32))
