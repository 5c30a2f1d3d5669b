"""One process per GPU: rank setup, the bench's reductions and the bucket
partition.

The force evaluation shards into independent buckets: each bucket's
accelerations depend only on the read-only moments and particles and on its
own list (HostCUDA.cu:1030-1033), and no two buckets write the same result
row.  So ranks need no collective on the data path:

* ``replicas`` (what bench.py --gpus N runs): every rank evaluates its own
  copy of the workload (weak scaling);
* ``partition_buckets``: contiguous bucket ranges in tree (key) order,
  balanced by interactions rather than by bucket count, the rule a sharded
  run uses (each rank builds or receives only its range's lists).

The only collectives are the timing barrier and the max / sum of scalars
over ranks; they run on NCCL with GPUs and on gloo without.
"""
from __future__ import annotations

import os

import numpy as np


def setup():
    """(world, rank, local_rank) from the torch.distributed.run environment;
    initialises the process group for world > 1 (NCCL on GPUs, else gloo)."""
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            if torch.cuda.is_available():
                torch.cuda.set_device(local)
                dist.init_process_group("nccl", device_id=torch.device("cuda", local))
            else:
                dist.init_process_group("gloo")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def _device():
    import torch.distributed as dist
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(world, x, op):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(world, x):
    import torch.distributed as dist
    return x if world == 1 else _reduce(world, x, dist.ReduceOp.MAX)


def sum_over_ranks(world, x):
    import torch.distributed as dist
    return x if world == 1 else _reduce(world, x, dist.ReduceOp.SUM)


def partition_buckets(work, n_parts):
    """Splits buckets 0..B-1 (tree order) into n_parts contiguous ranges
    whose summed work (interactions per bucket) is as even as a prefix
    split allows: range k ends at the first bucket where the running total
    reaches (k + 1) / n_parts of the whole.  Returns n_parts + 1 bounds."""
    w = np.asarray(work, dtype=np.float64)
    if n_parts < 1:
        raise ValueError("n_parts must be >= 1")
    cum = np.concatenate([[0.0], np.cumsum(w)])
    total = cum[-1]
    bounds = [0]
    for k in range(1, n_parts):
        b = int(np.searchsorted(cum, total * k / n_parts, side="left"))
        bounds.append(min(max(b, bounds[-1]), len(w)))
    bounds.append(len(w))
    return np.array(bounds, dtype=np.int64)


def bucket_work(lists):
    """Interactions per bucket of a TreeLists (cell + particle lists), in
    bucket-id order."""
    nb = len(lists.bucket_starts)
    w = np.zeros(nb, dtype=np.int64)
    for req in (lists.cells, lists.plist):
        lens = np.diff(req.markers.astype(np.int64)) * req.sizes.astype(np.int64)
        np.add.at(w, req.bucket_ids.astype(np.int64), lens)
    return w
