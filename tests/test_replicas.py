"""Multi-rank host logic on CPU (gloo, world size 2): the bench's barrier
and max / sum reductions, and the interaction-balanced bucket partition."""
import os
import socket

import numpy as np
import pytest

from changa_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    import torch.distributed as dist
    w, r, _ = replicas.setup()
    replicas.barrier(w)
    mx = replicas.max_over_ranks(w, 10.0 + r)
    sm = replicas.sum_over_ranks(w, 1.5 * (r + 1))
    q.put((r, w, mx, sm, dist.get_backend()))
    dist.destroy_process_group()


def test_gloo_world2_reductions():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for r, (rank, world, mx, sm, backend) in enumerate(got):
        assert (rank, world, backend) == (r, 2, "gloo")
        assert mx == 11.0 and sm == 4.5


def test_single_rank_is_identity():
    assert replicas.max_over_ranks(1, 3.25) == 3.25
    assert replicas.sum_over_ranks(1, 3.25) == 3.25


@pytest.mark.parametrize("n_parts", [1, 2, 3, 8])
def test_partition_balances_interactions(n_parts):
    rng = np.random.default_rng(3)
    work = rng.lognormal(8.0, 1.5, size=5000).astype(np.int64)
    b = replicas.partition_buckets(work, n_parts)
    assert b[0] == 0 and b[-1] == len(work) and (np.diff(b) >= 0).all()
    shares = np.array([work[b[k]:b[k + 1]].sum() for k in range(n_parts)]) / work.sum()
    # a prefix split is off by at most one bucket's work per boundary
    assert np.abs(shares - 1.0 / n_parts).max() <= work.max() / work.sum() + 1e-12


def test_bucket_work_matches_interactions(built):
    from changa_gb300 import ics, tree
    p = ics.plummer(2000, ics.rng_for(0))
    L = tree.build_lists(p["pos"], p["mass"], p["soft"], n_bucket=16, theta=0.7)
    w = replicas.bucket_work(L)
    assert w.sum() == L.interactions
    b = replicas.partition_buckets(w, 2)
    assert w[b[0]:b[1]].sum() + w[b[1]:b[2]].sum() == L.interactions
