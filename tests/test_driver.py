"""Host-side pair scheduling (PNAMP_Main.f90:60-84) and its multi-rank split on CPU (gloo)."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from sccm_gb300.driver import pair_list, rank_pairs


def test_pair_list_matches_reference_loops():
    # ICons = 1: all q' for every q; otherwise the upper triangle q' >= q
    assert pair_list(1, 2, 1, 3, icons=1) == [(1, 1), (1, 2), (1, 3), (2, 1), (2, 2), (2, 3)]
    assert pair_list(1, 3, 1, 3, icons=0) == [(1, 1), (1, 2), (1, 3), (2, 2), (2, 3), (3, 3)]


def test_rank_round_robin_is_a_partition():
    pairs = pair_list(1, 20, 1, 20, icons=0)
    for nprocs in (1, 2, 3, 8):
        parts = [rank_pairs(pairs, r, nprocs) for r in range(nprocs)]
        assert sorted(p for part in parts for p in part) == sorted(pairs)
        assert sum(len(p) for p in parts) == len(pairs)
        # rank == ic mod nprocs with ic from 1 (PNAMP_Main.f90:84)
        assert parts[1 % nprocs][0] == pairs[0]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pairs = pair_list(1, 20, 1, 20, icons=0)
    mine = rank_pairs(pairs, rank, world)
    # every rank reports its pairs; rank 0 checks the union is the full list, disjoint
    t = torch.full((len(pairs),), -1, dtype=torch.int64)
    for k, p in enumerate(pairs):
        if p in mine:
            t[k] = rank
    g = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(g, t)
    if rank == 0:
        owner = torch.stack(g).max(0).values
        count = (torch.stack(g) >= 0).sum(0)
        out.put((int(owner.min()), int(count.min()), int(count.max())))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_split_covers_every_pair_once():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert res == (0, 1, 1)
