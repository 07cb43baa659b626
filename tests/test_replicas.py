"""Replicas over ranks (world size 2, gloo on CPU): each rank solves its round-robin share of the
(energy, configuration) pairs and the results gather in order. The solves here are the oracle's
(CPU); on GPUs each rank runs the CUDA path on its own device the same way."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _energies():
    return [-0.12, -0.03, 0.04, 0.1, 0.15]


def _worker(rank, world, port, out_path):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist

    from caroli_gb300 import replicas
    from systems import magnetic_bhz, oracle_T

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys_ = magnetic_bhz(12, 8, configs=2)
        pairs = [(e, c) for e in _energies() for c in range(2)]
        mine, pos = replicas.shard(pairs, rank, world)
        sig = {e: sys_.self_energies(e) for e, _ in mine}
        local = [oracle_T(sys_, sig[e], config=c) for e, c in mine]
        full = replicas.gather(local, pos, len(pairs))
        if rank == 0:
            np.save(out_path, np.array(full))
    finally:
        dist.destroy_process_group()


def test_round_robin_replicas_gather_in_order(tmp_path):
    from systems import magnetic_bhz, oracle_T

    out = str(tmp_path / "t.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    sys_ = magnetic_bhz(12, 8, configs=2)
    want = [oracle_T(sys_, sys_.self_energies(e), config=c) for e in _energies() for c in range(2)]
    assert np.allclose(got, want, rtol=0, atol=1e-12)


def test_shard_covers_every_item_once():
    from caroli_gb300.replicas import shard

    items = list(range(11))
    seen = []
    for r in range(3):
        part, pos = shard(items, r, 3)
        assert part == [items[p] for p in pos]
        seen += pos
    assert sorted(seen) == items
