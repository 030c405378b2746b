"""Replicas on several GPUs: the host side, run as world-size-2 gloo process groups
on CPU (one process per rank, rendezvous on 127.0.0.1).

Checked: the wavelength shards of the 256-wavelength sweep are disjoint, complete and
balanced by cost; every rank computes the same split without communication; the
slowest rank's time is what every rank reports; the whole-job throughput counts every
rank's units; sweep shards merge back into wavelength order.
"""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from miepy_gb300 import replicas as RP
from miepy_gb300.sweep import SweepResult, adaptive_lmax


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _sweep_costs():
    wl = np.linspace(400e-9, 1000e-9, 256)
    return np.array([RP.unit_cost(100, L) for L in adaptive_lmax(wl)])


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        costs = _sweep_costs()
        mine = RP.my_shard(costs, rank, world)
        shards = RP.gather_objects(mine)
        t = RP.max_over_ranks(1.0 + rank)            # rank-dependent "time"
        load = [float(costs[s].sum()) for s in shards]
        np.save(os.path.join(out_dir, f"rank{rank}.npy"),
                np.array([t, len(mine), max(load) / np.mean(load)] + [len(s) for s in shards]))
        if rank == 0:
            allidx = np.sort(np.concatenate(shards))
            np.save(os.path.join(out_dir, "all.npy"), allidx)
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_and_timing(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    r0 = np.load(tmp_path / "rank0.npy")
    r1 = np.load(tmp_path / "rank1.npy")
    assert r0[0] == r1[0] == 2.0                     # both report the slowest rank's time
    assert np.array_equal(np.load(tmp_path / "all.npy"), np.arange(256))   # disjoint and complete
    assert r0[1] + r1[1] == 256
    assert r0[2] < 1.02                              # loads within 2 % of each other
    assert list(r0[3:]) == list(r1[3:])              # every rank derived the same split


def test_shard_balanced_single_process():
    costs = _sweep_costs()
    for world in (1, 3, 4, 8):
        parts = RP.shard_balanced(costs, world)
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(256))
        loads = np.array([costs[p].sum() for p in parts])
        assert loads.max() / loads.mean() < 1.05
    assert RP.aggregate_throughput([100, 156], [2.0, 2.5]) == 256 / 2.5
    assert RP.max_over_ranks(3.5) == 3.5             # no process group: the value itself


def test_merge_sweeps():
    def part(w):
        w = np.asarray(w, float)
        n = len(w)
        return SweepResult(wavelength=w, lmax=np.full(n, 3), C_sca=w[:, None] * 2, C_abs=w[:, None],
                           C_ext=w[:, None] * 3, status=np.zeros((n, 1), np.int32), iterations=np.ones((n, 1), int))
    m = RP.merge_sweeps([part([3.0, 1.0]), part([2.0, 4.0])])
    assert list(m.wavelength) == [1.0, 2.0, 3.0, 4.0]
    assert np.allclose(m.C_ext[:, 0], 3 * m.wavelength)
