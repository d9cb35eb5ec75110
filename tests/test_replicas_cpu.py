"""The multi-rank host logic on CPU: two gloo ranks (127.0.0.1) split the naive targets with
`target_range`, compute their share with the oracle, gather it and compare with the single-rank
result; the throughput reduction takes the slowest rank."""

import os
import socket

import numpy as np
import pytest

from nbody.replicas import target_range


def test_target_ranges_partition():
    for n in (0, 1, 7, 100, 1001):
        for ws in (1, 2, 3, 8):
            spans = [target_range(n, r, ws) for r in range(ws)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        target_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world_size, port, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "n-body-simulation_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch
    import torch.distributed as dist

    import oracle
    from nbody import generators
    from nbody.replicas import job_throughput, target_range
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world_size)
    d = generators.plummer(301, seed=5)
    b, e = target_range(301, rank, world_size)
    ax, ay, az = oracle.naive_accel_subset(d["m"], d["x"], d["y"], d["z"],
                                          np.arange(b, e, dtype=np.uint32), 1.0, 1e-6, threads=1)
    sizes = [target_range(301, r, world_size) for r in range(world_size)]
    width = max(s[1] - s[0] for s in sizes)  # all_gather wants equal shapes: pad the shorter
    part = torch.zeros(3, width, dtype=torch.float64)
    part[:, : e - b] = torch.tensor(np.stack([ax, ay, az]), dtype=torch.float64)
    bufs = [torch.zeros(3, width, dtype=torch.float64) for _ in sizes]
    dist.all_gather(bufs, part)
    bufs = [buf[:, : s[1] - s[0]] for buf, s in zip(bufs, sizes)]
    # rank r "took" 1 + r seconds for 10 steps: the job rate uses the slowest rank
    rate = job_throughput(10, 1.0 + rank, world_size)
    if rank == 0:
        full = torch.cat(bufs, dim=1).numpy()
        np.save(os.path.join(out_dir, "gathered.npy"), full)
        np.save(os.path.join(out_dir, "rate.npy"), np.array([rate]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_naive_targets(tmp_path):
    import torch.multiprocessing as mp

    import oracle
    from nbody import generators
    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2,
                       start_method="spawn", join=True)
    d = generators.plummer(301, seed=5)
    ref = np.stack(oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], 1.0, 1e-6, threads=1))
    np.testing.assert_array_equal(np.load(tmp_path / "gathered.npy"), ref)
    assert np.load(tmp_path / "rate.npy")[0] == pytest.approx(2 * 10 / 2.0)
