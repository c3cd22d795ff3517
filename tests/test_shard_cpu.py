"""The multi-rank layout on the CPU: two gloo ranks integrate their grain shards (with
replicas of the massive set) through the oracle and sum their images; the result equals
the oracle on the whole system.  The grains are independent given the massive bodies, so
the shards' states are bit-identical to the whole run's, and the summed image agrees to
summation order."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from diskdyn_gb300 import shard, synth


def test_shard_range_partitions_exactly():
    for n in (0, 1, 7, 1000, 1048577):
        for world in (1, 2, 3, 8):
            ranges = [shard.shard_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import oracle.cpu as oc
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s = synth.imaging(n_dust=3001, xsize=48, ysize=40, n_img=2)
        s.phys = dict(s.phys, Rmin=0.05)
        part = shard.shard_state(s.state, s.n_grav, rank, world)
        stepped = oc.step(part, s.n_grav, s.dt, s.size_table, s.phys, 3)
        img, _ = oc.image(stepped, s.n_grav, s.optics, s.size_table["size"], s.view, s.image_wj)
        t = shard.sum_over_ranks(torch.tensor(img))
        units, secs, rate = shard.job_rate(float(len(part["x"]) - s.n_grav), 1.0 + rank)
        gathered = [None] * world
        dist.all_gather_object(gathered, {k: stepped[k] for k in ("x", "y", "z", "vx", "vy", "vz", "N")})
        if rank == 0:
            np.savez(out, img=t.numpy(), units=units, secs=secs, rate=rate,
                     **{f"{k}_{r}": g[k] for r, g in enumerate(gathered) for k in g})
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_whole_system(tmp_path):
    import oracle.cpu as oc
    oc.lib()                                   # build the oracle before the ranks start
    out = str(tmp_path / "ranks.npz")
    world = 2
    mp.start_processes(_rank_main, args=(world, free_port(), out), nprocs=world, join=True, start_method="spawn")
    r = np.load(out)
    s = synth.imaging(n_dust=3001, xsize=48, ysize=40, n_img=2)
    s.phys = dict(s.phys, Rmin=0.05)
    whole = oc.step(s.state, s.n_grav, s.dt, s.size_table, s.phys, 3)
    img, _ = oc.image(whole, s.n_grav, s.optics, s.size_table["size"], s.view, s.image_wj)
    ng = s.n_grav
    for k in ("x", "y", "z", "vx", "vy", "vz", "N"):
        grains = np.concatenate([r[f"{k}_{q}"][ng:] for q in range(world)])
        np.testing.assert_array_equal(grains, whole[k][ng:], err_msg=k)
        for q in range(world):
            np.testing.assert_array_equal(r[f"{k}_{q}"][:ng], whole[k][:ng], err_msg=k)
    np.testing.assert_allclose(r["img"], img, rtol=1e-13, atol=0)
    assert r["units"] == 3001 and r["secs"] == 2.0 and r["rate"] == 3001 / 2.0
