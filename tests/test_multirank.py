"""Host logic of runs on several GPUs, with two gloo ranks on the CPU.

The oracle stands in for each rank's GPU: a round sharded over two ranks and gathered
must give every rank the results of the unsharded round, in pixel order.
"""
import os
import socket

import numpy as np
import pytest

from foort_gb300 import abi, multirank, workloads


def test_shard_range_covers_without_overlap():
    for n in (0, 1, 7, 100, 16384):
        for world in (1, 2, 3, 8):
            got = [multirank.shard_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            sizes = [hi - lo for lo, hi in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        multirank.shard_range(10, 2, 2)
    assert multirank.shard_images(64, 1, 2) == list(range(32, 64))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        wl = workloads.c1(side=12)
        px = wl.simple_pixels()
        res = multirank.sharded_round(px, lambda p: oracle.integrate(wl.desc, p, fast=False, nthreads=1),
                                      rank, world, dist)
        t = multirank.max_over_ranks(1.0 + rank, dist)
        np.save(os.path.join(outdir, f"rank{rank}.npy"), res)
        with open(os.path.join(outdir, f"rank{rank}.txt"), "w") as f:
            f.write(repr(t))
    finally:
        dist.destroy_process_group()


def test_sharded_round_over_two_gloo_ranks(oracle_mod, tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    wl = workloads.c1(side=12)
    want = oracle_mod.integrate(wl.desc, wl.simple_pixels(), fast=False)
    for r in range(world):
        got = np.load(tmp_path / f"rank{r}.npy")
        assert got.dtype == abi.RESULT_DTYPE and len(got) == len(want)
        for name in abi.RESULT_DTYPE.names:
            np.testing.assert_array_equal(got[name], want[name], err_msg=name)
        assert float((tmp_path / f"rank{r}.txt").read_text()) == 2.0  # max over ranks
