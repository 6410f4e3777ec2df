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


def _c2_shaped():
    """C2's shape at a size the oracle runs in seconds: Kerr a = 0.99 at 60 deg with a
    SquareSubdivisionMeshV2 (9^2 seed, MaxSubdivide 3: grid 33; 24 pixels per refinement
    round), camera and boundary sphere at r = 60 so that each ray is short."""
    wl = workloads.c2()
    d = wl.desc
    d.boundary_radius = 60.0
    keep = abi.attach_images(d, [abi.make_image((0.99,), r=60.0, theta=60 * workloads.DEG, half_width=12.0)])
    mesh = [("v2", dict(max_pixels=0, initial_pixels=81, max_subdivide=3, iteration_pixels=24,
                        initial_sub_to_final=0))]
    return d, mesh, keep


def _run_main(rank, world, port, outdir, waves=False):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        d, mesh, keep = _c2_shaped()
        seen, mine = [], []

        def integrate(p):
            mine.append(len(p))
            return oracle.integrate(d, p, fast=False, nthreads=1)

        rounds = multirank.sharded_run(mesh, d, integrate, rank, world, dist,
                                       on_round=lambda px, res: seen.append((px.copy(), res.copy())), waves=waves)
        np.savez(os.path.join(outdir, f"run{rank}.npz"), px=np.concatenate([p for p, _ in seen]),
                 res=np.concatenate([r for _, r in seen]), sizes=np.array([len(p) for p, _ in seen]),
                 mine=np.array(mine), rounds=rounds)
        del keep
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("waves", [False, True])
def test_sharded_c2_shaped_run_hands_out_the_single_rank_pixels(oracle_mod, tmp_path, waves):
    """A whole adaptive run (Main.cpp:313-419) over two gloo ranks, each integrating its
    contiguous half of every round with the oracle and gathering before the mesh ends the
    round (Mesh.cpp:1092-1186), must hand out the same pixels in the same order, with the
    same results, as the run on one rank; each rank integrated only its half. With waves
    the ranks split the level waves instead and replay the same rounds."""
    import foort_gb300
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_run_main, args=(world, _free_port(), str(tmp_path), waves), nprocs=world,
                       start_method="spawn")
    d, mesh, keep = _c2_shaped()
    seen = []
    rounds = foort_gb300.run_rounds(mesh, d, lambda p: oracle_mod.integrate(d, p, fast=False),
                                    on_round=lambda px, res: seen.append((px.copy(), res.copy())))
    want_px = np.concatenate([p for p, _ in seen])
    want_res = np.concatenate([r for _, r in seen])
    sizes = [len(p) for p, _ in seen]
    assert rounds >= 3 and sizes[0] == 81, sizes
    for r in range(world):
        f = np.load(tmp_path / f"run{r}.npz")
        assert int(f["rounds"]) == rounds and list(f["sizes"]) == sizes
        for name in abi.PIXEL_DTYPE.names:
            np.testing.assert_array_equal(f["px"][name], want_px[name], err_msg=name)
        for name in abi.RESULT_DTYPE.names:
            np.testing.assert_array_equal(f["res"][name], want_res[name], err_msg=name)
        if waves:
            d2, mesh2, keep2 = _c2_shaped()
            wsizes = []
            foort_gb300.run_rounds(mesh2, d2, lambda p: oracle_mod.integrate(d2, p, fast=False),
                                   on_round=lambda px, res: wsizes.append(len(px)), waves=True)
            assert len(wsizes) < len(sizes) and sum(wsizes) == sum(sizes)
            halves = [multirank.shard_range(n, r, world) for n in wsizes]
        else:
            halves = [multirank.shard_range(n, r, world) for n in sizes]
        assert list(f["mine"]) == [hi - lo for lo, hi in halves]
    del keep


@pytest.mark.parametrize("lookahead", [0, 100000])
@pytest.mark.parametrize("max_pixels", [0, 150])
def test_run_by_waves_matches_the_round_loop(oracle_mod, max_pixels, lookahead):
    """foort_gb300.run_by_waves (the level-wave schedule with any integrator, here the
    oracle) hands out the round loop's pixels and results, round by round, with or without
    a MaxPixels budget that cuts the rounds and with or without lookahead; with the budget
    its waves stop and the rounds integrate the rest."""
    import foort_gb300
    d, mesh, keep = _c2_shaped()
    spec = [(mesh[0][0], dict(mesh[0][1], max_pixels=max_pixels))]
    integ = lambda p: oracle_mod.integrate(d, p, fast=False)  # noqa: E731
    a, b = [], []
    ra = foort_gb300.run_rounds(spec, d, integ, on_round=lambda px, res: a.append((px.copy(), res.copy())))
    rb, calls = foort_gb300.run_by_waves(spec, d, integ, on_round=lambda px, res: b.append((px.copy(), res.copy())),
                                         lookahead=lookahead)
    assert ra == rb == len(a) == len(b) >= 2
    for (pa, xa), (pb, xb) in zip(a, b):
        assert np.array_equal(pa, pb)
        for name in abi.RESULT_DTYPE.names:
            np.testing.assert_array_equal(xa[name], xb[name], err_msg=name)
    if max_pixels:
        assert sum(len(p) for p, _ in a) <= max_pixels
    else:
        assert calls < ra
        if lookahead:  # MaxSubdivide 3: the seed, then one launch for both finer levels
            assert calls == 2
    del keep
