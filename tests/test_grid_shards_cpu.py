"""CPU: the grid over several ranks.  The (J, sector) points are independent
eigensolves, so N ranks split the J points (no exchange while solving) and
gather only the eigenvalues.  The shares, the gather, the sharded solve
driver (with the device solve replaced by a fake) and the bench's
max-over-ranks timing run here as two gloo ranks."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _package():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g

    return g.load_package()


def _bench():
    sys.path.insert(0, ROOT)
    import bench

    return bench


def test_shard_indices_partition(pkg):
    for n in [0, 1, 5, 64, 65, 320]:
        for world in [1, 2, 3, 8]:
            parts = [pkg.shard_indices(n, world, r) for r in range(world)]
            allp = np.concatenate(parts)
            assert np.array_equal(np.sort(allp), np.arange(n))
            assert len(allp) == n  # disjoint
            sizes = [len(x) for x in parts]
            assert max(sizes) - min(sizes) <= 1
    for bad in [(4, 0, 0), (4, 2, 2), (4, 2, -1), (-1, 1, 0)]:
        with pytest.raises(ValueError):
            pkg.shard_indices(*bad)


def test_bench_j_grid_shards(pkg):
    bench = _bench()
    # one rank: exactly the 64-point grid of the one-GPU line
    assert np.array_equal(bench.j_shard(pkg, 1, 0), bench.JS)
    # two ranks: 64 points each, together the 128-point grid on (0, 0.3]
    a, b = bench.j_shard(pkg, 2, 0), bench.j_shard(pkg, 2, 1)
    assert len(a) == len(b) == bench.NJ
    full = np.sort(np.concatenate([a, b]))
    np.testing.assert_allclose(full, 0.3 * (np.arange(2 * bench.NJ) + 1) / (2 * bench.NJ), rtol=0, atol=0)
    assert a.min() < 0.01 and b.max() == pytest.approx(0.3)


def test_gather_without_process_group(pkg):
    x = np.arange(12.0).reshape(4, 3)
    assert np.array_equal(pkg.gather_grid(x, 4), x)
    with pytest.raises(ValueError):
        pkg.gather_grid(x, 5)


def _fake_sectors(hams, J, U, mu, nev=10, **opt):
    # deterministic stand-in for the device solve: value = f(sector, J, level)
    J = np.asarray(J, np.float64)
    nh = len(hams)
    ev = np.array([[[100.0 * h + J[s] + 0.001 * k for k in range(nev)] for s in range(len(J))]
                   for h in range(nh)])
    nc = np.full((nh, len(J)), nev, np.int32)
    return ev, np.zeros_like(ev), nc, None


def _rank_main(rank, world, port, q):
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                          WORLD_SIZE=str(world))
        import torch.distributed as dist

        dist.init_process_group("gloo", rank=rank, world_size=world)
        pkg = _package()
        bench = _bench()
        n = 7  # uneven shares: 4 + 3
        mine = pkg.shard_indices(n, world, rank)
        local = np.stack([np.array([10.0 * i, 10.0 * i + 1.0]) for i in mine])
        full = pkg.gather_grid(local, n)
        want = np.stack([np.array([10.0 * i, 10.0 * i + 1.0]) for i in range(n)])
        ok_gather = np.array_equal(full, want)
        bad_share = False
        try:
            pkg.gather_grid(local[:0], n)
        except ValueError:
            bad_share = True
        # the sharded multi-sector driver with the device solve replaced
        pkg.eigsh_sectors = _fake_sectors
        J = 0.3 * (np.arange(9) + 1) / 9
        ev, nc, _ = pkg.eigsh_sectors_sharded([None, None, None], J, 1.0, 0.0, nev=4)
        ev_want, _, nc_want, _ = _fake_sectors([None, None, None], J, 1.0, 0.0, nev=4)
        ok_sharded = ev.shape == (3, 9, 4) and np.array_equal(ev, ev_want) and np.array_equal(nc, nc_want)
        # the bench's timing: max over ranks
        t = bench.max_over_ranks(0.5 + rank, world, "cpu")
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, bool(ok_gather), bool(bad_share), bool(ok_sharded), t))
    except Exception as e:  # reported to the parent
        q.put((rank, "error", repr(e)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_shard_and_gather():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = {}
    try:
        for _ in range(world):
            r = q.get(timeout=240)
            results[r[0]] = r
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    for r in range(world):
        rec = results[r]
        assert rec[1] != "error", rec
        _, ok_gather, bad_share, ok_sharded, t = rec
        assert ok_gather and bad_share and ok_sharded
        assert t == pytest.approx(1.5)
