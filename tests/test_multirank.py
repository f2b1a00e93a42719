"""Multi-rank host logic on CPU (gloo, world size 2): the kernel grid is sharded
tile by tile with no data exchange; only timings are max-reduced."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n1, n2, b, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    from nt_gb300.batching import rank_tiles, tile_grid
    tiles = tile_grid(n1, n2, b)
    mine = rank_tiles(tiles, world, rank)
    # the work of a rank is its tiles' entries; no data-path collective
    covered = torch.zeros(n1, n2, dtype=torch.int32)
    for r0, rn, c0, cn in mine:
        covered[r0:r0 + rn, c0:c0 + cn] += 1
    dist.all_reduce(covered)  # verification only
    t = torch.tensor([float(10 + rank)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    entries = torch.tensor([sum(rn * cn for _, rn, _, cn in mine)])
    dist.all_reduce(entries)
    q.put((rank, bool((covered == 1).all()), float(t.item()), int(entries.item())))
    dist.destroy_process_group()


@pytest.mark.parametrize('n1,n2,b', [(2000, 2000, 100), (5000, 5000, 128), (250, 96, 40)])
def test_tile_partition_world2(n1, n2, b):
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n1, n2, b, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ok, tmax, entries in out:
        assert ok, 'every entry of the grid is computed by exactly one rank'
        assert tmax == 11.0
        assert entries == n1 * n2


def test_rank_tiles_wraps_for_steps():
    from nt_gb300.batching import rank_tiles, tile_grid
    tiles = tile_grid(300, 300, 100)
    assert len(tiles) == 9
    assert rank_tiles(tiles, 4, 1, steps=5) == [tiles[1], tiles[5], tiles[0], tiles[4], tiles[8]]
    assert sorted(rank_tiles(tiles, 4, 0) + rank_tiles(tiles, 4, 1) + rank_tiles(tiles, 4, 2) +
                  rank_tiles(tiles, 4, 3)) == sorted(tiles)


@pytest.mark.parametrize('n,b,world', [(2000, 100, 2), (2000, 100, 8), (250, 40, 4), (7, 100, 3)])
def test_rank_rows_cover_every_row_once(n, b, world):
    """The end-to-end job under torchrun: each rank's contiguous block of tile rows."""
    from nt_gb300.batching import rank_rows
    rows = [rank_rows(n, b, world, r) for r in range(world)]
    assert rows[0][0] == 0 and rows[-1][1] == n
    for (a0, a1), (b0, b1) in zip(rows, rows[1:]):
        assert a1 == b0 and a0 <= a1
    for a0, a1 in rows:
        assert a0 % b == 0 or a0 == n
