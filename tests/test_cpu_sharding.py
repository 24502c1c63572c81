"""Sharding of the batched form across ranks (huji-rich_gb300/sharding.py):
contiguous, balanced problem ranges, and a world-size-2 run over gloo on the
CPU in which each rank advances only its own problems (the oracle stands in
for the GPU kernels here) and the gathered results equal a single-rank run
bit for bit, with no collective on the data path."""
import os
import socket

import numpy as np
import pytest

import oracle
import synthetic
from sharding import problem_shard

SEED, MIN_CELLS, MAX_CELLS, N_PROBLEMS, STEPS = 5, 64, 400, 7, 2


def test_shards_are_contiguous_balanced_and_complete():
    rng = np.random.default_rng(3)
    for _ in range(500):
        n, world = int(rng.integers(0, 30)), int(rng.integers(1, 9))
        counts = rng.integers(0, 500, n) * (rng.random(n) > 0.2)
        ranges = [problem_shard(counts, world, r) for r in range(world)]
        assert ranges[0][0] == 0 and ranges[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
        if counts.sum():
            share = counts.sum() / world
            assert all(abs(counts[lo:hi].sum() - share) <= counts.max() for lo, hi in ranges)
    with pytest.raises(ValueError):
        problem_shard([1, 2], 2, 2)


def advance(p):
    """Problem p of the test batch advanced STEPS steps by the oracle."""
    mesh, cells, gamma = synthetic.riemann_problem(p, SEED, MIN_CELLS, MAX_CELLS)
    ext = oracle.init_extensives(mesh, cells, gamma)
    c, e, dts = oracle.run(mesh, cells, ext, np.zeros((mesh.n_faces, 2)), gamma, STEPS)
    return mesh.n_cells, c, e, dts


def rank_main(rank, world, port, queue):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        counts = [synthetic.riemann_problem(p, SEED, MIN_CELLS, MAX_CELLS)[0].n_cells for p in range(N_PROBLEMS)]
        lo, hi = problem_shard(counts, world, rank)
        mine = {p: advance(p) for p in range(lo, hi)}
        # the measurement's only cross-rank traffic: the cell total
        total = torch.tensor([sum(r[0] for r in mine.values())], dtype=torch.int64)
        dist.all_reduce(total)
        gathered = [None] * world
        dist.all_gather_object(gathered, {p: r[1:] for p, r in mine.items()})
        if rank == 0:
            queue.put((int(total.item()), {p: r for part in gathered for p, r in part.items()}, (lo, hi)))
    finally:
        dist.destroy_process_group()


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_over_gloo_match_one_rank():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        total, results, first_range = queue.get(timeout=240)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    assert 0 < first_range[1] < N_PROBLEMS           # both ranks hold problems
    serial = {p: advance(p) for p in range(N_PROBLEMS)}
    assert total == sum(r[0] for r in serial.values())
    assert sorted(results) == list(range(N_PROBLEMS))
    for p, (c, e, dts) in results.items():
        assert np.array_equal(c, serial[p][1]) and np.array_equal(e, serial[p][2])
        assert np.array_equal(dts, serial[p][3])


def test_shard_batches_are_slices_of_the_full_batch():
    """A rank builds only its problems: the cell counts come without the
    meshes, and a range's batch is the full batch's problems in order."""
    full = synthetic.riemann_batch(N_PROBLEMS, SEED, MIN_CELLS, MAX_CELLS)
    counts = [synthetic.riemann_problem_cells(p, SEED, MIN_CELLS, MAX_CELLS) for p in range(N_PROBLEMS)]
    assert counts == [m.n_cells for m in full[4]]
    lo, hi = problem_shard(counts, 2, 1)
    part = synthetic.riemann_batch_range(range(lo, hi), SEED, MIN_CELLS, MAX_CELLS)
    off = full[1]
    assert np.array_equal(part[3], full[3][off[lo]:off[hi]])
    assert np.array_equal(part[2], full[2][lo:hi])
    assert np.array_equal(part[1], off[lo:hi + 1] - off[lo])
