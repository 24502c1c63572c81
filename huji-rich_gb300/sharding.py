"""Sharding of a batch of independent problems across ranks (one GPU each).

The batched form advances independent problems (no face couples two of
them), so N ranks split the problems into N contiguous ranges with about the
same number of cells each and run them with no data-path collective; the
only cross-rank traffic is the timing maximum and the cell total of the
measurement.  Each rank's range keeps the problems' order, so a rank's batch
is the concatenation of its problems exactly as a single-rank batch would
lay them out.
"""
import numpy as np


def problem_shard(cells_per_problem, world, rank):
    """[lo, hi) problem range of `rank` out of `world`: the cut before
    problem p goes to the first rank r whose share r * total / world the
    cumulative cell count before p reaches, so ranges are contiguous, cover
    every problem once and differ in cells by at most one problem's count."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of world {world}")
    counts = np.asarray(cells_per_problem, dtype=np.int64)
    if counts.ndim != 1 or (counts < 0).any():
        raise ValueError("cells_per_problem must be a 1-D array of non-negative counts")
    before = np.concatenate([[0], np.cumsum(counts)])[:-1]   # cells before each problem
    total = int(counts.sum())
    # problem p goes to rank floor(before[p] * world / total), the last rank for
    # trailing empty problems (all to rank 0 when there are no cells)
    owner = (np.minimum((before * world) // total, world - 1) if total > 0
             else np.zeros(len(counts), dtype=np.int64))
    lo = int(np.searchsorted(owner, rank, side="left"))
    hi = int(np.searchsorted(owner, rank, side="right"))
    return lo, hi
