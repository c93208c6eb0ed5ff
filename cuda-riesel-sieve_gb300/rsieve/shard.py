"""p-range sharding across ranks: one contiguous window per rank, no collective.

Primes are independent, so [p0, p1] splits into contiguous windows, one per
rank (GPU or box), and the factor lists concatenate: the merge is a sort of
the per-rank lists.  Only timing and the final gather cross ranks.
"""
from __future__ import annotations

import numpy as np


def shard_range(p0: int, p1: int, rank: int, world: int) -> tuple[int, int]:
    """Rank `rank`'s window [a, b] of [p0, p1] (inclusive); empty if a > b.

    Boundaries are even numbers, so no odd candidate is split or duplicated.
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    width = p1 - p0 + 1
    if width <= 0:
        return p0, p0 - 1
    cut = [p0 + (width * r) // world for r in range(world + 1)]
    cut = [c + (c & 1) if 0 < r < world else c for r, c in enumerate(cut)]  # interior cuts even
    a, b = cut[rank], cut[rank + 1] - 1
    if rank == world - 1:
        b = p1
    return a, b


def merge(parts) -> np.ndarray:
    """Concatenate per-rank factor arrays (fields p, k, n, and b, c when present)
    sorted by (p, k, n, b, c), the order rs_sieve_range returns."""
    parts = [np.asarray(x) for x in parts if len(x)]
    if not parts:
        return np.zeros(0, dtype=[("p", "<u8"), ("k", "<u4"), ("n", "<u4")])
    allf = np.concatenate(parts)
    keys = [allf[f] for f in ("c", "b") if f in allf.dtype.names] + [allf["n"], allf["k"], allf["p"]]
    return allf[np.lexsort(keys)]
