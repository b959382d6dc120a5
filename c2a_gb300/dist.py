"""Process-level replication of CA query batches.

CCD queries are independent, so N processes (one per GPU) each run their own
share of the queries; no data-path collective exists.  The only
communication is host-side: a barrier around timed regions, a max over ranks
of the elapsed time and (optionally) gathering results.
"""
from __future__ import annotations

import os


def env_rank() -> tuple[int, int, int]:
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def shard(n: int, rank: int, world: int) -> slice:
    """Contiguous block of ``n`` queries owned by ``rank`` (sizes differ by at most one)."""
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))
