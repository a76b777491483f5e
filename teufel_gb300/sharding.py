"""Sharding an observer's work across ranks: by pixels or by particles.

Pixels are independent observation points, so an observer splits into
contiguous pixel blocks with no exchange during the integration; the blocks
are gathered in rank order to rebuild the [pixel][sample][6] buffer.  (The
reference distributes particles instead and sums the per-rank traces with
MPI_Reduce, src/teufel_hybrid.cpp:746-754; pixel blocks need no reduction and
give the same traces on any number of ranks.)  rank_batches splits a bunch
by particles instead, for ranks that each integrate their own batches onto
the whole observer.
"""
from __future__ import annotations

import numpy as np


def shard(n: int, rank: int, world: int):
    """[lo, hi) of the pixels rank `rank` of `world` integrates."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return n * rank // world, n * (rank + 1) // world


def gather_traces(local: np.ndarray, n_pix: int, rank: int, world: int, dist=None):
    """Assemble the full trace buffer on every rank from the per-rank blocks
    (torch.distributed all_gather of equally padded blocks)."""
    if world == 1 or dist is None:
        return local
    import torch
    lo, hi = shard(n_pix, rank, world)
    width = max(shard(n_pix, r, world)[1] - shard(n_pix, r, world)[0] for r in range(world))
    pad = np.zeros((width,) + local.shape[1:], dtype=local.dtype)
    pad[:hi - lo] = local
    t = torch.from_numpy(pad)
    parts = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(parts, t)
    out = np.empty((n_pix,) + local.shape[1:], dtype=local.dtype)
    for r in range(world):
        a, b = shard(n_pix, r, world)
        out[a:b] = parts[r].numpy()[:b - a]
    return out


def rank_batches(rank: int, world: int, n_batches: int, batch: int, n_particles: int):
    """First particle of each of the n_batches batches of `batch` particles
    that rank `rank` of `world` integrates when the ranks share a bunch of
    n_particles by particles: rank r takes batches r*n_batches to
    r*n_batches + n_batches - 1, wrapping around the bunch, so the ranks'
    particles are disjoint while world * n_batches * batch <= n_particles.
    Each rank integrates its batches onto the whole observer with no
    exchange; the per-rank traces add up to the bunch's (the reference sums
    them with MPI_Reduce, src/teufel_hybrid.cpp:746-754)."""
    if world < 1 or not 0 <= rank < world or n_batches < 0 or batch < 1 or n_particles < 1:
        raise ValueError("bad rank/world/batch")
    return [((rank * n_batches + b) * batch) % n_particles for b in range(n_batches)]
