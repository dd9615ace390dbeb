"""Splitting the rotation search across ranks (one process per GPU).

Rotations are independent, so rank k searches a contiguous block of the
rotation grid and keeps its per-rotation (score, translation); there is no
exchange inside the search.  ``search_sharded`` (used by search_map_fft,
search_map_fft_prob and Aligner.align_many when given a process group)
gathers the blocks' results in rotation order.  Two small host exchanges
rebuild exactly what a single process computes:

* top-N: every rank contributes its local stable top-N as
  (score, global rotation index); the merge orders by score descending, then
  rotation index ascending -- the order of Python's stable
  ``sorted(..., reverse=True)`` over the full grid (VESPER_1_prob_new.py:664);
* prob-mode statistics (VESPER_1_prob_new.py:920-926): the per-rotation scores
  are gathered in rotation order so mean/std are computed over the same array,
  with the same numpy reductions, as in one process.
"""
from __future__ import annotations

import numpy as np


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous block [lo, hi) of n items for ``rank`` of ``world``."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def local_topn(scores: np.ndarray, n: int, offset: int = 0):
    """Stable top-n of a shard: (scores, global indices)."""
    order = sorted(range(len(scores)), key=lambda i: float(scores[i]), reverse=True)[:n]
    return np.asarray([scores[i] for i in order], np.float64), np.asarray([offset + i for i in order], np.int64)


def merge_topn(parts, n: int):
    """Merge per-rank (scores, global indices) into the global stable top-n."""
    sc = np.concatenate([np.asarray(p[0], np.float64) for p in parts]) if parts else np.zeros(0)
    ix = np.concatenate([np.asarray(p[1], np.int64) for p in parts]) if parts else np.zeros(0, np.int64)
    order = np.lexsort((ix, -sc))[:n]
    return sc[order], ix[order]


def gather_topn(scores: np.ndarray, n: int, offset: int, group=None):
    """All ranks: local stable top-n, all-gathered and merged (torch.distributed)."""
    import torch.distributed as dist
    mine = local_topn(scores, n, offset)
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, mine, group=group)
    return merge_topn(parts, n)


def gather_scores(scores: np.ndarray, group=None) -> np.ndarray:
    """All ranks: the per-rotation scores of every shard, in rotation order."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, np.asarray(scores), group=group)
    return np.concatenate(parts)


def search_sharded(search_block, nrot: int, group=None):
    """Split ``nrot`` rotations over the ranks of ``group``: this rank runs
    ``search_block(lo, hi)`` on its block [lo, hi) (returning host arrays
    scores [hi-lo][nscore], lin [hi-lo][nscore]), then every rank receives
    all ranks' results in rotation order -- the arrays one process would have
    computed, so top-N, statistics and refinement proceed unchanged."""
    import torch.distributed as dist
    lo, hi = shard_range(nrot, dist.get_rank(group), dist.get_world_size(group))
    sc, ln = search_block(lo, hi)
    return gather_scores(sc, group), gather_scores(ln, group)


def prob_stats(vscores_scaled: np.ndarray, pscores_scaled: np.ndarray):
    """(vstd, vave, pstd, pave) exactly as the single-process pass 1."""
    return (np.std(vscores_scaled), np.mean(vscores_scaled), np.std(pscores_scaled), np.mean(pscores_scaled))
