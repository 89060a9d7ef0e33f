"""Splitting one sampling job's shots over several processes (one per GPU).

Shots are independent and every random draw is keyed by (seed, event,
global shot word), so rank r simulating shots [first, first + count) of a
job -- a state with ``set_shot_offset(first)`` -- produces exactly the
records a single state holding all shots would produce for that range.  No
data-path collective is needed; ``gather_records`` concatenates the ranks'
record words on the host side (torch.distributed, any backend).
"""
from __future__ import annotations

from typing import Tuple

import numpy as np

WORD = 64  # shots per word; shard boundaries stay word-aligned


def shard_range(total_shots: int, world: int, rank: int) -> Tuple[int, int]:
    """(first_shot, count) of rank's share: contiguous, word-aligned, sizes
    differing by at most one word, covering [0, total_shots) exactly."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    if total_shots < 0:
        raise ValueError("negative shot count")
    words = (total_shots + WORD - 1) // WORD
    base, extra = divmod(words, world)
    first_w = rank * base + min(rank, extra)
    n_w = base + (1 if rank < extra else 0)
    first = first_w * WORD
    count = max(0, min(total_shots, (first_w + n_w) * WORD) - first)
    return first, count


def weak_range(shots_per_rank: int, rank: int) -> Tuple[int, int]:
    """Weak scaling: rank r holds shots [r*S, (r+1)*S) of a world*S-shot job
    (S a multiple of 64)."""
    if shots_per_rank % WORD:
        raise ValueError("shots per rank must be a multiple of 64")
    return rank * shots_per_rank, shots_per_rank


def records_to_bits(words: np.ndarray, shots: int) -> np.ndarray:
    """[nm, w] uint64 record words -> [nm, shots] uint8 (bit s of word k =
    shot 64k + s)."""
    b = np.unpackbits(np.ascontiguousarray(words).view(np.uint8), axis=1, bitorder="little")
    return b[:, :shots]


def gather_records(bits: np.ndarray, group=None) -> np.ndarray:
    """Concatenate every rank's [nm, count] record bits along the shot axis,
    in rank order (host-side gather; counts may differ by rank)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    t = torch.from_numpy(np.ascontiguousarray(bits, dtype=np.uint8))
    n = torch.tensor([t.shape[1]], dtype=torch.int64)
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(counts, n, group=group)
    width = int(max(c.item() for c in counts))
    pad = torch.zeros((t.shape[0], width), dtype=torch.uint8)
    pad[:, : t.shape[1]] = t
    parts = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return np.concatenate([p[:, : int(c.item())].numpy() for p, c in zip(parts, counts)], axis=1)
