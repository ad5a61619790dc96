"""The joint batch's item walk, restated on the host (no GPU).

A joint batch lists the scenes that take part in a phase with a prefix of
their item counts (batch.h, bat_build_list), and every CTA finds an item's
scene with a 32-way warp search of that prefix (bat_find): each round, lane k
tests position lo + k * step, and the highest lane whose prefix entry is <= t
narrows the range.  These tests run the same search in numpy and check that
every item of every listed scene is found exactly once, with its block index
inside the scene's count, for batch sizes around the 32-lane and 1024-scene
boundaries and for scenes that contribute no items to a phase.
"""
import numpy as np
import pytest


def build_prefix(counts):
    """bat_build_list: exclusive prefix over the listed scenes, then the total."""
    pre = np.zeros(len(counts) + 1, dtype=np.int64)
    pre[1:] = np.cumsum(counts)
    return pre


def warp_find(pre, nact, t):
    """bat_find: the last listed scene j with pre[j] <= t, by 32-way rounds."""
    lo, hi, rounds = 0, nact, 0
    while hi - lo > 1:
        step = (hi - lo + 31) >> 5
        j = lo + np.arange(32) * step
        ok = (j < hi) & (pre[np.minimum(j, len(pre) - 1)] <= t)
        assert ok[0], "lane 0 always holds"
        last = int(np.nonzero(ok)[0].max())
        assert np.all(ok[: last + 1]) and not np.any(ok[last + 1:]), "the ballot is a prefix of lanes"
        lo += last * step
        hi = min(hi, lo + step)
        rounds += 1
    return lo, t - int(pre[lo]), rounds


@pytest.mark.parametrize("nact", [1, 2, 31, 32, 33, 255, 256, 257, 1023, 1024, 1025])
def test_every_item_found_once(nact):
    rng = np.random.default_rng(nact)
    counts = rng.integers(0, 40, size=nact)
    counts[rng.random(nact) < 0.3] = 0      # scenes with no items of this kind
    if counts.sum() == 0:
        counts[-1] = 3
    pre = build_prefix(counts)
    total = int(pre[-1])
    seen = np.zeros((nact, int(counts.max()) + 1), dtype=np.int64)
    max_rounds = 0
    for t in range(total):
        j, b, rounds = warp_find(pre, nact, t)
        max_rounds = max(max_rounds, rounds)
        assert 0 <= j < nact and counts[j] > 0, (t, j)
        assert 0 <= b < counts[j], (t, j, b)
        seen[j, b] += 1
    for j in range(nact):
        assert np.all(seen[j, : counts[j]] == 1) and np.all(seen[j, counts[j]:] == 0), j
    # two rounds cover up to 1024 listed scenes, three beyond
    assert max_rounds <= (1 if nact <= 32 else 2 if nact <= 1024 else 3)


def test_grid_stride_covers_items_once():
    """Persistent CTAs take items blockIdx.x, blockIdx.x + gridDim.x, ...:
    every item once, for item totals below, at and above the grid size."""
    for grid in (1, 7, 1216):
        for total in (0, 1, grid - 1, grid, grid + 1, 5 * grid + 3):
            hits = np.zeros(max(total, 1), dtype=np.int64)
            for cta in range(grid):
                for t in range(cta, total, grid):
                    hits[t] += 1
            assert np.all(hits[:total] == 1), (grid, total)


def test_chunks_and_block_groups_cover_the_level():
    """Chunk items (chunk_of) cover every segment once with the warps' stride
    of 8; block-group items (group_end) cover every busy block once."""
    for nseg in (0, 1, 7, 8, 63, 64, 65, 1000):
        for cs in (16, 32, 64):
            items = max(1, (nseg + cs - 1) // cs)
            hits = np.zeros(max(nseg, 1), dtype=np.int64)
            for c in range(items):
                end = min(nseg, (c + 1) * cs)
                for w in range(8):
                    for s in range(c * cs + w, end, 8):
                        hits[s] += 1
            assert np.all(hits[:nseg] == 1), (nseg, cs)
    for busy in (1, 2, 7, 8, 9, 608):
        for bg in (4, 8, 16, 32):
            items = (busy + bg - 1) // bg
            blocks = [b for it in range(items) for b in range(it * bg, min(busy, (it + 1) * bg))]
            assert blocks == list(range(busy)), (busy, bg)
