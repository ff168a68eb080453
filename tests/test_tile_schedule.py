"""The dense operator's tile bookkeeping covers every tile exactly once.

A step's operator tiles are (row block, column chunk) pairs.  Full-width row
blocks have `nchunk` chunks, the row blocks of the last waves `nchunk2`.  The
step before may have streamed a prefix of the full-width tiles in column-major
order (early tiles u -> row block u % nrb_reg, chunk u // nrb_reg); the step
itself then enumerates the rest, row block after row block in its row order
(a permutation of the full-width blocks followed by one of the tail blocks).
This restates the kernel's index arithmetic (tile_geo, tile_index, the own-tile
walk in produce_stage) and checks, over seeded shapes, that early and own tiles
partition the tile set -- the property the schedule-invariance GPU test relies
on (a tile streamed twice or never would change or stall the step).
"""
import numpy as np
import pytest


def tile_index(nrb_big, nchunk, nchunk2, rb, c):
    return rb * nchunk + c if rb < nrb_big else nrb_big * nchunk + (rb - nrb_big) * nchunk2 + c


def tile_geo(nrb_big, nchunk, nchunk2, t):
    T1 = nrb_big * nchunk
    if t < T1:
        return t // nchunk, t % nchunk
    return nrb_big + (t - T1) // nchunk2, (t - T1) % nchunk2


def own_tile(k, order, nrb_reg, nchunk, nchunk2, spec_done):
    """The k-th tile the step streams itself (produce_stage, phase 0)."""
    cfull = spec_done // nrb_reg if nrb_reg else 0
    rem = spec_done % nrb_reg if nrb_reg else 0
    left = k
    for rb in order:
        c0 = cfull + (1 if rb < rem else 0) if rb < nrb_reg else 0
        cnt = (nchunk if rb < nrb_reg else nchunk2) - c0
        if left < cnt:
            return tile_index(nrb_reg, nchunk, nchunk2, rb, c0 + left)
        left -= cnt
    return None


def early_tile(u, nrb_reg, nchunk):
    """The u-th tile streamed ahead by the step before (column-major)."""
    return (u % nrb_reg) * nchunk + u // nrb_reg


@pytest.mark.parametrize("seed", range(40))
def test_early_and_own_tiles_partition_the_step(seed):
    rng = np.random.default_rng(seed)
    nrb = int(rng.integers(1, 40))
    nsmall = int(rng.integers(0, nrb + 1))
    nrb_reg = nrb - nsmall
    nchunk = int(rng.integers(1, 30))
    nchunk2 = int(rng.integers(1, 60))
    ntiles = nrb_reg * nchunk + nsmall * nchunk2
    cs = int(rng.integers(0, nchunk + 1))        # early column chunks allowed
    n_spec = cs * nrb_reg
    spec_done = int(rng.integers(0, n_spec + 1))
    order = list(rng.permutation(nrb_reg)) + [nrb_reg + int(x) for x in rng.permutation(nsmall)]
    if rng.random() < 0.3:
        order = list(range(nrb))
    seen = np.zeros(ntiles, dtype=np.int64)
    for u in range(spec_done):
        t = early_tile(u, nrb_reg, nchunk)
        rb, c = tile_geo(nrb_reg, nchunk, nchunk2, t)
        assert rb < nrb_reg and c < cs
        seen[t] += 1
    for k in range(ntiles - spec_done):
        t = own_tile(k, order, nrb_reg, nchunk, nchunk2, spec_done)
        assert t is not None and 0 <= t < ntiles
        seen[t] += 1
    assert np.all(seen == 1)
    # the tile geometry round-trips
    for t in range(ntiles):
        rb, c = tile_geo(nrb_reg, nchunk, nchunk2, t)
        assert tile_index(nrb_reg, nchunk, nchunk2, rb, c) == t


def test_row_order_puts_flagged_blocks_first_within_each_group():
    """rb_order: flagged (high-velocity) row blocks first, full-width group
    before the tail group, index order inside each part."""
    def rb_order(hot, nrb_reg):
        out = []
        for lo, hi in ((0, nrb_reg), (nrb_reg, len(hot))):
            out += [b for b in range(lo, hi) if hot[b]] + [b for b in range(lo, hi) if not hot[b]]
        return out
    hot = [0, 1, 0, 0, 1, 1, 0, 1]
    assert rb_order(hot, 5) == [1, 4, 0, 2, 3, 5, 7, 6]
    rng = np.random.default_rng(3)
    for _ in range(50):
        n = int(rng.integers(1, 60))
        h = list(rng.integers(0, 2, n))
        k = int(rng.integers(0, n + 1))
        o = rb_order(h, k)
        assert sorted(o) == list(range(n))
        assert all(b < k for b in o[:k])
