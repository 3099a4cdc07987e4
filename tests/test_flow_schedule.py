"""The ordering rule of the dataflow sweep (k_sweep_dep), checked by
simulation on the CPU.  A tile of half-sweep j on slab b writes colour j % 2
on slab b and reads the other colour on slabs b-1 (its last plane), b and
b+1 (its first plane); it may start once half-sweep j-1 has finished slabs
b-1, b and b+1.  Tickets go out in the kernel's order (half-sweep j, then its
slabs starting at slab j mod S, then the tiles of a slab) to at most M blocks
at a time, each of which waits for its tile's dependencies and then runs; a
random block finishes at each step.  Checked: every schedule finishes (no
deadlock, whatever M), and no two tiles that run at the same time touch the
same spins with at least one of them writing -- so every tile reads what the
reference's half-sweep j reads.  The GPU parity tests check the kernel
itself."""
import random

import pytest


def _tickets(nhalf, nslab, tiles):
    """(j, b, t) in ticket order: half-sweep, then slabs from slab j, then tiles"""
    return [(j, (i + j) % nslab, t) for j in range(nhalf) for i in range(nslab)
            for t in range(tiles)]


def _touch(j, b, nslab):
    """(writes, reads) as sets of (colour, slab)"""
    own, oth = j % 2, 1 - j % 2
    return {(own, b)}, {(oth, (b - 1) % nslab), (oth, b), (oth, (b + 1) % nslab)}


def _simulate(nhalf, nslab, tiles, blocks, rng):
    order = _tickets(nhalf, nslab, tiles)
    done = {}  # (j, b) -> finished tiles
    next_ticket, waiting, running, steps = 0, [], [], 0
    while len(done) < nhalf * nslab or waiting or running or next_ticket < len(order):
        steps += 1
        assert steps < 100000, "no progress: a deadlock"
        # blocks take tickets in order while there is room
        while next_ticket < len(order) and len(waiting) + len(running) < blocks:
            waiting.append(order[next_ticket])
            next_ticket += 1
        # a waiting block starts once half-sweep j-1 has finished its three slabs
        for tile in list(waiting):
            j, b, _ = tile
            ready = j == 0 or all(done.get((j - 1, (b + d) % nslab), 0) == tiles
                                  for d in (-1, 0, 1))
            if ready:
                waiting.remove(tile)
                running.append(tile)
        # no two running tiles conflict
        for x in range(len(running)):
            for y in range(x + 1, len(running)):
                (j1, b1, _), (j2, b2, _) = running[x], running[y]
                if j1 == j2:
                    continue
                w1, r1 = _touch(j1, b1, nslab)
                w2, r2 = _touch(j2, b2, nslab)
                assert not (w1 & r2 or w2 & r1 or w1 & w2), (running[x], running[y])
        if not running:
            assert waiting or next_ticket < len(order) or len(done) == nhalf * nslab
            continue
        fin = running.pop(rng.randrange(len(running)))
        done[(fin[0], fin[1])] = done.get((fin[0], fin[1]), 0) + 1
    return steps


@pytest.mark.parametrize("nhalf", [2, 4, 12])
@pytest.mark.parametrize("nslab", [1, 2, 3, 5, 8, 20])
def test_dataflow_order_finishes_without_conflicts(nhalf, nslab):
    rng = random.Random(nhalf * 100 + nslab)
    for tiles in (1, 3):
        for blocks in (1, 2, 7, 64):
            _simulate(nhalf, nslab, tiles, blocks, rng)


def test_each_tile_gets_exactly_one_ticket():
    order = _tickets(12, 20, 27)
    assert len(order) == len(set(order)) == 12 * 20 * 27
    # the slabs of half-sweep j start at slab j: its first slab's dependencies
    # (slabs j-1, j, j+1 of half-sweep j-1) went out near the start of j-1
    first = {j: order[j * 20 * 27][1] for j in range(12)}
    assert all(first[j] == j % 20 for j in range(12))
