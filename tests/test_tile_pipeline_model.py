"""The batched sweep's counted tile hand-off, modelled on the CPU.

In sa_batch_tile_kernel (sa_kernels.cuh, batch_tile_item_impl) the W warps of
a CTA walk the same sequence of row tiles g = 0, 1, ..., total - 1 through NB
shared-memory buffers (tile g in buffer g mod NB) without a CTA-wide barrier:
the first NB copies are issued up front; a warp waits for its buffer's copy
(an mbarrier phase, tested by parity), uses the tile, then counts itself done
with the buffer; the warp whose count completes the buffer resets the count
and issues the copy of tile g + NB into it. This model runs that protocol
under random interleavings of the warps and random copy latencies and checks
that every warp reads the right tile, that no copy overwrites a tile some
warp still needs, that a parity wait can never confuse two phases (a buffer
is never more than one phase ahead of a waiting warp), and that every run
finishes.
"""
from __future__ import annotations

import random

import pytest


def run_protocol(W: int, NB: int, total: int, seed: int) -> None:
    rng = random.Random(seed)
    content = [None] * NB          # tile held by each buffer once its copy lands
    landed = [0] * NB              # completed phases (copies landed) per buffer
    done = [0] * NB                # warps done with the buffer's current tile
    in_flight = []                 # (buffer, tile) copies issued, not landed
    users = [set() for _ in range(NB)]   # warps still to use the buffer's current tile
    nxt = [0] * W                  # next tile of each warp
    uses = [[0] * NB for _ in range(W)]  # buffer uses completed by each warp

    def issue(b: int, g: int) -> None:
        assert not users[b], f"tile {g} issued into buffer {b} while warps {users[b]} still need it"
        in_flight.append((b, g))

    for g in range(min(NB, total)):
        issue(g % NB, g)
    for b in range(NB):
        users[b] = set(range(W)) if b < total else set()

    steps = 0
    while any(n < total for n in nxt):
        steps += 1
        assert steps < 100 * W * total + 1000, "the protocol stalled"
        # Either a copy lands or a warp that can move does.
        movers = [w for w in range(W) if nxt[w] < total
                  and landed[nxt[w] % NB] > uses[w][nxt[w] % NB]]
        if in_flight and (not movers or rng.random() < 0.3):
            b, g = in_flight.pop(rng.randrange(len(in_flight)))
            content[b] = g
            landed[b] += 1
            continue
        assert movers, "no warp can move and no copy is in flight: deadlock"
        w = rng.choice(movers)
        g = nxt[w]
        b = g % NB
        # The parity wait: the buffer is at most one phase past this use.
        assert landed[b] - uses[w][b] == 1, "a parity wait could confuse two phases"
        assert content[b] == g, f"warp {w} read tile {content[b]} for tile {g}"
        uses[w][b] += 1
        users[b].discard(w)
        nxt[w] += 1
        done[b] += 1
        if done[b] == W:           # the last warp done with this tile refills the buffer
            done[b] = 0
            if g + NB < total:
                issue(b, g + NB)
                users[b] = set(range(W))
    assert not in_flight and all(d == 0 for d in done)


@pytest.mark.parametrize("W,NB", [(1, 2), (4, 2), (4, 3), (16, 3), (16, 2)])
def test_counted_hand_off_under_random_interleavings(W, NB):
    for seed in range(40):
        for total in (1, 2, NB, NB + 1, 64, 129):
            run_protocol(W, NB, total, seed)
