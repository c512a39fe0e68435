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


# --- The failure path -------------------------------------------------------
#
# A warp's wait is bounded (a poll limit); when it runs out the warp sets the
# CTA's fail flag, and every later wait returns false at once. Warps that
# failed keep walking the tiles without waiting (their `phase` bits still
# flip) so that the done counts stay consistent; no refill is issued once the
# flag is set. At the end the CTA decides uniformly, and one thread lets the
# copies still in flight land (bounded) before the CTA returns. mbarrier
# parity waits are modelled as the hardware answers them: waiting on parity
# P succeeds when the barrier's completed-phase count has the other parity.


def _parity_done(landed: int, parity: int) -> bool:
    return (landed & 1) != parity


def run_protocol_with_failures(W: int, NB: int, total: int, seed: int, limit: int,
                               drain: str = "issued") -> dict:
    """One run of the counted hand-off in which some copies are slow (they
    land only after the first timeout) or stuck (they never land). Returns
    what the end-of-item drain saw per buffer."""
    rng = random.Random(seed)
    content = [None] * NB
    landed = [0] * NB
    issued = [0] * NB
    done = [0] * NB
    in_flight = {}                 # buffer -> (tile, kind)
    fail = False
    nxt = [0] * W
    failed = [False] * W
    polls = [0] * W
    phase = [[0] * NB for _ in range(W)]

    def issue(b: int, g: int) -> None:
        assert b not in in_flight, "two copies in flight in one buffer"
        issued[b] += 1
        r = rng.random()
        kind = "stuck" if r < 0.04 else "slow" if r < 0.12 else "normal"
        in_flight[b] = (g, kind)

    def land(b: int) -> None:
        g, _ = in_flight.pop(b)
        content[b] = g
        landed[b] += 1

    def landable() -> list:
        return [b for b, (_, k) in in_flight.items() if k == "normal" or (k == "slow" and fail)]

    for g in range(min(NB, total)):
        issue(g % NB, g)

    steps = 0
    while any(n < total for n in nxt):
        steps += 1
        assert steps < 200 * W * (total + limit) + 1000, "the protocol stalled"
        can = landable()
        if can and rng.random() < 0.3:
            land(rng.choice(can))
            continue
        w = rng.choice([v for v in range(W) if nxt[v] < total])
        g = nxt[w]
        b = g % NB
        if not failed[w]:
            # One poll of tile_wait.
            if _parity_done(landed[b], phase[w][b]):
                ok = True
            elif fail:
                ok = False
            else:
                polls[w] += 1
                if polls[w] < limit:
                    continue
                fail = True
                ok = False
            polls[w] = 0
        else:
            ok = False
        phase[w][b] ^= 1
        failed[w] = not ok
        if ok:
            assert content[b] == g, f"warp {w} read tile {content[b]} for tile {g}"
        done[b] += 1
        if done[b] == W:
            done[b] = 0
            if g + NB < total and not fail:
                issue(b, g + NB)
        nxt[w] += 1
    assert all(d == 0 for d in done)

    # The uniform decision and the drain by thread 0 (warp 0).
    report = {"failed": any(failed), "missed": []}
    if not any(failed):
        assert not in_flight, "a successful item left a copy in flight"
        return report
    for b in range(NB):
        if drain == "issued":
            if issued[b] == 0:
                continue
            parity = (issued[b] - 1) & 1
        else:                      # the warps' own phase bits
            parity = phase[0][b]
        returned = False
        for _ in range(limit):
            if _parity_done(landed[b], parity):
                returned = True
                break
            can = landable()
            if b in can and rng.random() < 0.5:
                land(b)
        if returned and b in in_flight:
            report["missed"].append(b)
    return report


@pytest.mark.parametrize("W,NB", [(1, 2), (4, 3), (16, 3), (16, 2)])
def test_counted_hand_off_failure_path_drains_every_copy(W, NB):
    """With the drain on the phase of each buffer's last issued copy, the
    CTA never returns while a copy into its shared memory is in flight
    (unless that copy is stuck and the bounded wait gave up on it), every
    run ends, and no buffer ever has two copies in flight."""
    failures = 0
    for seed in range(300):
        for total in (1, NB, NB + 1, 40):
            r = run_protocol_with_failures(W, NB, total, seed, limit=6)
            failures += r["failed"]
            assert not r["missed"], (seed, total, r)
    assert failures > 50, "the runs did not reach the failure path"


def test_phase_bits_alone_would_miss_a_copy_in_flight():
    """The warps' phase bits also count the tiles skipped after a failure,
    so a drain on them can return while the last copy is still landing; the
    kernel drains on the issued-copy count instead."""
    missed = 0
    for seed in range(400):
        r = run_protocol_with_failures(4, 3, 40, seed, limit=6, drain="phase")
        missed += bool(r["missed"])
    assert missed > 0


def run_barrier_form_with_failures(W: int, total: int, seed: int, limit: int) -> dict:
    """The dense kernel's form: two buffers, tile g in buffer g & 1, every
    warp waits (bounded) for tile g, a CTA-wide OR decides, thread 0 refills
    the buffer with tile g + 2. On a failure the drain waits on both
    buffers: on tile g's phase in buffer g & 1 (its parity bit already
    flipped, so flipped back) and on the other buffer's next phase, which is
    tile g + 1's when the run has one (else that wait just runs out)."""
    rng = random.Random(seed)
    landed = [0, 0]
    content = [None, None]
    in_flight = {}
    parity = [0, 0]                # thread 0's parity bits (all warps alike)

    def issue(g: int) -> None:
        b = g & 1
        assert b not in in_flight
        r = rng.random()
        in_flight[b] = (g, "stuck" if r < 0.03 else "slow" if r < 0.1 else "normal")

    def land(b: int) -> None:
        g, _ = in_flight.pop(b)
        content[b] = g
        landed[b] += 1

    for g in range(min(2, total)):
        issue(g)
    for g in range(total):
        h = g & 1
        oks = []
        for w in range(W):
            ok = False
            for _ in range(limit):
                if _parity_done(landed[h], parity[h]):
                    ok = True
                    break
                if h in in_flight and in_flight[h][1] == "normal" and rng.random() < 0.5:
                    land(h)
            if ok:
                assert content[h] == g
            oks.append(ok)
        parity[h] ^= 1
        if not all(oks):
            waits = [(b, parity[b] ^ (1 if b == h else 0)) for b in (0, 1)]
            missed = []
            for b, p in waits:
                returned = False
                for _ in range(limit):
                    if _parity_done(landed[b], p):
                        returned = True
                        break
                    if b in in_flight and in_flight[b][1] != "stuck" and rng.random() < 0.5:
                        land(b)
                if returned and b in in_flight:
                    missed.append(b)
            return {"failed": True, "missed": missed, "left": [b for b in in_flight if in_flight[b][1] != "stuck"]}
        if g + 2 < total:
            issue(g + 2)
    assert not in_flight
    return {"failed": False, "missed": [], "left": []}


def test_barrier_form_failure_path_drains_every_copy():
    failures = 0
    for seed in range(600):
        for total in (1, 2, 3, 40):
            r = run_barrier_form_with_failures(4, total, seed, limit=6)
            failures += r["failed"]
            assert not r["missed"], (seed, total, r)
    assert failures > 50


def run_ring_with_failures(S: int, n: int, seed: int, limit: int) -> dict:
    """The tensor-core initial-field product's ring (sa_init.cu,
    init_gemm_kernel): a copy thread loads chunk i into stage i mod S once
    the MMAs released the stage's previous chunk (`empty`), an MMA thread
    waits for each chunk (`full`), issues its MMAs and releases the stage
    when they complete. Both waits are bounded; a thread whose wait runs out
    stops. The copy thread then waits (bounded) on each stage's last copy,
    the phase (last // S) of stage s with last = s + ((issued - 1 - s) // S) * S."""
    rng = random.Random(seed)
    full = [0] * S                 # landed copies per stage
    empty = [0] * S                # released stages (MMAs completed)
    copies = {}                    # stage -> (chunk, kind)
    mmas = {}                      # stage -> (chunk, kind)
    content = [None] * S
    prod = {"i": 0, "polls": 0, "state": "run", "issued": 0, "drain_s": 0, "missed": []}
    cons = {"i": 0, "polls": 0, "state": "run"}

    def kind() -> str:
        r = rng.random()
        return "stuck" if r < 0.02 else "slow" if r < 0.08 else "normal"

    def landable(d: dict, late: bool) -> list:
        return [s for s, (_, k) in d.items() if k == "normal" or (k == "slow" and late)]

    steps = 0
    while prod["state"] != "done" or cons["state"] != "done":
        steps += 1
        assert steps < 100 * (n + S * limit) + 1000, "the ring stalled"
        late = prod["state"] != "run" or cons["state"] != "run"
        events = []
        if landable(copies, late):
            events.append("copy")
        if landable(mmas, late):
            events.append("mma")
        if prod["state"] != "done":
            events.append("prod")
        if cons["state"] != "done":
            events.append("cons")
        if not events:                       # only stuck work left
            break
        e = rng.choice(events)
        if e == "copy":
            s = rng.choice(landable(copies, late))
            content[s] = copies.pop(s)[0]
            full[s] += 1
        elif e == "mma":
            s = rng.choice(landable(mmas, late))
            mmas.pop(s)
            empty[s] += 1
        elif e == "prod":
            if prod["state"] == "run":
                i = prod["i"]
                if i == n:
                    prod["state"] = "drain"
                    continue
                s, u = i % S, i // S
                if u > 0 and not _parity_done(empty[s], (u - 1) & 1):
                    prod["polls"] += 1
                    if prod["polls"] >= limit:
                        prod["state"] = "drain"
                    continue
                prod["polls"] = 0
                assert s not in copies, "two copies in flight in one stage"
                copies[s] = (i, kind())
                prod["i"] = i + 1
                prod["issued"] = i + 1
            else:                            # the drain, one stage at a time
                s = prod["drain_s"]
                issued = prod["issued"]
                if s >= min(S, issued):
                    prod["state"] = "done"
                    continue
                last = s + ((issued - 1 - s) // S) * S
                assert full[s] in (last // S, last // S + 1), "the drain could confuse two phases"
                if _parity_done(full[s], (last // S) & 1):
                    if s in copies:
                        prod["missed"].append(s)
                    prod["drain_s"] += 1
                    prod["polls"] = 0
                else:
                    prod["polls"] += 1
                    if prod["polls"] >= limit:
                        prod["drain_s"] += 1
                        prod["polls"] = 0
        else:
            i = cons["i"]
            if i == n or cons["state"] == "stop":
                cons["state"] = "done"
                continue
            s, u = i % S, i // S
            if not _parity_done(full[s], u & 1):
                cons["polls"] += 1
                if cons["polls"] >= limit:
                    cons["state"] = "stop"
                continue
            cons["polls"] = 0
            assert content[s] == i, f"MMA read chunk {content[s]} for chunk {i}"
            assert s not in mmas
            mmas[s] = (i, kind())
            cons["i"] = i + 1
    failed = prod["i"] < n or cons["i"] < n
    return {"failed": failed, "missed": prod["missed"]}


@pytest.mark.parametrize("S", [4, 6])
def test_init_ring_failure_path_drains_every_copy(S):
    failures = 0
    for seed in range(400):
        for n in (1, S - 1, S, S + 1, 12, 3 * S + 2):
            r = run_ring_with_failures(S, n, seed, limit=6)
            failures += r["failed"]
            assert not r["missed"], (seed, n, r)
    assert failures > 50
