"""The named-barrier sequence of the persistent SOR kernel (csrc/cnv_poisson.cu), checked on the
CPU by running it under many random schedules.

A block of k_poisson has 32 warps: warps 0-30 update cells (0-11 also the tile's frame) and warp
31, the signal warp, does the inter-block work. They meet only at named barriers, which cannot
time out, so the sequence must never pair arrivals of two different instances of one barrier
(PTX bar semantics: an instance completes when its expected count of warps has arrived, and
later arrivals count toward the next instance). The model below restates the sequences of
signal_warp() and cell_warps() warp by warp and checks, for SOR/Gauss-Seidel (two half-sweeps
per sweep) and Jacobi (one), every stop point and many interleavings, that
  - every completed barrier instance holds arrivals of one sweep / half-sweep only,
  - no schedule deadlocks,
  - the signal warp reads a sweep's norm partials before the cell warps overwrite them.
The earlier order, in which the signal warp took sweep k-1's partials after its first PUB of
sweep k, must fail the check for Jacobi (it hung on the GPU that way).
"""
from __future__ import annotations

import random

import pytest

CELL_WARPS, FRAME_WARPS = 31, 12  # kCellWarps, kFrameWarps of csrc/cnv_poisson.cu
SIGNAL_WARP = CELL_WARPS
EXPECTED = {"DEC": CELL_WARPS + 1, "GO": FRAME_WARPS + 1, "PUB": FRAME_WARPS + 1, "END": CELL_WARPS,
            "NORM": CELL_WARPS + 1}


def signal_ops(kmax, halves, stop_at, norm_before_go=True):
    """signal_warp(): DEC arrival, then per half-sweep the neighbour polls, (first half: NORM wait
    for the previous sweep's partials), GO arrival, PUB wait, flag, (first half: contribute)."""
    for k in range(1, kmax + 1):
        yield ("arrive", "DEC", (k,))
        if stop_at == k:
            if k >= 2:
                yield ("sync", "NORM", (k - 1,))
            return
        for h in range(halves):
            if norm_before_go and h == 0 and k >= 2:
                yield ("sync", "NORM", (k - 1,))
            yield ("arrive", "GO", (k, h))
            yield ("sync", "PUB", (k, h))
            if not norm_before_go and h == 0 and k >= 2:
                yield ("sync", "NORM", (k - 1,))
            if h == 0 and k >= 2:
                yield ("read", (k - 1) & 1, k - 1)  # contribute(k-1) reads part[(k-1) & 1]
    if kmax >= 1:
        yield ("sync", "NORM", (kmax,))
        yield ("read", kmax & 1, kmax)


def cell_ops(warp, kmax, halves, stop_at):
    """cell_warps(): DEC wait, per half-sweep (frame warps: GO wait, frame, PUB arrival) interior
    and END wait, then the warp's norm partials and a NORM arrival."""
    for k in range(1, kmax + 1):
        yield ("sync", "DEC", (k,))
        if stop_at == k:
            return
        for h in range(halves):
            if warp < FRAME_WARPS:
                yield ("sync", "GO", (k, h))
                yield ("arrive", "PUB", (k, h))
            yield ("sync", "END", (k, h))
        yield ("write", k & 1, k)
        yield ("arrive", "NORM", (k,))


def run_schedule(kmax, halves, stop_at, seed, norm_before_go=True):
    """One random interleaving; returns None or a description of what went wrong."""
    rnd = random.Random(seed)
    gens = {SIGNAL_WARP: signal_ops(kmax, halves, stop_at, norm_before_go)}
    for w in range(CELL_WARPS):
        gens[w] = cell_ops(w, kmax, halves, stop_at)
    cur = {w: next(g, None) for w, g in gens.items()}
    blocked, bars, part = set(), {b: [] for b in EXPECTED}, {0: None, 1: None}
    while True:
        ready = [w for w in cur if cur[w] is not None and w not in blocked]
        if not ready:
            left = [w for w in cur if cur[w] is not None]
            return f"deadlock: warps {left}" if left else None
        w = rnd.choice(ready)
        op = cur[w]
        if op[0] in ("arrive", "sync"):
            name, tag = op[1], op[2]
            bars[name].append((w, tag, op[0] == "sync"))
            if len(bars[name]) == EXPECTED[name]:
                tags = {t for _, t, _ in bars[name]}
                if len(tags) != 1:
                    return f"{name} instance mixes {sorted(tags)}"
                for ww, _, waits in bars[name]:
                    if waits and ww != w:
                        blocked.discard(ww)
                        cur[ww] = next(gens[ww], None)
                bars[name] = []
                cur[w] = next(gens[w], None)
            elif op[0] == "sync":
                blocked.add(w)
            else:
                cur[w] = next(gens[w], None)
        elif op[0] == "write":
            part[op[1]] = op[2]
            cur[w] = next(gens[w], None)
        else:  # read
            if part[op[1]] != op[2]:
                return f"signal warp read sweep {part[op[1]]}'s partials, wanted sweep {op[2]}'s"
            cur[w] = next(gens[w], None)


def failures(halves, norm_before_go, seeds):
    out = []
    for kmax in (1, 2, 3, 5, 8):
        for stop_at in [None] + list(range(3, kmax + 1)):
            for seed in range(seeds):
                r = run_schedule(kmax, halves, stop_at, seed, norm_before_go)
                if r:
                    out.append((kmax, stop_at, seed, r))
    return out


@pytest.mark.parametrize("halves", [2, 1], ids=["sor_gs", "jacobi"])
def test_kernel_barrier_sequence_never_mispairs(halves):
    assert failures(halves, True, 60) == []


def test_old_order_mispairs_for_jacobi():
    bad = failures(1, False, 60)
    assert bad and all("NORM" in r for *_, r in bad)


def test_model_matches_the_kernel_layout():
    """The model's warp counts are the kernel's (kThreads / 32 - 1 cell warps, kFrameWarps)."""
    import os
    import re

    src = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "fluid-dynamics1_gb300", "csrc",
                            "cnv_poisson.cu")).read()
    threads = int(re.search(r"constexpr int kThreads = (\d+);", src).group(1))
    frame = int(re.search(r"constexpr int kFrameWarps = (\d+);", src).group(1))
    assert (threads // 32 - 1, frame) == (CELL_WARPS, FRAME_WARPS)
