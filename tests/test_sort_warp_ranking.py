"""The radix sort's warp-level rules (csrc/sort.cu: k_rs_hist, k_rs_scatter),
restated lane by lane in Python and checked against their definitions on the
CPU; the kernels themselves are checked against the oracle's stable
permutation by tests/test_gpu_ops.py.

* Histogram: each run of equal neighbouring digits among a group's valid lanes
  (a prefix of the 32) adds its length once, at its first lane; the totals are
  the digit counts whatever the order (a digit that recurs starts a new run).
* Scatter ranking of a round whose valid digits are non-decreasing across the
  lanes: the run's first lane reads the warp's counter for its digit and
  advances it by the run length; every lane's rank is that old count plus its
  offset in the run. That is the number of items with its digit before it in
  (round, lane) order, as the match.any ranking gives.
"""

from __future__ import annotations

import numpy as np

FULL = 0xFFFFFFFF


def _upto(lane: int) -> int:
    return FULL >> (31 - lane)


def _runs(d, ok):
    """(heads mask, run end per lane) as the kernels compute them."""
    heads = 0
    for lane in range(32):
        dprev = d[lane - 1] if lane > 0 else d[0]
        if ok[lane] and (lane == 0 or d[lane] != dprev):
            heads |= 1 << lane
    nvalid = sum(ok)
    ends = []
    for lane in range(32):
        above = heads & ~_upto(lane) & FULL
        ends.append((above & -above).bit_length() - 1 if above else nvalid)
    return heads, ends


def _hist_by_runs(d, ok, cnt):
    heads, ends = _runs(d, ok)
    for lane in range(32):
        if heads >> lane & 1:
            cnt[d[lane]] = cnt.get(d[lane], 0) + ends[lane] - lane


def _rank_in_order_round(d, ok, whist):
    heads, ends = _runs(d, ok)
    old = [0] * 32
    for lane in range(32):
        if ok[lane] and heads >> lane & 1:
            old[lane] = whist.get(d[lane], 0)
            whist[d[lane]] = old[lane] + ends[lane] - lane
    ranks = []
    for lane in range(32):
        hb = heads & _upto(lane)
        hl = hb.bit_length() - 1  # -1: no valid lane at all
        ranks.append(old[hl & 31] + lane - hl)
    return ranks


def _round(rng, in_order: bool):
    nvalid = 32 if rng.random() < 0.7 else int(rng.integers(0, 33))
    ok = [lane < nvalid for lane in range(32)]
    base = int(rng.integers(0, 480))
    d = list(rng.integers(base, base + int(rng.choice([1, 2, 4, 32])), size=32))
    if in_order:
        d.sort()
    d = [int(v) if ok[lane] else 0 for lane, v in enumerate(d)]
    return d, ok


def test_run_histogram_counts_every_digit():
    rng = np.random.default_rng(5)
    for _ in range(3000):
        d, ok = _round(rng, in_order=bool(rng.random() < 0.5))
        cnt = {}
        _hist_by_runs(d, ok, cnt)
        ref = {}
        for lane in range(32):
            if ok[lane]:
                ref[d[lane]] = ref.get(d[lane], 0) + 1
        assert cnt == ref


def test_run_ranking_equals_match_ranking_on_in_order_rounds():
    rng = np.random.default_rng(6)
    for _ in range(300):
        whist_run, whist_ref = {}, {}
        for _ in range(16):  # a warp's 16 rounds
            d, ok = _round(rng, in_order=True)
            ranks = _rank_in_order_round(d, ok, whist_run)
            for lane in range(32):
                if ok[lane]:
                    assert ranks[lane] == whist_ref.get(d[lane], 0), (d, ok, lane)
                    whist_ref[d[lane]] = whist_ref.get(d[lane], 0) + 1
            assert whist_run == whist_ref
