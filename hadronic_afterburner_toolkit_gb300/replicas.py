"""Replicas over oversample groups: one process per GPU.

The pair binning of one buffer (oversample group) is independent of every
other buffer except through the needed_number_of_pairs caps, whose counters
run over the whole job in the reference's order.  With no cap that can
bind, ranks bin disjoint shards of the groups into their own histograms and
one sum at the end gives the single-process histograms: counts, denominators
and pair counters exactly (integer sums), the FP64 sums up to summation
order.  No collective runs on the data path.  Each replica (one process per
GPU, on one box or many) saves its histograms with save_hist; one host
process adds the files with sum_hists and writes the reference's output
files from the sum (hbt_host_write).
"""
from __future__ import annotations

from typing import Dict, List, Sequence

import numpy as np

# histogram arrays summed exactly (integer-valued) and in FP64
COUNT_KEYS = ("count", "den", "qinv_count", "qinv_den", "ctr_num", "ctr_den", "ctr_num_qinv",
              "ctr_den_qinv")
SUM_KEYS = ("q_out", "q_side", "q_long", "num", "qinv_sum", "qinv_num")
SCALAR_KEYS = ("pairs_same", "pairs_mixed", "anomalies")


def shard(n_items: int, rank: int, world: int) -> List[int]:
    """Items of this rank: round robin, so uneven group sizes spread out."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world of %d" % (rank, world))
    return list(range(rank, n_items, world))


def caps_allow_sharding(params: dict, total_same_pairs: int, total_mixed_pairs: int) -> bool:
    """True when no needed_number_of_pairs cap can bind over the whole job
    (every counter stays below the cap), so the order of the groups does not
    matter.  Otherwise the job must run in one process."""
    cap = float(params.get("needed_number_of_pairs", 1e18))
    ok = max(total_same_pairs, total_mixed_pairs) <= cap
    if params.get("invariant_radius_flag", 0) == 1:
        ok = ok and max(total_same_pairs, total_mixed_pairs) < 50 * cap
    return ok


def sum_hists(hists: Sequence[Dict[str, np.ndarray]]) -> Dict[str, np.ndarray]:
    """Host-side sum of the histograms of several replicas, in the order
    given: counts and pair counters as exact int64 sums (returned in their
    own dtype), the FP64 sums added in float64, the scalar totals as ints."""
    if not hists:
        raise ValueError("no histograms to sum")
    out: Dict[str, np.ndarray] = {}
    for k in COUNT_KEYS:
        if k in hists[0]:
            acc = np.zeros(np.asarray(hists[0][k]).shape, dtype=np.int64)
            for h in hists:
                acc += np.asarray(h[k]).astype(np.int64)
            out[k] = acc.astype(np.asarray(hists[0][k]).dtype)
    for k in SUM_KEYS:
        if k in hists[0]:
            acc = np.zeros(np.asarray(hists[0][k]).shape, dtype=np.float64)
            for h in hists:
                acc += np.asarray(h[k], dtype=np.float64)
            out[k] = acc
    for k in SCALAR_KEYS:
        if k in hists[0]:
            out[k] = int(sum(int(h[k]) for h in hists))
    return out


def save_hist(path: str, h: Dict[str, np.ndarray]) -> None:
    """One replica's histograms (Engine.hist()) as an .npz file."""
    np.savez(path, **{k: np.asarray(v) for k, v in h.items()})


def load_hist(path: str) -> Dict[str, np.ndarray]:
    d = dict(np.load(path))
    for k in SCALAR_KEYS:
        if k in d:
            d[k] = int(d[k])
    return d


def bin_shard(binner, groups: Sequence, rank: int, world: int) -> List[int]:
    """Bins this rank's groups (each (same_cols8, [(list1, list2), ...]))
    with `binner` (an Engine, or anything with bin_same / bin_mixed);
    returns the group indices it took."""
    mine = shard(len(groups), rank, world)
    for g in mine:
        cols, mixed = groups[g]
        binner.bin_same(cols)
        for l1, l2 in mixed:
            binner.bin_mixed(l1, l2)
    return mine
