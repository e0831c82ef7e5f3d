"""Replicas over oversample groups: one process per GPU.

The pair binning of one buffer (oversample group) is independent of every
other buffer except through the needed_number_of_pairs caps, whose counters
run over the whole job in the reference's order.  With no cap that can
bind, ranks bin disjoint shards of the groups into their own histograms and
one sum at the end gives the single-process histograms: counts, denominators
and pair counters exactly (integer sums), the FP64 sums up to summation
order.  No collective runs on the data path; the one reduction uses
torch.distributed (gloo on CPU tensors, NCCL on GPU tensors).
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


def allreduce_hist(h: Dict[str, np.ndarray], device=None) -> Dict[str, np.ndarray]:
    """Sums a histogram dict over all ranks of the default process group.
    Counts travel as int64 (exact), sums as float64."""
    import torch
    import torch.distributed as dist
    out = dict(h)
    for keys, dtype in ((COUNT_KEYS, torch.int64), (SUM_KEYS, torch.float64)):
        present = [k for k in keys if k in h]
        if not present:
            continue
        flat = np.concatenate([np.asarray(h[k]).ravel().astype(
            np.int64 if dtype == torch.int64 else np.float64) for k in present])
        t = torch.from_numpy(flat)
        if device is not None:
            t = t.to(device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        flat = t.cpu().numpy()
        at = 0
        for k in present:
            n = np.asarray(h[k]).size
            part = flat[at:at + n].reshape(np.asarray(h[k]).shape)
            out[k] = part.astype(np.asarray(h[k]).dtype) if dtype == torch.int64 else part
            at += n
    sc = [k for k in SCALAR_KEYS if k in h]
    if sc:
        t = torch.tensor([int(h[k]) for k in sc], dtype=torch.int64)
        if device is not None:
            t = t.to(device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        for k, v in zip(sc, t.cpu().tolist()):
            out[k] = int(v)
    return out


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
