"""Replicas over oversample groups (hadronic_afterburner_toolkit_gb300/
replicas.py) with world_size 2 over gloo on the CPU: each rank bins its
shard of the groups; the benchmark's one all-reduce (bench.allreduce_hist)
and the host-side sum of the ranks' saved histograms (replicas.sum_hists)
both give the single-process binning of every group (counts exact, FP64
sums within 1e-12 relative).  The CPU oracle stands in for the GPU engine
here; the engine exposes the same bin_same / bin_mixed / hist interface."""
import os
import socket

import numpy as np
import pytest

import oracle_lib
import parity

P = dict(qnpts=11, q_min=-0.15, q_max=0.15, n_KT=4, KT_min=0.0, KT_max=1.0, n_Kphi=4,
         azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
         needed_number_of_pairs=1e18)


def _groups(seed=5, n_groups=5):
    from hadronic_afterburner_toolkit_gb300 import synth
    out = []
    for g in range(n_groups):
        ev = synth.generate(4, 40.0 + 20 * g, seed=seed * 100 + g, sigma_xy=2.0, tau_mean=3.0)
        cols = parity.cols8(ev)
        mixed = []
        o = ev.offsets
        for e in range(ev.n_events):
            l1 = parity.rotated4(ev, 0.0, o[e], o[e + 1])
            l2 = parity.rotated4(ev, 0.3 + e, o[(e + 1) % ev.n_events], o[(e + 1) % ev.n_events + 1])
            mixed.append((l1, l2))
        out.append((cols, mixed))
    return out


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    from hadronic_afterburner_toolkit_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        groups = _groups()
        orc = oracle_lib.Oracle(**P)
        mine = replicas.bin_shard(orc, groups, rank, world)
        replicas.save_hist(os.path.join(out_dir, "rank%d.npz" % rank), orc.hist())
        import bench
        h = bench.allreduce_hist(orc.hist())
        if rank == 0:
            np.savez(os.path.join(out_dir, "reduced.npz"), mine=np.array(mine),
                     **{k: np.asarray(v) for k, v in h.items()})
    finally:
        dist.destroy_process_group()


def test_shard_covers_every_group_once():
    from hadronic_afterburner_toolkit_gb300 import replicas
    for n in (0, 1, 5, 8):
        for world in (1, 2, 3):
            got = sorted(g for r in range(world) for g in replicas.shard(n, r, world))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_caps_decide_whether_groups_can_shard():
    from hadronic_afterburner_toolkit_gb300 import replicas
    assert replicas.caps_allow_sharding(P, 10**9, 10**9)
    assert not replicas.caps_allow_sharding(dict(P, needed_number_of_pairs=100), 1000, 10)


def test_two_gloo_ranks_equal_one_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    red = dict(np.load(tmp_path / "reduced.npz"))
    assert list(red.pop("mine")) == [0, 2, 4]
    orc = oracle_lib.Oracle(**P)
    for cols, mixed in _groups():
        orc.bin_same(cols)
        for l1, l2 in mixed:
            orc.bin_mixed(l1, l2)
    ref = orc.hist()
    for k in ("pairs_same", "pairs_mixed", "anomalies"):
        red[k] = int(red[k])
    assert ref["count"].sum() > 100 and ref["den"].sum() > 100
    scale = 0.15 + 0.3 / 10
    parity.compare(red, ref, scale)
    # the same sum on the host from the ranks' saved histograms
    from hadronic_afterburner_toolkit_gb300 import replicas
    summed = replicas.sum_hists([replicas.load_hist(str(tmp_path / ("rank%d.npz" % r)))
                                 for r in range(2)])
    parity.compare(summed, ref, scale)
