"""Batched persistent binning (hbt_bin_batch): many same-event and
mixed-event jobs of uneven sizes in one launch, lists sorted in momentum
space and tile pairs culled.  The result must equal the oracle binning the
same jobs one by one: counts exact, FP64 sums within tests/parity.py's
tolerance."""
import numpy as np
import pytest

import oracle_lib
import parity

pytestmark = pytest.mark.gpu

BASE = dict(qnpts=13, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=6,
            azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
            needed_number_of_pairs=1e18)


def _qscale(p):
    return max(abs(p["q_min"]), abs(p["q_max"])) + (p["q_max"] - p["q_min"]) / (p["qnpts"] - 1)


def _uneven_jobs(seed, n_groups=5):
    """Groups of log-uniform multiplicity events (the uneven workload's shape,
    scaled down), with tiny and empty lists mixed in."""
    from hadronic_afterburner_toolkit_gb300 import synth
    rng = np.random.default_rng(seed)
    jobs = []
    for g in range(n_groups):
        mult = np.floor(np.exp(rng.uniform(np.log(2), np.log(400), size=6))).astype(np.int64)
        if g == 1:
            mult[:3] = [0, 1, 2]
        ev = synth.generate(mult.size, mult, seed=seed * 100 + g, sigma_xy=2.0, tau_mean=3.0,
                            T=0.4 if g % 2 else 0.25)
        cols = parity.cols8(ev)
        jobs.append(("same", cols))
        o = ev.offsets
        for e in range(ev.n_events):
            l1 = parity.rotated4(ev, 0.0, o[e], o[e + 1])
            l2 = parity.rotated4(ev, 0.5 + e, o[(e + 1) % ev.n_events], None)
            jobs.append(("mixed", l1, l2))
    return jobs


def _run_oracle(p, jobs, psi=0.0):
    orc = oracle_lib.Oracle(**p)
    orc.set_psi_ref(psi)
    for j in jobs:
        if j[0] == "same":
            orc.bin_same(j[1])
        else:
            orc.bin_mixed(j[1], j[2])
    return orc.hist()


@pytest.mark.parametrize("az,boost,order", [(0, 1, 0), (1, 1, 0), (0, 0, 0), (1, 0, 0),
                                            (0, 1, 1), (1, 0, 1)])
def test_batch_matches_oracle(az, boost, order):
    """order = 1: the same-event tile pairs taken in momentum-region order
    (hbt_tuning.order_items); the bins and counts do not depend on it."""
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE, azimuthal_flag=az, long_comoving_boost=boost)
    jobs = _uneven_jobs(seed=3 + az + 2 * boost)
    eng = E.Engine(**p)
    eng.set_tuning(order_items=order)
    eng.set_psi_ref(0.7)
    eng.bin_batch(jobs)
    h = _run_oracle(p, jobs, psi=0.7)
    assert h["count"].sum() > 500 and h["den"].sum() > 500
    parity.compare(eng.hist(), h, _qscale(p))


def test_batch_equals_single_calls_and_grid_kernels():
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE, azimuthal_flag=1)
    jobs = _uneven_jobs(seed=11, n_groups=3)
    out = []
    for kernel in (E.KERNEL_SCREENED, E.KERNEL_SCREENED_GRID):
        eng = E.Engine(kernel=kernel, **p)
        eng.set_psi_ref(-0.3)
        for j in jobs:
            if j[0] == "same":
                eng.bin_same(j[1])
            else:
                eng.bin_mixed(j[1], j[2])
        out.append(eng.hist())
    engb = E.Engine(**p)
    engb.set_psi_ref(-0.3)
    engb.bin_batch(jobs)
    out.append(engb.hist())
    for h in out[1:]:
        for k in ("count", "den", "ctr_num", "ctr_den"):
            assert np.array_equal(h[k], out[0][k]), k


def test_batch_with_binding_caps_runs_in_reference_order():
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE, needed_number_of_pairs=30)
    jobs = _uneven_jobs(seed=21, n_groups=2)
    eng = E.Engine(**p)
    eng.bin_batch(jobs)
    h = _run_oracle(p, jobs)
    assert (h["ctr_num"] == 31).any() and (h["ctr_den"] == 31).any()
    parity.compare(eng.hist(), h, _qscale(p))


def test_batch_mixed_jobs_admitted_together():
    """Binding caps on a batch of many mixed-event jobs: their pairs are
    admitted together in the jobs' joint row order (one count pass, one cut
    per slot and one order pass; each slot's cut row inside its own job),
    with K_phi edges within a wide deferral tolerance (1e-3 rad: thousands of
    pairs, within the 65536 a count pass may hand over) decided on the host.
    Equal to the oracle binning the jobs one by one in the reference's
    order."""
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE, azimuthal_flag=1, needed_number_of_pairs=40)
    jobs = _uneven_jobs(seed=51, n_groups=3)
    eng = E.Engine(kphi_defer_tol=1e-3, **p)
    eng.set_psi_ref(0.4)
    eng.bin_batch(jobs)
    h = _run_oracle(p, jobs, psi=0.4)
    assert (h["ctr_den"] == 41).any() and (h["ctr_den"] < 41).any()
    st = eng.stats()
    assert st["deferred_kphi"] > 0
    # one admission for all mixed jobs, at most one per same-event job
    assert st["ordered_passes"] <= 1 + sum(1 for j in jobs if j[0] == "same")
    parity.compare(eng.hist(), h, _qscale(p))


def test_batch_cap_passes_skip_tile_pairs_of_full_slots():
    """Once the busiest slots are past the cap, the count and order passes
    skip the tile pairs whose pairs can reach only those slots: fewer tile
    pairs kept than an uncapped launch of the same job keeps, with counts
    and counters equal to the oracle's."""
    from hadronic_afterburner_toolkit_gb300 import engine as E
    from hadronic_afterburner_toolkit_gb300 import synth
    p0 = dict(BASE, azimuthal_flag=1)
    a = parity.cols8(synth.generate(1, np.array([3000]), seed=71))
    b = parity.cols8(synth.generate(1, np.array([3000]), seed=72))
    first = _run_oracle(p0, [("same", a)], psi=0.3)["ctr_num"]
    cap = float(np.median(first[first > 0]))
    p = dict(p0, needed_number_of_pairs=cap)
    jobs = [("same", a), ("same", b)]
    eng = E.Engine(**p)
    eng.set_psi_ref(0.3)
    eng.bin_batch(jobs[:1])
    eng.bin_batch(jobs[1:])
    kept = eng.stats()["tiles_same_kept"]
    free = E.Engine(**p0)
    free.set_psi_ref(0.3)
    free.bin_batch(jobs[1:])
    assert 0 < kept < free.stats()["tiles_same_kept"]
    h = _run_oracle(p, jobs, psi=0.3)
    assert (h["ctr_num"] > cap).any() and (h["ctr_num"] <= cap).any()
    parity.compare(eng.hist(), h, _qscale(p))


def test_batch_fp32w_counts_exact():
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE, azimuthal_flag=1)
    jobs = _uneven_jobs(seed=31, n_groups=4)
    eng = E.Engine(precision=E.PRECISION_FP32W, **p)
    eng.set_psi_ref(0.2)
    eng.bin_batch(jobs)
    h = _run_oracle(p, jobs, psi=0.2)
    worst = parity.compare(eng.hist(), h, _qscale(p), rtol=1e-5)
    assert worst["num"] < 1e-6


def test_batch_counts_do_not_depend_on_the_schedule():
    """The histogram updates are atomic and every pair is visited once, so
    counts, denominators and counters come out the same whatever the number
    of persistent CTAs, the sort cells or the item order (the sums agree to
    rounding: their order changes)."""
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE, azimuthal_flag=1)
    jobs = _uneven_jobs(seed=61, n_groups=3)
    ref = None
    for bps, cell, order in ((0, 0.02, 1), (1, 0.02, 0), (2, 0.01, 1), (3, 0.04, 0),
                             (5, 0.02, 1), (8, 0.01, 0)):
        eng = E.Engine(**p)
        eng.set_tuning(blocks_per_sm=bps, cell_pt=cell, order_items=order)
        eng.set_psi_ref(0.25)
        eng.bin_batch(jobs)
        h = eng.hist()
        eng.close()
        if ref is None:
            ref = h
            continue
        for k in ("count", "den", "ctr_num", "ctr_den"):
            assert np.array_equal(h[k], ref[k]), (k, bps, cell, order)
        for k in ("q_out", "q_side", "q_long", "num"):
            np.testing.assert_allclose(h[k], ref[k], rtol=0, atol=1e-12 * (ref["count"].max() + 1))


def test_batch_device_resident():
    torch = pytest.importorskip("torch")
    from hadronic_afterburner_toolkit_gb300 import engine as E
    jobs = _uneven_jobs(seed=41, n_groups=2)
    djobs = []
    for j in jobs:
        if j[0] == "same":
            djobs.append(("same", [torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in j[1]]))
        else:
            djobs.append(("mixed", [torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in j[1]],
                          [torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in j[2]]))
    a, b = E.Engine(**BASE), E.Engine(**BASE)
    a.bin_batch(jobs)
    b.bin_batch(djobs, device=True)
    ha, hb = a.hist(), b.hist()
    for k in ("count", "den"):
        assert np.array_equal(ha[k], hb[k])


def test_async_readback_is_a_snapshot():
    """hbt_read_hist_async: the arrays equal hbt_read_hist at the time of the
    call, although more pairs are binned while the copies are in flight; a
    second call waits for the first; K_phi slots (deferred edges drained)."""
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE, azimuthal_flag=1)
    jobs = _uneven_jobs(seed=17)
    eng = E.Engine(**p)
    eng.set_psi_ref(0.3)
    eng.bin_batch(jobs[:len(jobs) // 2])
    n = int(eng.L.hbt_n_bins(eng.handle))
    sync = [np.zeros(n) for _ in range(6)]
    eng._check(eng.L.hbt_read_hist(eng.handle, *[a.ctypes.data_as(E._PD) for a in sync]))
    snap = [np.full(n, -1.0) for _ in range(6)]
    eng._check(eng.L.hbt_read_hist_async(eng.handle, *[a.ctypes.data_as(E._PD) for a in snap]))
    eng.bin_batch(jobs[len(jobs) // 2:])  # binning goes on while the copy is in flight
    eng._check(eng.L.hbt_read_hist_wait(eng.handle))
    for a, b in zip(snap, sync):
        np.testing.assert_array_equal(a, b)
    # the second snapshot holds all jobs and equals the oracle's binning
    full = [np.zeros(n) for _ in range(6)]
    eng._check(eng.L.hbt_read_hist_async(eng.handle, *[a.ctypes.data_as(E._PD) for a in full]))
    eng._check(eng.L.hbt_read_hist_wait(eng.handle))
    eng._check(eng.L.hbt_read_hist_wait(eng.handle))  # nothing pending: returns at once
    h = eng.hist()
    for a, k in zip(full, ("count", "q_out", "q_side", "q_long", "num", "den")):
        np.testing.assert_array_equal(a, h[k])
    assert full[0].sum() > sync[0].sum()
