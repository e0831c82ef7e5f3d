"""GPU parity at the benchmark configurations' full sizes.

The other parity tests use small q grids and a few thousand particles.
These run the engine on whole benchmark workloads and check every bin
against the CPU oracle (oracle/hbt_oracle.cpp, pinned byte for byte to the
reference's files) on the same inputs:

* the small configuration in full: 100 pi+ events, Poisson(500),
  oversample 10 (10 groups of ~5k particles), 41^3 q grid, 4 K_T bins,
  5 rotated partners per event, seed 1 - once through one hbt_bin_batch
  call for the whole run, once through the drop-in executable (read, bin,
  write) against the oracle's output files;
* one group of the central configuration: ~150k pi+ particles (100 events
  of Poisson(1500)), 8 K_T x 8 K_phi bins with psi_ref from the event
  plane, 10 partners - against the oracle's multi-threaded pair loops;
* the precision configuration on that group and on three K+ groups: the
  FP32-weight and double-float forms against the same oracle;
* three ~50k-particle groups of the uneven-multiplicity configuration in
  one batched call, FP64 and (autotuned, replayed as a CUDA graph)
  FP32-weight forms.

The reference path these cover is src/HBT_correlation.cpp:177-218 (driver),
:291-461 (same-event loop) and :563-689 (mixed-event loop).  Partners and
rotation angles come from the drop-in's own draws (hbt_host_mixed_plan,
itself checked against the oracle's on the CPU); rotations use the C
library's cos and sin as the reference does.
"""
import ctypes
import math
import os
import subprocess

import numpy as np
import pytest

import oracle_lib
import parity
from hadronic_afterburner_toolkit_gb300 import build, engine, synth

pytestmark = pytest.mark.gpu

EXE = os.path.join(oracle_lib.REPO, "hadronic_afterburner_toolkit_gb300", "lib",
                   "hbt_afterburner.e")
NTHREADS = max(1, os.cpu_count() or 1)
YCUT = (math.tanh(-1.0), math.tanh(1.0))


@pytest.fixture(scope="module")
def host():
    lib = build.build_host()
    L = ctypes.CDLL(lib)
    _pi = ctypes.POINTER(ctypes.c_int32)
    L.hbt_host_mixed_plan.restype = ctypes.c_int64
    L.hbt_host_mixed_plan.argtypes = [ctypes.c_int32, ctypes.c_int32, _pi, _pi, ctypes.c_int32,
                                      ctypes.c_int64, _pi, ctypes.POINTER(ctypes.c_double)]
    return L


def mixed_plan(host, seed, nev, n_partners):
    """Partner ids and angles per buffer: list of (partners[nev, nmix], angles[nev, nmix])."""
    nev = np.ascontiguousarray(nev, dtype=np.int32)
    total = int(nev.sum()) * n_partners
    p = np.zeros(total, dtype=np.int32)
    a = np.zeros(total)
    _pi = ctypes.POINTER(ctypes.c_int32)
    got = host.hbt_host_mixed_plan(seed, nev.size, nev.ctypes.data_as(_pi),
                                   nev.ctypes.data_as(_pi), n_partners, total,
                                   p.ctypes.data_as(_pi),
                                   a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert got == total
    out, at = [], 0
    for n in nev:
        k = int(n) * n_partners
        out.append((p[at:at + k].reshape(n, n_partners), a[at:at + k].reshape(n, n_partners)))
        at += k
    return out


def _cut(cols, lo, hi):
    """The rapidity gather of src/HBT_correlation.cpp:254-285 (strict)."""
    r = cols[2][lo:hi] / cols[3][lo:hi]
    keep = (r > YCUT[0]) & (r < YCUT[1])
    return [np.ascontiguousarray(c[lo:hi][keep]) for c in cols]


def buffer_jobs(g, partners, angles):
    """Same-event job and one mixed job per event of one buffer, built as the
    drop-in builds them (src/HBT_correlation.cpp:254-285, :466-552)."""
    cols = [np.ascontiguousarray(getattr(g, k)) for k in ("px", "py", "pz", "E", "x", "y", "z", "t")]
    jobs = [("same", _cut(cols, 0, g.n_particles))]
    for e in range(g.n_events):
        l1 = _cut(cols[:4], int(g.offsets[e]), int(g.offsets[e + 1]))
        parts = []
        for m, phi in zip(partners[e], angles[e]):
            c, s = math.cos(float(phi)), math.sin(float(phi))
            px, py, pz, E = _cut(cols[:4], int(g.offsets[m]), int(g.offsets[m + 1]))
            parts.append((px * c - py * s, px * s + py * c, pz, E))
        l2 = [np.ascontiguousarray(np.concatenate([p[f] for p in parts])) for f in range(4)]
        jobs.append(("mixed", l1, l2))
    return jobs


def engine_hist(p, jobs, psi=None, precision=engine.PRECISION_FP64, calls=None):
    eng = engine.Engine(device=0, precision=precision, **p)
    if psi is not None:
        eng.set_psi_ref(psi)
    for chunk in (calls or [jobs]):
        eng.bin_batch(chunk)
    h = eng.hist()
    st = eng.stats()
    eng.close()
    return h, st


SMALL = dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=8,
             azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
             needed_number_of_pairs=1e18)


@pytest.fixture(scope="module")
def small_run(host):
    ev = synth.small_pions(seed=1)
    bufs = synth.buffers(ev, 5000)
    plans = mixed_plan(host, 1, [b - a for a, b in bufs], 5)
    orc = oracle_lib.Oracle(number_of_mixed_events=5, seed=1, **SMALL)
    jobs = []
    for (a, b), (partners, angles) in zip(bufs, plans):
        g = synth.subset(ev, a, b)
        orc.process_buffer(g)
        jobs += buffer_jobs(g, partners, angles)
    return ev, bufs, orc, jobs


def test_small_configuration_in_one_batched_call(small_run):
    """All 10 groups and 100 mixed jobs of the small configuration in one
    hbt_bin_batch call: counts, denominators and pair counters identical to
    the oracle's buffer loop, sums within parity.RTOL."""
    ev, bufs, orc, jobs = small_run
    assert len(bufs) == 10 and len(jobs) == 110
    h, st = engine_hist(SMALL, jobs)
    o = orc.hist()
    assert o["pairs_same"] + o["pairs_mixed"] > 2.5e8
    assert o["count"].sum() > 1e7 and o["den"].sum() > 1e7
    parity.compare(h, o, q_scale=0.15)
    assert st["tiles_same_kept"] < st["tiles_same"]  # the cull ran on this batch


def test_small_configuration_through_the_drop_in(small_run, tmp_path):
    """lib/hbt_afterburner.e reads the small configuration's samples (mode 10,
    event_buffer_size 5000, hbt_mixed_partners 5), bins each buffer in one
    batched call and writes the reference's files: they match the oracle's
    files for the same run (denominator column identical, numerator and mean
    q to the printed precision), and the logged pair totals agree."""
    from test_dropin_gpu import compare_files
    ev, bufs, orc, _ = small_run
    res = tmp_path / "results"
    res.mkdir()
    synth.write_mode10(str(res / "particle_samples.gz"), ev)
    keys = dict(echo_level=9, read_in_mode=10, ecoOutput=0, analyze_flow=0, analyze_HBT=1,
                analyze_balance_function=0, analyze_ebe_yield=0, randomSeed=1,
                read_in_real_mixed_events=0, particle_monval=211, distinguish_isospin=1,
                resonance_weak_feed_down_flag=0, resonance_feed_down_flag=0,
                select_resonances_flag=0, net_particle_flag=0, flag_charge_dependence=0,
                event_buffer_size=5000, rapidity_shift=0.0, readRapidityShiftFromFile=0,
                long_comoving_boost=1, needed_number_of_pairs=1e18, invariant_radius_flag=0,
                azimuthal_flag=0, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=8, HBTrap_min=-1.0,
                HBTrap_max=1.0, qnpts=41, q_min=-0.15, q_max=0.15, hbt_mixed_partners=5)
    (tmp_path / "parameters.dat").write_text("".join("%s = %s\n" % kv for kv in keys.items()))
    proc = subprocess.run([EXE], cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-2000:]
    same = sum(int(l.split(":")[1]) for l in proc.stdout.splitlines()
               if l.startswith("[Info] number of pairs:"))
    mixed = sum(int(l.split(":")[1]) for l in proc.stdout.splitlines()
                if l.startswith("[Info] number of mixed pairs:"))
    o = orc.hist()
    assert (same, mixed) == (o["pairs_same"], o["pairs_mixed"])
    want_dir = tmp_path / "oracle"
    want_dir.mkdir()
    orc.write(str(want_dir))
    want = sorted(f for f in os.listdir(want_dir) if f.startswith("HBT_correlation"))
    got = sorted(f for f in os.listdir(res) if f.startswith("HBT_correlation"))
    assert got == want and len(want) == 4
    for f in want:
        compare_files((res / f).read_text(), (want_dir / f).read_text(), f)


CENTRAL = dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=9, KT_min=0.0, KT_max=1.0, n_Kphi=8,
               azimuthal_flag=1, invariant_radius_flag=0, long_comoving_boost=1,
               needed_number_of_pairs=1e18)


def oracle_mt(p, jobs, psi=None, seed=1, nmix=10):
    orc = oracle_lib.Oracle(number_of_mixed_events=nmix, seed=seed, **p)
    if psi is not None:
        orc.set_psi_ref(psi)
    for job in jobs:
        if job[0] == "same":
            orc.bin_same(job[1], nthreads=NTHREADS)
        else:
            orc.bin_mixed(job[1], job[2], nthreads=NTHREADS)
    h = orc.hist()
    anum = np.zeros_like(h["num"])
    L = oracle_lib.lib()
    L.orc_get_abs_num.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    L.orc_get_abs_num(orc._h, anum.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    h["abs_num"] = anum
    return h


@pytest.fixture(scope="module")
def central_group(host):
    ev = synth.central_pions(seed=1)
    a, b = synth.buffers(ev, 150000)[0]
    g = synth.subset(ev, a, b)
    psi = oracle_lib.event_plane_angle(g.px, g.py, 2)
    partners, angles = mixed_plan(host, 1, [g.n_events], 10)[0]
    jobs = buffer_jobs(g, partners, angles)
    return g, psi, jobs, oracle_mt(CENTRAL, jobs, psi)


def test_central_group_with_kphi_bins(central_group):
    """One central group (~150k particles, 1.1e10 same-event and 2.3e9
    mixed-event candidate pairs, 72 slots of 41^3 bins, psi_ref != 0) in one
    batched call: every count, denominator and pair counter identical to the
    oracle, sums within parity.RTOL; pairs on K_phi edges decided on the host
    as the reference decides them."""
    g, psi, jobs, o = central_group
    assert g.n_particles > 140000 and abs(psi) > 1e-3
    h, st = engine_hist(CENTRAL, jobs, psi)
    assert o["pairs_same"] > 1e10 and o["count"].sum() > 1e9
    parity.compare(h, o, q_scale=0.15)
    assert st["anomalies"] == o["anomalies"]
    assert st["tiles_same_kept"] < st["tiles_same"]


def _precision_errors(h, o, scale_q=0.15):
    """Per-bin errors of a reduced-precision form against the FP64 oracle:
    numerator |dnum| per pair and per sum of |cos|, relative error of bins
    with at least 2 pairs, mean-q error per pair."""
    cnt = o["count"]
    sel = cnt >= 2
    dn = np.abs(h["num"] - o["num"])
    out = dict(
        num_per_pair=float((dn[sel] / cnt[sel]).max()),
        num_per_abs_cos=float((dn[sel] / np.maximum(o["abs_num"][sel], 1e-300)).max()),
        num_rel_count_ge2=float((dn[sel] / np.maximum(np.abs(o["num"][sel]), 1e-300)).max()),
        q_per_pair=max(float((np.abs(h[k] - o[k])[sel] / cnt[sel]).max())
                       for k in ("q_out", "q_side", "q_long")))
    return out


# Stated bounds of the two reduced-precision forms, per pair of a bin: the
# cos(q.dx) numerator, and the q sums relative to the window Q = 0.15 GeV.
BOUNDS = {engine.PRECISION_FP32W: (1e-6, 1e-5), engine.PRECISION_DF64: (1e-11, 1e-11)}


@pytest.mark.parametrize("precision", [engine.PRECISION_FP32W, engine.PRECISION_DF64])
def test_central_group_precision_forms_against_the_oracle(central_group, precision):
    """The FP32-weight and double-float forms on the central group against
    the FP64 oracle: counts and denominators identical; per bin the numerator
    error is at most 1e-6 (FP32 weights) or 1e-11 (double-float) per pair,
    and the q sums at most 1e-5 or 1e-11 of the window per pair."""
    g, psi, jobs, o = central_group
    h, _ = engine_hist(CENTRAL, jobs, psi, precision=precision)
    for k in ("count", "den", "ctr_num", "ctr_den"):
        assert np.array_equal(np.asarray(h[k]), np.asarray(o[k])), k
    e = _precision_errors(h, o)
    b_num, b_q = BOUNDS[precision]
    assert e["num_per_pair"] <= b_num, e
    assert e["q_per_pair"] <= b_q * 0.15, e


def test_kaon_groups_precision_forms_against_the_oracle(host):
    """The precision configuration's K+ run (Poisson(250), oversample 100,
    three groups, 10 partners): FP64 form within parity.RTOL, FP32-weight
    and double-float forms within their per-pair bounds, counts identical."""
    ev = synth.central_kaons(seed=2)
    bufs = synth.buffers(ev, 25000)[:3]
    plans = mixed_plan(host, 1, [b - a for a, b in bufs], 10)
    jobs = []
    calls = []
    for (a, b), (partners, angles) in zip(bufs, plans):
        g = synth.subset(ev, a, b)
        bj = buffer_jobs(g, partners, angles)
        calls.append(bj)
        jobs += bj
    p = dict(CENTRAL, azimuthal_flag=0)
    o = oracle_mt(p, jobs)
    h, _ = engine_hist(p, jobs, calls=calls)
    parity.compare(h, o, q_scale=0.15)
    for precision, (b_num, b_q) in BOUNDS.items():
        h, _ = engine_hist(p, jobs, precision=precision, calls=calls)
        assert np.array_equal(h["count"], o["count"]) and np.array_equal(h["den"], o["den"])
        e = _precision_errors(h, o)
        assert e["num_per_pair"] <= b_num and e["q_per_pair"] <= b_q * 0.15, (precision, e)


@pytest.mark.parametrize("azimuthal", [0, 1])
def test_small_configuration_with_a_binding_cap(small_run, azimuthal):
    """The small configuration in full with needed_number_of_pairs = 1e6,
    which binds in the busiest K_T (x K_phi) slots within the first buffers:
    pairs are admitted in the reference's order (src/HBT_correlation.cpp
    :400-406, :651-655) through the batched kernels' count and order passes
    plus the pair-by-pair cut row: each buffer's same-event job alone, its
    mixed-event jobs together in their joint row order.  Counts,
    denominators and counters identical to the oracle's buffer loop; K_phi
    edges decided on the host take part in the order."""
    ev, bufs, _, jobs = small_run
    p = dict(SMALL, needed_number_of_pairs=1e6, azimuthal_flag=azimuthal, n_Kphi=4)
    orc = oracle_lib.Oracle(number_of_mixed_events=5, seed=1, **p)
    psis = []
    for a, b in bufs:
        g = synth.subset(ev, a, b)
        orc.process_buffer(g)
        psis.append(oracle_lib.event_plane_angle(g.px, g.py, 2) if azimuthal else None)
    o = orc.hist()
    eng = engine.Engine(device=0, **p)
    at = 0
    for (a, b), psi in zip(bufs, psis):
        nj = 1 + (b - a)
        if psi is not None:
            eng.set_psi_ref(psi)
        eng.bin_batch(jobs[at:at + nj])
        at += nj
    h = eng.hist()
    st = eng.stats()
    eng.close()
    assert st["ordered_passes"] > 0
    assert (o["ctr_num"] > 1e6).any() and (o["ctr_den"] > 1e6).any()
    parity.compare(h, o, q_scale=0.15)


def test_small_configuration_with_qinv_histograms(small_run):
    """invariant_radius_flag = 1 on the small configuration in one batched
    call: the q_inv bins are decided in FP32 with an error bound on the
    batched kernels (src/HBT_correlation.cpp:331-356, :595-607), pairs near a
    q_inv edge by the reference chain; q_inv counts and denominators and the
    3-D histograms identical to the oracle's, sums within parity.RTOL."""
    ev, bufs, _, jobs = small_run
    p = dict(SMALL, invariant_radius_flag=1)
    orc = oracle_lib.Oracle(number_of_mixed_events=5, seed=1, **p)
    for a, b in bufs:
        orc.process_buffer(synth.subset(ev, a, b))
    o = orc.hist()
    h, st = engine_hist(p, jobs)
    assert o["qinv_count"].sum() > 1e6 and o["qinv_den"].sum() > 1e6
    parity.compare(h, o, q_scale=0.15)


def test_central_group_with_qinv_and_kphi(central_group):
    """One central group with the q_inv histograms and 8 K_phi bins on the
    batched kernels (kernel 0): every count identical to the oracle's,
    sums within parity.RTOL."""
    g, psi, jobs, _ = central_group
    p = dict(CENTRAL, invariant_radius_flag=1)
    o = oracle_mt(p, jobs, psi)
    h, st = engine_hist(p, jobs, psi)
    assert o["qinv_count"].sum() > 1e9
    parity.compare(h, o, q_scale=0.15)


UNEVEN = dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=8,
              azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
              needed_number_of_pairs=1e18)


@pytest.fixture(scope="module")
def uneven_groups(host):
    """The first three ~50k-particle groups of the uneven-multiplicity
    workload (4096 pi+ events, multiplicities log-uniform in [20, 3000],
    sigma_xy = 1.2 N^(1/3) fm), 10 rotated partners per event."""
    ev = synth.uneven_pions(seed=3)
    bufs = synth.buffers(ev, 50000)[:3]
    plans = mixed_plan(host, 1, [b - a for a, b in bufs], 10)
    jobs = []
    for (a, b), (partners, angles) in zip(bufs, plans):
        jobs += buffer_jobs(synth.subset(ev, a, b), partners, angles)
    return jobs, oracle_mt(UNEVEN, jobs)


def _device_jobs(jobs):
    torch = pytest.importorskip("torch")

    def dev(cols):
        return [torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in cols]
    return [("same", dev(j[1])) if j[0] == "same" else ("mixed", dev(j[1]), dev(j[2]))
            for j in jobs]


def test_uneven_configuration_groups_in_one_batched_call(uneven_groups):
    """Three groups of the uneven-multiplicity configuration at full size
    (41^3 grid, 4 K_T bins) with every same-event and mixed-event list of
    them in one batched call, as the benchmark runs it: the FP64 form against
    the oracle (counts identical, sums within parity.RTOL); then the
    FP32-weight form, autotuned and launched twice from device arrays (the
    second launch replays the captured CUDA graph): counts exactly twice the
    oracle's, the numerator within 1e-6 and the q sums within 1e-5 x 0.15 GeV
    per pair."""
    jobs, o = uneven_groups
    assert o["pairs_same"] > 1e9 and o["count"].sum() > 1e8
    h, st = engine_hist(UNEVEN, jobs)
    parity.compare(h, o, q_scale=0.15)
    assert st["anomalies"] == o["anomalies"]

    djobs = _device_jobs(jobs)
    eng = engine.Engine(device=0, precision=engine.PRECISION_FP32W, **UNEVEN)
    eng.autotune(djobs)
    eng.set_tuning(use_graph=1)
    eng.bin_batch(djobs, device=True)
    eng.bin_batch(djobs, device=True)
    h = eng.hist()
    st = eng.stats()
    eng.close()
    assert st["graph_replays"] + st["graph_captures"] >= 1
    o2 = {k: 2 * np.asarray(o[k]) for k in ("count", "den", "ctr_num", "ctr_den", "num",
                                            "abs_num", "q_out", "q_side", "q_long")}
    for k in ("count", "den", "ctr_num", "ctr_den"):
        assert np.array_equal(np.asarray(h[k]), o2[k]), k
    e = _precision_errors(h, o2)
    assert e["num_per_pair"] <= 1e-6 and e["q_per_pair"] <= 1e-5 * 0.15, e
