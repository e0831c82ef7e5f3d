"""Benchmark of the GB300 HBT pair-binning engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload central|medium|small] [--precision fp64|fp32w|df64]
                    [--no-uneven] [--no-serving] [--serving-jobs J]

Workload "central" (default): 1000 pi+ events, multiplicity Poisson(1500),
emission source sigma_xy = 7 fm, tau0 = 12 fm/c, oversample factor 100
(event_buffer_size = 150000 -> ~150k particles per group), 41^3 q grid on
[-0.15, 0.15] GeV, 8 K_T bins on [0, 1] GeV x 8 K_phi bins, 10 rotated
mixed-event partners per event, no pair cap (needed_number_of_pairs = 1e18).
Synthetic, seeded data of those shapes (no public dataset exists).

One step = one oversample group through the hot path: its same-event pairs
i < j plus every event's mixed pairs against its 10 partners.  The unit of
work is the reference's candidate pair (n(n-1)/2 same-event plus n1*n2
mixed-event pairs).  `value` times the device-resident entry points with
CUDA events on the engine's stream; `e2e` times the host-buffer C-ABI calls
(pinned host arrays copied in, histograms copied back every step) with the
host clock.  The L2 is flushed (256 MB write) between timed steps.

Two more legs are reported in the same JSON line.  "uneven": the
uneven-multiplicity workload (4096 events, log-uniform multiplicity in
[20, 3000], ~50k-particle groups, 10 partners, 41^3 grid, 4 K_T bins), all
groups and partners in one batched launch per step, FP64 and FP32 weights,
against the plain FP64 reference-chain kernel on a sample of groups.
"serving": a Poisson stream of requests at 200 jobs/s (10-500 events each,
mu in [50, 2000], pi+ or K+, qnpts in {21, 41, 61}, q_max in [0.1, 0.3] GeV,
2-8 K_T bins; each event its own same-event list, one rotated partner per
event) through the serving loop, with p50 / p99 request latency and pairs/s,
against the plain per-job path.

"ingest": the sample reader on a 200-event central-like gzip file, the
line-by-line reader against the block reader (parallel parse) and the
binary sidecar, plus the writer on the central histograms.  "average": the
event averaging of HBT files over event folders against a restatement of
the reference's averaging script.

--impl reference times the reference algorithm on the host cores (the CPU
oracle, multi-threaded) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

# The reference's per-pair chain (src/HBT_correlation.cpp:311-458), counted
# from its code, per stage: FP64 add/mul, divide, square root, cos, FP64
# atomics (histogram adds).  Stages: all pairs; K_T passed; q_out passed;
# q_side passed; binned.
STAGE_COUNTS_SAME = ((11, 0, 0, 0, 0), (8, 3, 1, 0, 0), (4, 1, 0, 0, 0), (7, 3, 1, 0, 0),
                     (13, 1, 0, 1, 5))
STAGE_COUNTS_MIXED = ((11, 0, 0, 0, 0), (8, 3, 1, 0, 0), (4, 1, 0, 0, 0), (7, 3, 1, 0, 0),
                      (1, 1, 0, 0, 1))
STAGE_OPS_SAME = tuple(sum(c[:4]) for c in STAGE_COUNTS_SAME)
STAGE_OPS_MIXED = tuple(sum(c[:4]) for c in STAGE_COUNTS_MIXED)

# FP64-pipe instructions (warp-level, ncu smsp__inst_executed_pipe_fp64.sum)
# that k_persistent_same executes per binned same-event pair in the FP64
# form, all of the kernel's FP64 work (values, undecided pairs, tile loads)
# divided by the pairs it bins: measured on one central group launch,
# profiles/k_persistent_same_fp64_central.md.
FP64_WARP_INST_PER_BINNED_PAIR = 1899528993 / 1942004247
# DRAM bytes (read + write) of one k_persistent_same launch on a central
# group, FP64 form, same-event items in momentum-region order (the default
# hbt_tuning.order_items): profiles/k_persistent_same_fp64_central.md.
CENTRAL_SAME_DRAM_BYTES = 187360768 + 331953920


def workload_params(name: str) -> dict:
    if name == "small":
        return dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0,
                    n_Kphi=8, azimuthal_flag=0, invariant_radius_flag=0,
                    long_comoving_boost=1, needed_number_of_pairs=1e18)
    return dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=9, KT_min=0.0, KT_max=1.0, n_Kphi=8,
                azimuthal_flag=1, invariant_radius_flag=0, long_comoving_boost=1,
                needed_number_of_pairs=1e18)


def make_workload(name: str, seed: int = 1, max_groups: int | None = None):
    """Groups of (same-event SoA, [(list1 SoA4, list2 SoA4) per event])."""
    from hadronic_afterburner_toolkit_gb300 import synth
    if name == "small":
        ev = synth.small_pions(seed=seed)
        buf, nmix = 5000, 5
    elif name == "kaons":
        # the precision configuration's K+ run: oversample factor 100
        ev = synth.central_kaons(seed=seed + 1)
        buf, nmix = 25000, 10
    elif name == "medium":
        # the central workload's events and grid, 30x oversampling (profiling)
        ev = synth.central_pions(n_events=300, seed=seed)
        buf, nmix = 45000, 10
    else:
        ev = synth.central_pions(seed=seed)
        buf, nmix = 150000, 10
    rng = np.random.default_rng(seed + 1000)
    groups = []
    for (a, b) in synth.buffers(ev, buf):
        if max_groups is not None and len(groups) >= max_groups:
            break
        g = synth.subset(ev, a, b)
        cols = [np.ascontiguousarray(getattr(g, k)) for k in
                ("px", "py", "pz", "E", "x", "y", "z", "t")]
        nev = g.n_events
        mixed = []
        for e in range(nev):
            lo, hi = g.offsets[e], g.offsets[e + 1]
            l1 = [c[lo:hi].copy() for c in cols[:4]]
            parts = []
            for _ in range(nmix):
                m = int(rng.integers(nev))
                while m == e and nev > 1:
                    m = int(rng.integers(nev))
                phi = rng.uniform(0, 2 * np.pi)
                c, s = np.cos(phi), np.sin(phi)
                mlo, mhi = g.offsets[m], g.offsets[m + 1]
                px, py = cols[0][mlo:mhi], cols[1][mlo:mhi]
                parts.append((px * c - py * s, px * s + py * c, cols[2][mlo:mhi], cols[3][mlo:mhi]))
            l2 = [np.ascontiguousarray(np.concatenate([p[f] for p in parts])) for f in range(4)]
            mixed.append((l1, l2))
        groups.append((cols, mixed))
    return groups


def group_pairs(group) -> int:
    cols, mixed = group
    n = cols[0].size
    return n * (n - 1) // 2 + sum(l1[0].size * l2[0].size for l1, l2 in mixed)


def survival_fractions(group, p, sample=400_000, seed=7):
    """Stage survival fractions of the same-event chain on sampled pairs
    (K_T pass, q_out pass, q_side pass, binned), FP64 numpy."""
    cols = group[0]
    n = cols[0].size
    rng = np.random.default_rng(seed)
    i = rng.integers(0, n, sample)
    j = rng.integers(0, n, sample)
    keep = i != j
    i, j = i[keep], j[keep]
    px, py, pz, E = cols[0], cols[1], cols[2], cols[3]
    Kx = 0.5 * (px[i] + px[j]); Ky = 0.5 * (py[i] + py[j])
    Kz = 0.5 * (pz[i] + pz[j]); KE = 0.5 * (E[i] + E[j])
    Kp2 = Kx * Kx + Ky * Ky
    kt = (Kp2 >= p["KT_min"] ** 2) & (Kp2 <= p["KT_max"] ** 2)
    Kp = np.sqrt(Kp2)
    qx = px[i] - px[j]; qy = py[i] - py[j]; qz = pz[i] - pz[j]; qE = E[i] - E[j]
    dq = (p["q_max"] - p["q_min"]) / (p["qnpts"] - 1)
    lo, hi = p["q_min"] - dq / 2 + 1e-8, p["q_max"] + dq / 2 - 1e-8
    with np.errstate(all="ignore"):
        qo = (qx * Kx + qy * Ky) / Kp
        qs = (qy * Kx - qx * Ky) / Kp
        Mt = np.sqrt(KE * KE - Kz * Kz)
        ql = (KE / Mt) * (qz - (Kz / KE) * qE)
    o = kt & (qo >= lo) & (qo <= hi)
    s = o & (qs >= lo) & (qs <= hi)
    b = s & (ql >= lo) & (ql <= hi)
    m = float(i.size)
    return (1.0, kt.sum() / m, o.sum() / m, s.sum() / m, b.sum() / m)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(k)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def measure_fp64_peak() -> dict:
    """Live FP64 / FP32 FMA issue rate on this GPU (hbt_probe)."""
    import ctypes
    from hadronic_afterburner_toolkit_gb300 import build
    L = ctypes.CDLL(build.build_probe())
    out = {}
    for name, fn, iters in (("fp64", L.hbt_probe_fp64, 1 << 14), ("fp32", L.hbt_probe_fp32, 1 << 16)):
        fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                       ctypes.POINTER(ctypes.c_double)]
        ms, fl = ctypes.c_float(), ctypes.c_double()
        best = 0.0
        for _ in range(3):
            if fn(152 * 16, iters, ctypes.byref(ms), ctypes.byref(fl)) != 0:
                raise RuntimeError("probe failed")
            best = max(best, fl.value / (ms.value * 1e-3))
        out[name + "_tflops"] = best / 1e12
    # FP64 divide, square root and cos, each with one add (the reference
    # chain's other operations)
    fn = L.hbt_probe_op64
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                   ctypes.POINTER(ctypes.c_double)]
    for key, op, iters in (("div_gops", 0, 1 << 11), ("sqrt_gops", 1, 1 << 11),
                           ("cos_gops", 2, 1 << 10)):
        ms, ops = ctypes.c_float(), ctypes.c_double()
        best = 0.0
        for _ in range(3):
            if fn(op, 152 * 8, iters, ctypes.byref(ms), ctypes.byref(ops)) != 0:
                raise RuntimeError("probe failed")
            best = max(best, ops.value / (ms.value * 1e-3))
        out[key] = best / 1e9
    # scattered FP64 atomic adds: over 32 MB (L2-resident, the atomic units'
    # rate) and over 256 MB (beyond L2, like the whole histogram)
    fn = L.hbt_probe_atomic
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                   ctypes.POINTER(ctypes.c_double)]
    for key, log2 in (("atomic_gops_l2", 22), ("atomic_gops_256mb", 25)):
        ms, ops = ctypes.c_float(), ctypes.c_double()
        best = 0.0
        for _ in range(3):
            if fn(152 * 16, 256, log2, ctypes.byref(ms), ctypes.byref(ops)) != 0:
                raise RuntimeError("probe failed")
            best = max(best, ops.value / (ms.value * 1e-3))
        out[key] = best / 1e9
    return out


def step_mix(group) -> float:
    """Share of same-event pairs among a group's candidate pairs."""
    cols, mixed = group
    n = cols[0].size
    same = n * (n - 1) / 2
    return same / (same + sum(l1[0].size * l2[0].size for l1, l2 in mixed))


def oracle_sample(orc, group, same_pairs, mixed_pairs, first_row=0, first_event=0):
    """Times the oracle (one host thread) on a bounded sample of one group:
    the same-event pairs of a contiguous slice of its list, then mixed
    pairs of its events from `first_event` on (the last event's list 1 cut
    short to fit).  Returns (pairs, seconds)."""
    cols, mixed = group
    n = cols[0].size
    ns = int(min(n - first_row, max(2, round(np.sqrt(2.0 * same_pairs)))))
    pieces, acc = [], 0
    e = first_event % len(mixed)
    while acc < mixed_pairs and len(pieces) < len(mixed):
        l1, l2 = mixed[e]
        n1 = int(min(l1[0].size, max(1, round((mixed_pairs - acc) / l2[0].size))))
        pieces.append(([c[:n1] for c in l1], l2))
        acc += n1 * l2[0].size
        e = (e + 1) % len(mixed)
    t0 = time.perf_counter()
    orc.bin_same([c[first_row:first_row + ns] for c in cols])
    for l1, l2 in pieces:
        orc.bin_mixed(l1, l2)
    dt = time.perf_counter() - t0
    return ns * (ns - 1) // 2 + acc, dt


def cpu_baseline(group, p, target_s=12.0) -> dict:
    """The oracle (sequential restatement of the reference loops) on one
    host core, on a bounded sample of the group with the step's mix of
    same-event and mixed-event pairs."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    orc = oracle_lib.Oracle(**p)
    f = step_mix(group)
    pairs, dt = oracle_sample(orc, group, 2e6 * f, 2e6 * (1 - f))  # calibration
    rate = pairs / max(dt, 1e-6)
    pairs, dt = oracle_sample(orc, group, rate * target_s * f, rate * target_s * (1 - f))
    return {"value": pairs / dt, "unit": "pairs/s", "cores": 1, "kind": "port",
            "sample": "one host core: same-event pairs of a %.3g-pair slice of one ~%dk-particle "
                      "group and mixed pairs of its events, %.1f%% same-event as in the step "
                      "(%.3g pairs, %.1f s)" % (pairs * f, group[0][0].size // 1000, 100 * f,
                                                pairs, dt)}


_REF = {}


def _ref_init(workload):
    """Worker of the reference arm: the workload's first group and one
    oracle context, built once per process."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    _REF["group"] = make_workload(workload, max_groups=1)[0]
    _REF["orc"] = oracle_lib.Oracle(**workload_params(workload))


def _ref_task(args):
    w, nproc, same_pairs, mixed_pairs = args
    cols, mixed = _REF["group"]
    n = cols[0].size
    row = (w * n) // nproc
    row = min(row, max(0, n - int(np.sqrt(2.0 * same_pairs)) - 1))
    return oracle_sample(_REF["orc"], _REF["group"], same_pairs, mixed_pairs, row,
                         (w * len(mixed)) // nproc)


def run_reference(args) -> None:
    """The reference arm: the reference's CPU algorithm (the oracle port:
    the reference binary is built for this container's x86 host and its
    sources do not travel) on every host core as independent processes,
    one oracle per core, each step a bounded sample of the workload's group
    with the step's share of same-event pairs.  The timed steps add up to
    at least 10 s of sampling."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    nproc = os.cpu_count() or 1
    p = workload_params(args.workload)
    group = make_workload(args.workload, max_groups=1)[0]
    f = step_mix(group)
    ctx = mp.get_context("spawn")
    with ctx.Pool(nproc, initializer=_ref_init, initargs=(args.workload,)) as pool:
        # one process alone: the per-core rate, and the sample size
        pairs, dt = pool.apply(_ref_task, ((0, nproc, 4e6 * f, 4e6 * (1 - f)),))
        pairs, dt = pool.apply(_ref_task, ((0, nproc, 4e7 * f, 4e7 * (1 - f)),))
        per_core = pairs / dt
        step_s = max(0.5, 10.0 / max(1, args.steps))
        budget = per_core * step_s
        steps = []
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_ref_task, [(w, nproc, budget * f, budget * (1 - f))
                                       for w in range(nproc)])
            wall = time.perf_counter() - t0
            if k >= args.warmup:
                steps.append((sum(r[0] for r in res), max(r[1] for r in res), wall))
    v = sum(s[0] for s in steps) / sum(s[1] for s in steps)
    timed = sum(s[1] for s in steps)
    sample = ("%d processes, one oracle each, %d timed steps of %.2g s: same-event pairs of a "
              "slice of one ~%dk-particle group and mixed pairs of its events, %.1f%% "
              "same-event as in the GPU step; %.3g pairs per step in all, %.1f s timed"
              % (nproc, len(steps), step_s, group[0][0].size // 1000, 100 * f,
                 steps[-1][0], timed))
    line = {"impl": "reference", "metric": "candidate pairs binned per second (same + mixed event)",
            "value": v, "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "ms_per_step": 1e3 * timed / len(steps),
            "config": {"workload": args.workload, "reference_arm": "CPU oracle port of the "
                       "reference pair loops, one process per host core"},
            "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": nproc, "kind": "port",
                             "processes": nproc, "per_core_value": per_core,
                             "sample": sample},
            "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


UNEVEN_PARAMS = dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0,
                     n_Kphi=8, azimuthal_flag=0, invariant_radius_flag=0,
                     long_comoving_boost=1, needed_number_of_pairs=1e18)


def allreduce_hist(h: dict, device=None) -> dict:
    """Sums a histogram dict (Engine.hist()) over the ranks of the default
    process group: the replicas' one reduction when bench.py runs under
    torchrun.  Counts travel as int64 (exact), sums as float64."""
    import torch
    import torch.distributed as dist
    from hadronic_afterburner_toolkit_gb300 import replicas
    out = dict(h)
    for keys, dtype in ((replicas.COUNT_KEYS, torch.int64), (replicas.SUM_KEYS, torch.float64)):
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
    sc = [k for k in replicas.SCALAR_KEYS if k in h]
    if sc:
        t = torch.tensor([int(h[k]) for k in sc], dtype=torch.int64)
        if device is not None:
            t = t.to(device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        for k, v in zip(sc, t.cpu().tolist()):
            out[k] = int(v)
    return out


def make_uneven(seed: int = 3, group_particles: int = 50_000, nmix: int = 10):
    """The uneven-multiplicity workload: 4096 pi+ events with log-uniform
    multiplicities in [20, 3000] (sigma_xy = 1.2 N^(1/3) fm), oversample
    groups of ~50k particles, 10 rotated partners per event drawn inside
    its group.  Returns the groups in make_workload's layout."""
    from hadronic_afterburner_toolkit_gb300 import synth
    ev = synth.uneven_pions(seed=seed)
    rng = np.random.default_rng(seed + 1000)
    groups = []
    for (a, b) in synth.buffers(ev, group_particles):
        g = synth.subset(ev, a, b)
        cols = [np.ascontiguousarray(getattr(g, k)) for k in
                ("px", "py", "pz", "E", "x", "y", "z", "t")]
        mixed = []
        for e in range(g.n_events):
            lo, hi = g.offsets[e], g.offsets[e + 1]
            ms = [int(m) for m in rng.integers(0, g.n_events, size=nmix)]
            ms = [(m + 1) % g.n_events if (m == e and g.n_events > 1) else m for m in ms]
            phis = rng.uniform(0, 2 * np.pi, size=nmix)
            parts = []
            for m, phi in zip(ms, phis):
                c, s = np.cos(phi), np.sin(phi)
                mlo, mhi = g.offsets[m], g.offsets[m + 1]
                px, py = cols[0][mlo:mhi], cols[1][mlo:mhi]
                parts.append((px * c - py * s, px * s + py * c, cols[2][mlo:mhi],
                              cols[3][mlo:mhi]))
            l1 = [c[lo:hi] for c in cols[:4]]
            l2 = [np.concatenate([pp[f] for pp in parts]) for f in range(4)]
            mixed.append((l1, l2))
        groups.append((cols, mixed))
    return groups


def uneven_leg(E, torch, dev, stream, flush, local, steps=2) -> dict:
    """All groups and partners of the uneven workload in one batched
    persistent launch per step (FP64 and FP32 weights), against the plain
    FP64 reference-chain kernel called list by list on a sample of groups."""
    groups = make_uneven()
    dgroups = [([torch.from_numpy(c).to(dev) for c in cols],
                [([torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in l1],
                  [torch.from_numpy(x).to(dev) for x in l2]) for l1, l2 in mixed])
               for cols, mixed in groups]
    total_pairs = sum(group_pairs(g) for g in groups)
    jobs = []
    for dc, dm in dgroups:
        jobs.append(("same", dc))
        jobs += [("mixed", l1, l2) for l1, l2 in dm]

    def timed(fn, n):
        ms = []
        for k in range(n):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms

    out = {"events": 4096, "groups": len(groups), "group_particles": "~50k",
           "mixed_partners": 10, "pairs_per_step": total_pairs, "qnpts": 41, "n_KT_bins": 4}
    for label, prec in (("batched-fp64", E.PRECISION_FP64), ("batched-fp32w", E.PRECISION_FP32W),
                        ("batched-df64", E.PRECISION_DF64)):
        eng = E.Engine(device=local, precision=prec, kernel=E.KERNEL_SCREENED, **UNEVEN_PARAMS)
        eng.set_stream(stream.cuda_stream)
        default_ms = statistics.median(timed(lambda: eng.bin_batch(jobs, device=True), 2))
        # autotune on a sample of the batch, then warm up: the second launch
        # of the same batch is captured into a CUDA graph, later ones re-launch it
        tuned, tune_ms = eng.autotune(jobs, max_pairs=4e9)
        timed(lambda: eng.bin_batch(jobs, device=True), 2)
        st0 = eng.stats()
        ms = timed(lambda: eng.bin_batch(jobs, device=True), steps)
        st1 = eng.stats()
        out[label] = {"value": total_pairs / (statistics.median(ms) * 1e-3), "unit": "pairs/s",
                      "ms_per_step": statistics.median(ms), "steps": steps,
                      "jobs_per_launch": len(jobs), "tuning": tuned,
                      "ms_per_step_default_tuning": default_ms,
                      "graph_replays_timed": st1["graph_replays"] - st0["graph_replays"]}
        eng.close()
    # plain: the reference chain on every pair, one call per list, on the
    # first groups (about 3e9 pairs)
    eng = E.Engine(device=local, precision=E.PRECISION_FP64, kernel=E.KERNEL_REFERENCE_CHAIN,
                   **UNEVEN_PARAMS)
    eng.set_stream(stream.cuda_stream)
    n_sample, acc = 0, 0
    for g in groups:
        if acc >= 3e9:
            break
        acc += group_pairs(g)
        n_sample += 1

    def plain_run():
        for dc, dm in dgroups[:n_sample]:
            eng.bin_same(dc, device=True)
            for l1, l2 in dm:
                eng.bin_mixed(l1, l2, device=True)

    timed(lambda: eng.bin_same(dgroups[0][0], device=True), 1)
    ms = timed(plain_run, 1)
    out["plain-fp64"] = {"value": acc / (ms[0] * 1e-3), "unit": "pairs/s",
                         "sample": "%d of %d groups (%.3g pairs)" % (n_sample, len(groups), acc),
                         "kernel": "reference chain, one launch per list"}
    eng.close()
    for k in ("batched-fp64", "batched-fp32w", "batched-df64"):
        out[k]["speedup_vs_plain"] = out[k]["value"] / out["plain-fp64"]["value"]
    return out


def small_leg(E, torch, dev, stream, flush, local, steps=3) -> dict:
    """The reference's CPU-runnable case (100 pi+ events,
    Poisson(500), oversample 10 -> 10 groups of ~5k particles, 5 rotated
    partners, 41^3 grid, 4 K_T bins): every group and partner in one batched
    FP64 launch per step, against the oracle on one host core."""
    groups = make_workload("small")
    p = workload_params("small")
    dgroups = [([torch.from_numpy(c).to(dev) for c in cols],
                [([torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in l1],
                  [torch.from_numpy(x).to(dev) for x in l2]) for l1, l2 in mixed])
               for cols, mixed in groups]
    jobs = []
    for dc, dm in dgroups:
        jobs.append(("same", dc))
        jobs += [("mixed", l1, l2) for l1, l2 in dm]
    total = sum(group_pairs(g) for g in groups)
    eng = E.Engine(device=local, precision=E.PRECISION_FP64, kernel=E.KERNEL_SCREENED, **p)
    eng.set_stream(stream.cuda_stream)
    ms = []
    for k in range(3 + steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.bin_batch(jobs, device=True)
        e1.record(stream)
        e1.synchronize()
        if k >= 3:
            ms.append(e0.elapsed_time(e1))
    eng.close()
    value = total / (statistics.median(ms) * 1e-3)
    cpu = cpu_baseline(groups[0], p, target_s=3.0)
    return {"events": 100, "groups": len(groups), "pairs_per_step": total,
            "jobs_per_launch": len(jobs), "value": value, "unit": "pairs/s",
            "ms_per_step": statistics.median(ms), "steps": steps,
            "cpu_oracle_pairs_per_s": cpu["value"], "cpu_cores": 1,
            "speedup_vs_cpu_core": value / cpu["value"]}


INGEST_PARAMS = """echo_level = 0
read_in_mode = 10
read_in_real_mixed_events = 0
particle_monval = 211
resonance_weak_feed_down_flag = 0
resonance_feed_down_flag = 0
event_buffer_size = 150000
rapidity_shift = 0.0
"""


DROPIN_PARAMS = """echo_level = 9
read_in_mode = 10
ecoOutput = 0
analyze_flow = 0
analyze_HBT = 1
analyze_balance_function = 0
analyze_ebe_yield = 0
randomSeed = 1
read_in_real_mixed_events = 0
particle_monval = 211
distinguish_isospin = 1
resonance_weak_feed_down_flag = 0
resonance_feed_down_flag = 0
select_resonances_flag = 0
net_particle_flag = 0
flag_charge_dependence = 0
rapidity_shift = 0.0
readRapidityShiftFromFile = 0
long_comoving_boost = 1
needed_number_of_pairs = 1e18
invariant_radius_flag = 0
KT_min = 0.0
KT_max = 1.0
n_Kphi = 8
HBTrap_min = -1.0
HBTrap_max = 1.0
qnpts = 41
q_min = -0.15
q_max = 0.15
"""


def dropin_leg(seed: int = 1) -> dict:
    """The drop-in executable end to end (lib/hbt_afterburner.e: read the
    gzip samples, bin every buffer - its same-event list and every event's
    rotated partners in one batched call - and write the reference's
    HBT_correlation_function files) on the small configuration (100 pi+
    events, Poisson(500), buffers of 5000, 5 partners, 4 K_T bins) and on
    one central buffer (100 events of Poisson(1500), ~150k particles, 10
    partners, 8 K_T x 8 K_phi bins).  Against the oracle's restatement of
    the reference's buffer loop and writer on one host core on the small
    configuration (the whole run)."""
    from hadronic_afterburner_toolkit_gb300 import synth
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    exe = os.path.join(REPO, "hadronic_afterburner_toolkit_gb300", "lib", "hbt_afterburner.e")
    out = {}
    cases = (("small", synth.small_pions(seed=seed), 5000, 5, 5, 0),
             ("central_buffer", synth.central_pions(n_events=100, seed=seed), 150000, 10, 9, 1))
    for name, ev, buf, nmix, nkt, az in cases:
        with tempfile.TemporaryDirectory() as work:
            res = os.path.join(work, "results")
            os.makedirs(res)
            synth.write_mode10(os.path.join(res, "particle_samples.gz"), ev)
            with open(os.path.join(work, "parameters.dat"), "w") as f:
                f.write(DROPIN_PARAMS + "event_buffer_size = %d\nn_KT = %d\nazimuthal_flag = %d\n"
                        "hbt_mixed_partners = %d\n" % (buf, nkt, az, nmix))
            t0 = time.perf_counter()
            proc = subprocess.run([exe], cwd=work, capture_output=True, text=True, timeout=600)
            wall = time.perf_counter() - t0
            if proc.returncode != 0:
                raise RuntimeError("drop-in failed: " + proc.stderr[-500:])
            pairs = sum(int(l.split(":")[1]) for l in proc.stdout.splitlines()
                        if l.startswith("[Info] number of") and "pairs:" in l)
            files = [f for f in os.listdir(res) if f.startswith("HBT_correlation")]
            r = {"particles": ev.n_particles, "buffers": len(synth.buffers(ev, buf)),
                 "pairs": pairs, "wall_s": wall, "pairs_per_s": pairs / wall,
                 "files_written": len(files)}
            if name == "small":
                # the oracle's buffer loop and writer, one host core
                p = dict(workload_params("small"), n_KT=nkt)
                orc = oracle_lib.Oracle(number_of_mixed_events=nmix, seed=1, **p)
                t0 = time.perf_counter()
                for a, b in synth.buffers(ev, buf):
                    orc.process_buffer(synth.subset(ev, a, b))
                os.makedirs(os.path.join(work, "oracle"))
                orc.write(os.path.join(work, "oracle"))
                cpu = time.perf_counter() - t0
                r.update(cpu_oracle_s=cpu, cpu_cores=1, speedup_vs_cpu_core=cpu / wall)
            out[name] = r
    return out


def capped_leg(E, torch, dev, dgroups, groups, p, local, uncapped_ms, cap=3e7, n_groups=3):
    """The central workload at the reference's default pair cap,
    needed_number_of_pairs = 3e7 (parameters.dat), which binds in the first
    group: every job runs the two passes of ordered cap admission (count
    survivors per row, admit the rows before each slot's cut) on the batched
    kernels, and the cut rows pair by pair in the reference's order: the
    same-event job alone, the group's mixed-event jobs together in their
    joint row order.  Later groups find the busiest slots full; the passes'
    tile cull skips tile pairs whose pairs can reach only full slots.
    Device-resident inputs, CUDA events around each group."""
    eng = E.Engine(device=local, **dict(p, needed_number_of_pairs=cap))
    stream = torch.cuda.Stream(device=dev)
    eng.set_stream(stream.cuda_stream)
    ms, prs = [], 0
    for g in range(min(n_groups, len(dgroups))):
        dc, dm = dgroups[g]
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        eng.bin_batch([("same", dc)] + [("mixed", l1, l2) for l1, l2 in dm], device=True)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        prs += group_pairs(groups[g])
    ctr = eng.counters()
    st = eng.stats()
    eng.close()
    return {"needed_number_of_pairs": cap, "groups": len(ms), "ms_per_group": ms,
            "pairs_per_s": prs / (sum(ms) * 1e-3),
            "uncapped_ms_per_group": uncapped_ms,
            "first_group_vs_uncapped": ms[0] / uncapped_ms,
            "slots_at_cap": int((ctr["num"] > cap).sum()),
            "ordered_passes": st["ordered_passes"],
            "path": "count and order passes on the batched screened kernels (tile pairs "
                    "reaching only full slots skipped), cut rows by the pair-order kernel; "
                    "same-event job alone, mixed-event jobs together"}


def ingest_leg(n_events: int = 200, seed: int = 3) -> dict:
    """The reader (read_in_mode 10: gzip text, ~100 oversampled events per
    150k-particle buffer as on the central workload): the line-by-line
    reader (strtod per number, the reference's reading rule) against the
    block reader (inflate on its own thread, parallel from_chars parse and
    boost on all host threads) and the binary sidecar (written on a first
    pass, replayed after); all give bit-identical particles
    (tests/test_host_cpu.py).  text_MB_per_s counts the bytes each source
    read (text, or the sidecar's records)."""
    import ctypes
    from hadronic_afterburner_toolkit_gb300 import build, synth
    L = ctypes.CDLL(build.build_host())
    L.hbt_host_time_reader.restype = ctypes.c_int
    L.hbt_host_time_reader.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                       ctypes.POINTER(ctypes.c_char_p),
                                       ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64)]
    d = tempfile.mkdtemp(prefix="hbt_ingest_")
    res = os.path.join(d, "results")
    os.makedirs(res)
    ev = synth.central_pions(n_events=n_events, seed=seed)
    synth.write_mode10(os.path.join(res, "particle_samples.gz"), ev)
    pfile = os.path.join(d, "parameters.dat")
    with open(pfile, "w") as f:
        f.write(INGEST_PARAMS)
    out = {"events": n_events, "particles": int(ev.px.size),
           "gz_bytes": os.path.getsize(os.path.join(res, "particle_samples.gz")),
           "host_threads": os.cpu_count()}
    for label, args, reps in (("line-reader", ["hbt_fast_reader=0"], 2),
                              ("block-reader", ["hbt_fast_reader=1"], 2),
                              ("block-reader-writing-cache", ["hbt_binary_cache=1"], 1),
                              ("binary-cache-replay", ["hbt_binary_cache=1"], 2)):
        best = None
        for _ in range(reps):
            argv = (ctypes.c_char_p * len(args))(*[a.encode() for a in args])
            sec, npart, nbytes = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
            rc = L.hbt_host_time_reader(pfile.encode(), res.encode(), len(args), argv,
                                        ctypes.byref(sec), ctypes.byref(npart), ctypes.byref(nbytes))
            if rc != 0:
                raise RuntimeError("reader failed")
            if best is None or sec.value < best[0]:
                best = (sec.value, npart.value, nbytes.value)
        out[label] = {"seconds": best[0], "particles_per_s": best[1] / best[0],
                      "text_MB_per_s": best[2] / best[0] / 1e6}
    # the writer: the central workload's 64 files (9 K_T edges x 8 K_phi,
    # 41^3 rows each, ~408 MB of text) from random histograms
    L.hbt_host_write.restype = ctypes.c_int
    _PD = ctypes.POINTER(ctypes.c_double)
    _PU = ctypes.POINTER(ctypes.c_uint64)
    from hadronic_afterburner_toolkit_gb300 import engine as E
    L.hbt_host_write.argtypes = [ctypes.POINTER(E.HbtParams), ctypes.c_char_p,
                                 ctypes.c_int32] + [_PD] * 10 + [_PU] * 4
    hp = E.HbtParams(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=9, KT_min=0.0, KT_max=1.0,
                     n_Kphi=8, azimuthal_flag=1, invariant_radius_flag=0)
    nb = 72 * 41 ** 3
    rng = np.random.default_rng(1)
    arr = [rng.integers(0, 100, nb).astype(float)] + [rng.normal(0, 1, nb) for _ in range(4)] + \
          [rng.integers(0, 200, nb).astype(float)] + [np.zeros(9 * 41) for _ in range(4)]
    ctr = [np.full(72, 1000, np.uint64), np.full(72, 1200, np.uint64), np.zeros(9, np.uint64),
           np.zeros(9, np.uint64)]
    wdir = os.path.join(d, "written")
    os.makedirs(wdir)
    t0 = time.perf_counter()
    rc = L.hbt_host_write(ctypes.byref(hp), wdir.encode(), 0, *[a.ctypes.data_as(_PD) for a in arr],
                          *[c.ctypes.data_as(_PU) for c in ctr])
    tw = time.perf_counter() - t0
    wbytes = sum(os.path.getsize(os.path.join(wdir, f)) for f in os.listdir(wdir))
    out["writer"] = {"ok": rc == 0, "files": len(os.listdir(wdir)), "MB": wbytes / 1e6,
                     "seconds": tw, "MB_per_s": wbytes / 1e6 / tw}
    out["speedup"] = out["line-reader"]["seconds"] / out["block-reader"]["seconds"]
    out["speedup_cached"] = (out["line-reader"]["seconds"] /
                             out["binary-cache-replay"]["seconds"])
    import shutil
    shutil.rmtree(d, ignore_errors=True)
    return out


def average_leg(n_events: int = 12, seed: int = 11) -> dict:
    """Event averaging of the HBT files over event folders: 12 UrQMD*
    folders, each with the 4 files of a 21^3 grid and 5 K_T edges
    (9261 rows x 5 columns per file, written by the drop-in's writer from
    random histograms): hbt_host_average_events on all host threads against
    the CPU restatement of the reference's averaging script (numpy.loadtxt /
    savetxt, oracle/average_events.py)."""
    import ctypes
    import shutil
    from hadronic_afterburner_toolkit_gb300 import build, engine as E
    L = ctypes.CDLL(build.build_host())
    _PD = ctypes.POINTER(ctypes.c_double)
    _PU = ctypes.POINTER(ctypes.c_uint64)
    L.hbt_host_write.restype = ctypes.c_int
    L.hbt_host_write.argtypes = [ctypes.POINTER(E.HbtParams), ctypes.c_char_p,
                                 ctypes.c_int32] + [_PD] * 10 + [_PU] * 4
    L.hbt_host_average_events.restype = ctypes.c_int
    L.hbt_host_average_events.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32]
    d = tempfile.mkdtemp(prefix="hbt_avg_")
    work = os.path.join(d, "work")
    hp = E.HbtParams(qnpts=21, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0,
                     n_Kphi=1, azimuthal_flag=0, invariant_radius_flag=0)
    nb = 5 * 21 ** 3
    rng = np.random.default_rng(seed)
    for ev in range(n_events):
        res = os.path.join(work, "UrQMDev_%d" % ev, "UrQMD_results")
        os.makedirs(res)
        arr = [rng.integers(0, 60, nb).astype(float)] + [rng.normal(0, 1, nb) for _ in range(4)] + \
              [rng.integers(0, 90, nb).astype(float)] + [np.zeros(5 * 21) for _ in range(4)]
        ctr = [np.full(5, 1000, np.uint64), np.full(5, 1100, np.uint64), np.zeros(5, np.uint64),
               np.zeros(5, np.uint64)]
        L.hbt_host_write(ctypes.byref(hp), res.encode(), 0, *[a.ctypes.data_as(_PD) for a in arr],
                         *[c.ctypes.data_as(_PU) for c in ctr])
    text_mb = sum(os.path.getsize(os.path.join(r, f)) for r, _, fs in os.walk(work)
                  for f in fs) / 1e6
    t0 = time.perf_counter()
    n = L.hbt_host_average_events(work.encode(), os.path.join(d, "ours").encode(), 0)
    t_ours = time.perf_counter() - t0
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import average_events
    t0 = time.perf_counter()
    average_events.average_events(work, os.path.join(d, "port"))
    t_port = time.perf_counter() - t0
    same = all(open(os.path.join(d, "ours", f), "rb").read() ==
               open(os.path.join(d, "port", f), "rb").read()
               for f in os.listdir(os.path.join(d, "port")))
    shutil.rmtree(d, ignore_errors=True)
    return {"folders": n_events, "files": n, "text_MB": text_mb, "seconds": t_ours,
            "MB_per_s": text_mb / t_ours, "cpu_port_seconds": t_port,
            "cpu_port": "numpy loadtxt/savetxt restatement of the reference script, 1 thread",
            "speedup": t_port / t_ours, "outputs_identical": same,
            "host_threads": os.cpu_count()}


def bf_leg(n_events: int = 200, seed: int = 21) -> dict:
    """Balance function (pi+ / pi-): 200 events with Poisson(700) pi+ and
    pi-, Poisson(120) K+ and K-; Bnpts = 41 on |Delta y| <= 2, pT in
    [0.2, 2] GeV; every event against itself (4 same-event histograms) and
    against a drawn partner event with a random rotation (4 mixed-event
    histograms): all 8 x 200 event pairs in one hbt_bf_bin call, against
    the CPU oracle's restatement of the reference loop on a sample."""
    import ctypes
    from hadronic_afterburner_toolkit_gb300 import bf, synth
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    rng = np.random.default_rng(seed)
    kinds = [(211, synth.PION_MASS, 0.25, 700.0), (-211, synth.PION_MASS, 0.25, 700.0),
             (321, synth.KAON_MASS, 0.30, 120.0), (-321, synth.KAON_MASS, 0.30, 120.0)]
    gens = [synth.generate(n_events, mu, seed=seed + k, mass=m, monval=mon, T=T, y_max=2.0)
            for k, (mon, m, T, mu) in enumerate(kinds)]
    # species lists a = pi+, abar = pi-, b = pi-, bbar = pi+ (alpha 211, beta -211)
    lists = []
    for g in (gens[0], gens[1], gens[1], gens[0]):
        kin = oracle_lib.bf_boost(g)
        keep = ~((kin["pT"] < 0.2) | (kin["pT"] > 2.0))
        evid = np.repeat(np.arange(g.n_events), g.multiplicities())
        off = np.zeros(g.n_events + 1, np.int64)
        np.cumsum(np.bincount(evid[keep], minlength=g.n_events), out=off[1:])
        lists.append((off, kin["phi"][keep], kin["y"][keep]))
    lists = lists + lists  # the mixed-event pool is the buffer itself
    pairs_of = [(0, 2), (1, 3), (0, 3), (1, 2)]
    jobs = []
    for h, (la, lb) in enumerate(pairs_of):
        for e in range(n_events):
            jobs.append((h, la, e, lb, e, 0, 0.0))
            jobs.append((4 + h, la, e, 4 + lb, int(rng.integers(n_events)), 1,
                         float(rng.uniform(0, 2 * np.pi))))
    n_pairs = sum(int((lists[la][0][ea + 1] - lists[la][0][ea]) *
                      (lists[lb][0][eb + 1] - lists[lb][0][eb]))
                  for (h, la, ea, lb, eb, mx, rot) in jobs)
    eng = bf.BfEngine(41, 2.0)
    jarr = bf.job_array(jobs)
    eng.bin(lists, jarr)  # warm-up
    eng.reset()
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        eng.bin(lists, jarr)
        times.append(time.perf_counter() - t0)
    t_gpu = min(times)
    st = eng.stats()
    # CPU: the oracle's pair loop on the first jobs, ~5 s
    orc = oracle_lib.BfOracle(particle_alpha=211, particle_beta=-211, BpT_min=0.2, BpT_max=2.0,
                              Bnpts=41, Brap_max=2.0, rap_type=1, seed=1)
    L = oracle_lib._bf_lib()
    done, t0 = 0, time.perf_counter()
    for (h, la, ea, lb, eb, mx, rot) in jobs:
        A, B = lists[la], lists[lb]
        a0, a1, b0, b1 = A[0][ea], A[0][ea + 1], B[0][eb], B[0][eb + 1]
        cols = [np.ascontiguousarray(x) for x in (np.ones(a1 - a0), A[1][a0:a1], A[2][a0:a1],
                                                   np.ones(b1 - b0), B[1][b0:b1], B[2][b0:b1])]
        L.orc_bf_bin(orc._h, h, a1 - a0, *[oracle_lib._pd(c) for c in cols[:3]], b1 - b0,
                     *[oracle_lib._pd(c) for c in cols[3:]], mx, rot)
        done += int((a1 - a0) * (b1 - b0))
        if time.perf_counter() - t0 > 5.0:
            break
    t_cpu = time.perf_counter() - t0
    return {"events": n_events, "event_pairs": len(jobs), "pairs": n_pairs,
            "seconds": t_gpu, "pairs_per_s": n_pairs / t_gpu,
            "timing": "host clock around hbt_bf_bin (list upload, kernel, sync)",
            "kernel_ms": st["kernel_ms"], "upload_ms": st["upload_ms"],
            "kernel_pairs_per_s": n_pairs / (st["kernel_ms"] * 1e-3),
            "bytes_uploaded": st["bytes_uploaded"],
            "fp64_fallback_fraction": st["fp64_pairs"] / max(n_pairs, 1),
            "cpu_oracle_pairs_per_s": done / t_cpu, "cpu_cores": 1,
            "cpu_sample_pairs": done, "speedup_vs_cpu_core": (n_pairs / t_gpu) / (done / t_cpu)}


def fit_tables_synthetic(n_tables: int, seed: int = 31, nq: int = 41, q_max: float = 0.15):
    """Eight-column correlation tables of a 41^3 q grid on [-0.15, 0.15] GeV
    (the shape the HBT writer gives per K_T bin), pair-averaged q jitter,
    C from a Gaussian source with random radii plus noise."""
    rng = np.random.default_rng(seed)
    q = np.linspace(-q_max, q_max, nq)
    dq = q[1] - q[0]
    ql, qo, qs = [a.ravel() for a in np.meshgrid(q, q, q, indexing="ij")]
    out = []
    for _ in range(n_tables):
        lam, ro, rs, rl, ros, rol = (rng.uniform(0.3, 0.9), rng.uniform(3, 8), rng.uniform(3, 7),
                                     rng.uniform(3, 9), rng.uniform(0.6, 2.0), rng.uniform(0.5, 1.6))
        t = np.empty((qo.size, 8))
        t[:, 0] = qo + 0.1 * dq * rng.uniform(-1, 1, qo.size)
        t[:, 1] = qs + 0.1 * dq * rng.uniform(-1, 1, qo.size)
        t[:, 2] = ql + 0.1 * dq * rng.uniform(-1, 1, qo.size)
        a = np.array([ro, rs, rl, ros, rol]) / 0.19733
        c0 = lam * np.exp(-((a[0] * t[:, 0]) ** 2 + (a[1] * t[:, 1]) ** 2 + (a[2] * t[:, 2]) ** 2
                            + 2 * t[:, 0] * t[:, 1] * a[3] ** 2 + 2 * t[:, 0] * t[:, 2] * a[4] ** 2))
        err = 0.004 + 0.03 * c0
        t[:, 3] = 1000.0
        t[:, 5] = 1000.0
        t[:, 6] = c0 + err * rng.standard_normal(qo.size)
        t[:, 4] = 1000.0 * t[:, 6]
        t[:, 7] = err
        out.append(t)
    return out


def fit_leg(n_tables: int = 256, cpu_seconds: float = 8.0) -> dict:
    """Radii fits: 256 correlation tables (64 events x 4 K_T bins) of 41^3
    rows, five q cuts each (1280 fits) in one hbt_fit_radii call, against
    the oracle's scipy curve_fit loop (the reference script's) on one host
    core for a bounded sample of tables."""
    from hadronic_afterburner_toolkit_gb300 import radii
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    tabs = fit_tables_synthetic(n_tables)
    f = radii.Fitter()
    f.fit(tabs[:8])  # warm-up
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        rows = f.fit(tabs)
        times.append(time.perf_counter() - t0)
    st = f.stats()
    n_fits = n_tables * len(radii.Q_CUT_MAX_LIST)
    res = {"tables": n_tables, "rows_per_table": int(tabs[0].shape[0]), "fits": n_fits,
           "seconds": min(times), "fits_per_s": n_fits / min(times),
           "timing": "host clock around hbt_fit_radii (packing, upload, fits, results)",
           "kernel_ms": st["kernel_ms"], "upload_ms": st["upload_ms"],
           "points": st["points"], "passes": st["passes"],
           "converged": int((f.last["status"] == 0).sum())}
    try:
        import fit_radii
    except ImportError as exc:  # scipy missing
        res["cpu_oracle"] = "unavailable: %s" % exc
        return res
    done, t0 = 0, time.perf_counter()
    worst = 0.0
    for k, t in enumerate(tabs):
        o = fit_radii.fit_table(t)
        done += o.shape[0]
        worst = max(worst, float(np.max(np.abs(o[:, 1::2] - rows[k, :, 1::2]) / o[:, 2::2])))
        if time.perf_counter() - t0 > cpu_seconds:
            break
    t_cpu = time.perf_counter() - t0
    res.update({"cpu_oracle_fits_per_s": done / t_cpu, "cpu_cores": 1, "cpu_sample_fits": done,
                "speedup_vs_cpu_core": (n_fits / min(times)) / (done / t_cpu),
                "max_param_diff_in_errors_vs_oracle": worst})
    return res


def precision_leg(E, groups, p, local, n_kaon_groups: int = 3) -> dict:
    """The precision configuration against the FP64 oracle: one central pi+
    group and the first K+ groups (1000 K+ events, Poisson(250), T = 0.30
    GeV, oversample 100, 10 partners), same grid and bins, each binned by
    the FP64, FP32-weight and double-float forms on the GPU and by the
    oracle's pair loops on every host core.  Per form: counts and
    denominators identical or not; numerator (sum of cos(q.dx)) error per
    bin as |dnum| / count (over every bin with a pair), as |dnum| / sum of
    |cos| and as |dnum| / |num| (both over the bins with at least 2 pairs,
    the ones the writer prints); the mean-q sums' error per pair."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import oracle_lib
    L = oracle_lib.lib()
    import ctypes
    L.orc_get_abs_num.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    nthreads = os.cpu_count() or 1

    def run(groups_, prec):
        eng = E.Engine(device=local, precision=prec, **p)
        for cols, mixed in groups_:
            eng.bin_batch([("same", cols)] + [("mixed", l1, l2) for l1, l2 in mixed])
        h = eng.hist()
        eng.close()
        return h

    def oracle(groups_):
        orc = oracle_lib.Oracle(**p)
        t0 = time.perf_counter()
        for cols, mixed in groups_:
            orc.bin_same(cols, nthreads=nthreads)
            for l1, l2 in mixed:
                orc.bin_mixed(l1, l2, nthreads=nthreads)
        h = orc.hist()
        dt = time.perf_counter() - t0
        h["abs_num"] = np.zeros_like(h["num"])
        L.orc_get_abs_num(orc._h, h["abs_num"].ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return h, dt

    def errors(ho, hg):
        cnt = ho["count"]
        m, sel = cnt > 0, cnt >= 2
        dn = np.abs(hg["num"] - ho["num"])
        out = {"counts_identical": bool(np.array_equal(ho["count"], hg["count"])),
               "den_identical": bool(np.array_equal(ho["den"], hg["den"])),
               "counters_identical": bool(np.array_equal(ho["ctr_num"], hg["ctr_num"]) and
                                          np.array_equal(ho["ctr_den"], hg["ctr_den"])),
               "num_max_err_per_pair": float((dn[m] / cnt[m]).max()),
               "num_max_err_per_abs_cos": float((dn[sel] / np.maximum(ho["abs_num"][sel],
                                                                     1e-300)).max()),
               "num_max_rel_err": float((dn[sel] / np.maximum(np.abs(ho["num"][sel]),
                                                             1e-300)).max())}
        for k in ("q_out", "q_side", "q_long"):
            out[k + "_max_err_per_pair_gev"] = float(
                (np.abs(hg[k] - ho[k])[m] / cnt[m]).max())
        return out

    res = {"bin_selection": "per pair: bins with >= 1 pair; per |cos| sum and relative: bins "
                            "with >= 2 pairs (the ones the reference's writer prints)",
           "oracle": "oracle pair loops on %d host threads" % nthreads}
    for name, gs in (("pi+", groups[:1]),
                     ("K+", make_workload("kaons", max_groups=n_kaon_groups))):
        ho, dt = oracle(gs)
        r = {"groups": len(gs), "particles_per_group": int(np.mean([g[0][0].size for g in gs])),
             "bins_with_pairs": int((ho["count"] > 0).sum()), "oracle_s": dt}
        for label, prec in (("fp64", E.PRECISION_FP64), ("fp32w", E.PRECISION_FP32W),
                            ("df64", E.PRECISION_DF64)):
            r[label] = errors(ho, run(gs, prec))
        res[name] = r
    return res


def make_requests(n_jobs: int, seed: int = 5):
    """Requests of the serving workload: 10-500 events each, multiplicity
    Poisson(mu) with mu uniform in [50, 2000], pi+ or K+, qnpts in
    {21, 41, 61} on [-q_max, q_max] with q_max uniform in [0.1, 0.3] GeV,
    2-8 K_T bins on [0, 1] GeV."""
    from hadronic_afterburner_toolkit_gb300 import synth
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(n_jobs):
        nev = int(rng.integers(10, 501))
        mu = float(rng.uniform(50, 2000))
        kaon = bool(rng.random() < 0.5)
        qnpts = int(rng.choice([21, 41, 61]))
        qmax = float(rng.uniform(0.1, 0.3))
        nkt = int(rng.integers(2, 9)) + 1
        kw = dict(mass=synth.KAON_MASS, monval=321, T=0.30) if kaon else {}
        ev = synth.generate(nev, mu, seed=seed * 100_000 + k, sigma_xy=5.0, tau_mean=10.0, **kw)
        cols = [np.ascontiguousarray(getattr(ev, f)) for f in
                ("px", "py", "pz", "E", "x", "y", "z", "t")]
        prm = dict(qnpts=qnpts, q_min=-qmax, q_max=qmax, n_KT=nkt, KT_min=0.0, KT_max=1.0,
                   n_Kphi=8, azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
                   needed_number_of_pairs=1e18)
        reqs.append((cols, np.ascontiguousarray(ev.offsets, dtype=np.int64), prm, k + 1))
    return reqs


def serving_stream(E, local, reqs, rate, n, precision, seed):
    """n requests at Poisson arrivals of `rate` jobs/s through the serving
    loop.  Each request takes one event set of the pool `reqs` (in turn)
    with its own draw of the configuration's analysis parameters (qnpts in
    {21, 41, 61}, q_max in [0.1, 0.3] GeV, 2-8 K_T bins).  A second thread
    waits for the requests in order, records their latency (submit to
    results in host memory) and releases them.  Latency percentiles are
    taken over the steady-state window: requests that arrived between 10 %
    and 90 % of the arrival span."""
    import threading
    from hadronic_afterburner_toolkit_gb300 import server
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
    prms = []
    for k in range(n):
        qmax = float(rng.uniform(0.1, 0.3))
        prms.append(dict(reqs[k % len(reqs)][2], qnpts=int(rng.choice([21, 41, 61])),
                         q_min=-qmax, q_max=qmax, n_KT=int(rng.integers(2, 9)) + 1,
                         precision=precision, kernel=E.KERNEL_SCREENED))
    ids = [None] * n
    lat = np.zeros(n)
    pairs = [0]
    submitted = threading.Event()
    with server.Server(device=local) as srv:
        def waiter():
            for k in range(n):
                while ids[k] is None:
                    time.sleep(1e-4)
                srv.wait(ids[k])
                inf = srv.info(ids[k])
                lat[k] = inf["latency_ms"]
                pairs[0] += inf["pairs_same"] + inf["pairs_mixed"]
                srv.release(ids[k])
        th = threading.Thread(target=waiter)
        th.start()
        t0 = time.perf_counter()
        late = 0.0
        for k in range(n):
            now = time.perf_counter() - t0
            if arrivals[k] > now:
                time.sleep(arrivals[k] - now)
            else:
                late = max(late, now - arrivals[k])
            cols, off, _, sd = reqs[k % len(reqs)]
            ids[k] = srv.submit(cols, off, prms[k], oversample=1, mixed_partners=1, seed=sd + k)
        submitted.set()
        th.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
    span = float(arrivals[-1])
    win = (arrivals >= 0.1 * span) & (arrivals <= 0.9 * span)
    return {"requests": n, "rate_jobs_per_s": rate, "arrival_span_s": span, "wall_s": wall,
            "pairs_per_s": pairs[0] / wall,
            "offered_pairs_per_s": pairs[0] / span,
            "p50_ms": float(np.percentile(lat[win], 50)),
            "p99_ms": float(np.percentile(lat[win], 99)),
            "max_ms": float(lat[win].max()), "window_requests": int(win.sum()),
            "all_p99_ms": float(np.percentile(lat, 99)),
            "submit_lag_max_s": late, "rounds": st["rounds"], "peak_active": st["peak_active"],
            "peak_device_bytes": st["peak_bytes"], "gpu_busy_ms": st["gpu_busy_ms"]}


def steady_serving_leg(E, local, n=1000, seed=7) -> dict:
    """Serving at steady state and overloaded, each over n >= 1000
    requests: first config 5's 200 jobs/s, which is above what the GPU
    sustains for these requests (its throughput over the run is the
    measured capacity), then 60 % of that capacity in jobs/s, for the FP64
    and FP32-weight forms."""
    reqs = make_requests(48, seed)
    out = {"job_semantics": "each event of a request is its own same-event list (oversample "
                            "1) with one rotated partner event; config 5's one-buffer jobs "
                            "with nev/2+1 partners would offer ~1e12 pairs/s at 200 jobs/s, "
                            "tens of times this GPU's capacity",
           "event_sets": len(reqs)}
    over = serving_stream(E, local, reqs, 200.0, n, E.PRECISION_FP64, seed)
    out["overloaded-fp64"] = over
    mean_pairs = over["pairs_per_s"] * over["wall_s"] / n
    capacity = over["pairs_per_s"] / mean_pairs  # jobs/s the GPU sustained
    out["capacity_jobs_per_s_fp64"] = capacity
    out["mean_pairs_per_request"] = mean_pairs
    rate = 0.6 * capacity
    out["steady-fp64"] = serving_stream(E, local, reqs, rate, n, E.PRECISION_FP64, seed + 1)
    out["steady-fp32w"] = serving_stream(E, local, reqs, rate, n, E.PRECISION_FP32W, seed + 1)
    return out


def serving_leg(E, local, n_jobs=48, rate=200.0, seed=5) -> dict:
    """A Poisson request stream at `rate` jobs/s through the serving loop:
    continuous batching (FP64 and FP32 weights) against the plain per-job
    path (reference-chain kernel, one request at a time, list by list);
    the double-float form beside them."""
    from hadronic_afterburner_toolkit_gb300 import server
    reqs = make_requests(n_jobs, seed)
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n_jobs))

    def stream_run(precision, kernel):
        with server.Server(device=local) as srv:
            ids = []
            t0 = time.perf_counter()
            for (cols, off, prm, sd), t in zip(reqs, arrivals):
                now = time.perf_counter() - t0
                if t > now:
                    time.sleep(t - now)
                ids.append(srv.submit(cols, off, dict(prm, precision=precision, kernel=kernel),
                                      oversample=1, mixed_partners=1, seed=sd))
            for j in ids:
                srv.wait(j)
            wall = time.perf_counter() - t0
            st = srv.stats()
            infos = [srv.info(j) for j in ids]
        pairs = sum(i["pairs_same"] + i["pairs_mixed"] for i in infos)
        return {"pairs_per_s": pairs / wall, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                "mean_ms": st["mean_ms"], "max_ms": st["max_ms"], "wall_s": wall,
                "rounds": st["rounds"], "peak_active": st["peak_active"],
                "peak_device_bytes": st["peak_bytes"], "gpu_busy_ms": st["gpu_busy_ms"],
                "pairs": pairs}

    out = {"jobs": n_jobs, "rate_jobs_per_s": rate, "oversample": 1, "mixed_partners": 1,
           "arrival_span_s": float(arrivals[-1])}
    out["batched-fp64"] = stream_run(E.PRECISION_FP64, E.KERNEL_SCREENED)
    out["batched-fp32w"] = stream_run(E.PRECISION_FP32W, E.KERNEL_SCREENED)
    out["batched-df64"] = stream_run(E.PRECISION_DF64, E.KERNEL_SCREENED)
    out["plain-per-job-fp64"] = stream_run(E.PRECISION_FP64, E.KERNEL_REFERENCE_CHAIN)
    out["offered_pairs_per_s"] = out["batched-fp64"]["pairs"] / float(arrivals[-1])
    for k in ("batched-fp64", "batched-fp32w", "batched-df64"):
        out[k]["speedup_vs_plain"] = (out[k]["pairs_per_s"] /
                                      out["plain-per-job-fp64"]["pairs_per_s"])
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="central", choices=["central", "medium", "small"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32w", "df64"])
    ap.add_argument("--kernel", default="screened", choices=["screened", "reference-chain"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the one-step measurement of the plain reference-chain kernel")
    ap.add_argument("--no-uneven", action="store_true",
                    help="skip the uneven-multiplicity workload (one batched launch)")
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the Poisson request stream through the serving loop")
    ap.add_argument("--serving-jobs", type=int, default=48)
    ap.add_argument("--no-bf", action="store_true",
                    help="skip the balance-function leg")
    ap.add_argument("--no-fit", action="store_true",
                    help="skip the radii-fit leg")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the FP32-weight against FP64 error report")
    ap.add_argument("--order-items", type=int, default=1, choices=[0, 1],
                    help="hbt_tuning.order_items of the timed engine: same-event tile pairs "
                         "in momentum-region order")
    ap.add_argument("--no-capped", action="store_true",
                    help="skip the central workload at the default pair cap (3e7)")
    ap.add_argument("--no-ingest", action="store_true",
                    help="skip the reader timing (line-by-line against block reader)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    from hadronic_afterburner_toolkit_gb300 import engine as E

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    p = workload_params(args.workload)
    prec = {"fp64": E.PRECISION_FP64, "fp32w": E.PRECISION_FP32W,
            "df64": E.PRECISION_DF64}[args.precision]
    n_groups = args.warmup + args.steps
    groups = make_workload(args.workload, seed=1 + rank, max_groups=n_groups)
    dev = torch.device("cuda", local)

    # device-resident inputs
    dgroups = []
    for cols, mixed in groups:
        dc = [torch.from_numpy(c).to(dev) for c in cols]
        dm = [([torch.from_numpy(x).to(dev) for x in l1], [torch.from_numpy(x).to(dev) for x in l2])
              for l1, l2 in mixed]
        dgroups.append((dc, dm))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    kern = E.KERNEL_SCREENED if args.kernel == "screened" else E.KERNEL_REFERENCE_CHAIN
    eng = E.Engine(device=local, precision=prec, kernel=kern, **p)
    eng.set_stream(stream.cuda_stream)
    batched = kern == E.KERNEL_SCREENED
    if batched:
        # CUDA events around the persistent kernels (the roofline's kernel time)
        eng.set_tuning(time_kernels=1, order_items=args.order_items)

    def run_group(engine, grp, batch, device=True):
        """One oversample group: its same-event pairs and every event's
        mixed pairs, as one batch (persistent launch) or call by call."""
        dc, dm = grp
        if batch:
            engine.bin_batch([("same", dc)] + [("mixed", l1, l2) for l1, l2 in dm],
                             device=device)
        else:
            engine.bin_same(dc, device=device)
            for l1, l2 in dm:
                engine.bin_mixed(l1, l2, device=device)

    for k in range(args.warmup):
        run_group(eng, dgroups[k % len(dgroups)], batched)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = eng.stats()["launches"]
    ctr0 = eng.counters()
    ms_steps, pairs, same_ms, mixed_ms = [], 0, [], []
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            g = args.warmup + k
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run_group(eng, dgroups[g % len(dgroups)], batched)
            e1.record(stream)
            e1.synchronize()
            ms_steps.append(e0.elapsed_time(e1))
            pairs += group_pairs(groups[g % len(groups)])
            if batched:
                kst = eng.stats()
                same_ms.append(kst["same_kernel_ms"])
                mixed_ms.append(kst["mixed_kernel_ms"])
    torch.cuda.synchronize()
    launches = eng.stats()["launches"] - launches0
    ctr1 = eng.counters()
    # binned pairs of the timed steps (the pair counters are exact)
    binned_same = int(ctr1["num"].sum()) - int(ctr0["num"].sum())
    binned_mixed = int(ctr1["den"].sum()) - int(ctr0["den"].sum())
    t_ms = sum(ms_steps)
    reduced_bins = None
    if world > 1:
        # replicas: one histogram sum at the end (outside the timed region)
        reduced_bins = int(allreduce_hist(eng.hist(), device=dev)["count"].sum())
        t = torch.tensor([t_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_ms = float(t.item())
        pt = torch.tensor([float(pairs)], device=dev)
        torch.distributed.all_reduce(pt)
        pairs_all = float(pt.item())
    else:
        pairs_all = float(pairs)
    value = pairs_all / (t_ms * 1e-3)

    def time_variant(kernel, precision, nsteps, label, batch, **over):
        """Same workload, another kernel family / precision (or parameters
        `over`), same GPU."""
        engv = E.Engine(device=local, precision=precision, kernel=kernel, **dict(p, **over))
        engv.set_stream(stream.cuda_stream)
        ms_tot, prs = 0.0, 0
        for k in range(nsteps + 1):  # the first step warms up
            g = (args.warmup + k) % len(dgroups)
            with torch.cuda.stream(stream):
                flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run_group(engv, dgroups[g], batch)
            e1.record(stream)
            e1.synchronize()
            if k > 0:
                ms_tot += e0.elapsed_time(e1)
                prs += group_pairs(groups[g])
        st = engv.stats()
        engv.close()
        out = {"kernel": label, "value": prs / (ms_tot * 1e-3),
               "ms_per_step": ms_tot / nsteps, "steps": nsteps}
        if batch and kernel == E.KERNEL_SCREENED:
            # tile pairs of the last launch the cull kept, of the candidates
            out["tiles_same_kept"] = [st["tiles_same_kept"], st["tiles_same"]]
        return out

    # the plain form (FP64 reference chain on every pair, one call per list)
    # and the other forms, on the same GPU
    plain = None
    variants = {}
    if not args.no_plain and kern == E.KERNEL_SCREENED:
        plain = time_variant(E.KERNEL_REFERENCE_CHAIN, E.PRECISION_FP64, 1,
                             "reference-chain (FP64 reference order on every pair)", False)
        labels = {E.PRECISION_FP64: ("batched-fp64", "FP64"),
                  E.PRECISION_FP32W: ("batched-fp32w", "FP32 weights"),
                  E.PRECISION_DF64: ("batched-df64", "double-float values")}
        for other in labels:
            if other != prec:
                variants[labels[other][0]] = time_variant(
                    E.KERNEL_SCREENED, other, 2, "batched persistent, " + labels[other][1], True)
        variants["grid-" + args.precision] = time_variant(
            E.KERNEL_SCREENED_GRID, prec, 1,
            "screened, one launch per list, no sorting or culling", False)
        # the same workload with the q_inv histograms too
        # (invariant_radius_flag = 1): 1-D q_inv numerator and denominator
        # beside the 3-D ones, tile pairs kept for either window
        variants["batched-" + args.precision + "-qinv"] = time_variant(
            E.KERNEL_SCREENED, prec, 2,
            "batched persistent, with the q_inv histograms (invariant_radius_flag = 1)", True,
            invariant_radius_flag=1)

    # roofline of the dominant kernel, k_persistent_same: the FP64-pipe
    # instructions it executes (ncu count per binned pair, see
    # FP64_WARP_INST_PER_BINNED_PAIR) over its own time (CUDA events around
    # its launches), against the FP64 FMA instruction rate measured live on
    # this GPU (one FMA = one instruction on both sides)
    peaks = measure_fp64_peak()
    g0 = groups[args.warmup % len(groups)]
    fr = survival_fractions(g0, p)
    t_step = statistics.median(ms_steps) * 1e-3
    t_same_all = sum(same_ms) * 1e-3 if same_ms and min(same_ms) > 0 else t_ms * 1e-3
    t_same = t_same_all / max(1, len(same_ms) or args.steps)
    inst_peak = peaks["fp64_tflops"] * 1e12 / 2.0          # FP64 FMA instructions / s
    per_binned = FP64_WARP_INST_PER_BINNED_PAIR if (
        batched and args.precision == "fp64") else None
    achieved = (per_binned * 32.0 * binned_same / t_same_all) if per_binned else None
    # the reference's chain at the measured rates of its operations
    # (the bound for an implementation that evaluates it on every pair)
    n = g0[0][0].size
    P_same = n * (n - 1) / 2
    P_mixed = sum(l1[0].size * l2[0].size for l1, l2 in g0[1])
    rates = (inst_peak, peaks["div_gops"] * 1e9, peaks["sqrt_gops"] * 1e9,
             peaks["cos_gops"] * 1e9, peaks["atomic_gops_l2"] * 1e9)

    def chain_seconds(counts, P):
        return sum(P * f * sum(c / r for c, r in zip(stage, rates))
                   for stage, f in zip(counts, fr))
    chain_s = chain_seconds(STAGE_COUNTS_SAME, P_same) + chain_seconds(STAGE_COUNTS_MIXED, P_mixed)
    # DRAM bytes per launch of k_persistent_same on this workload (ncu,
    # profiles/k_persistent_same_fp64_central.md; not measured in this run)
    traffic = CENTRAL_SAME_DRAM_BYTES if (args.workload == "central" and
                                          args.precision == "fp64" and batched) else None
    try:
        hbm_peak = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, ValueError, KeyError):
        hbm_peak = 6800.0
    roofline = {"bound": "fp64", "achieved": achieved, "peak": inst_peak,
                "unit": "FP64 inst/s (warp instructions x 32)",
                "frac": achieved / inst_peak if achieved else None, "traffic": traffic,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                  "k_persistent_same, one central launch "
                                  "(profiles/k_persistent_same_fp64_central.md)" if traffic else None,
                "kernel": "k_persistent_same (same-event pairs; CUDA events around its "
                          "launch)" if batched and same_ms else "pair-binning kernels",
                "kernel_ms": t_same * 1e3,
                "mixed_kernel_ms": statistics.median(mixed_ms) if mixed_ms else None,
                "algorithmic_work": "FP64-pipe instructions per binned same-event pair "
                                    "(ncu, one central launch) x binned pairs of the timed "
                                    "launches; peak = live FP64 FMA probe / 2 (instructions)",
                "fp64_warp_inst_per_binned_pair": per_binned,
                "binned_same_pairs_per_launch": binned_same / max(1, args.steps),
                "hbm": {"achieved_gbs": traffic / t_same / 1e9 if traffic else None,
                        "peak_gbs": hbm_peak, "peak_source": "MEASURED_PEAKS.json",
                        "frac": (traffic / t_same / 1e9 / hbm_peak) if traffic else None},
                "peak_source": "measured live: FP64 FMA probe (lib/libhbt_probe.so)",
                "probes": {k: peaks[k] for k in ("fp64_tflops", "fp32_tflops", "div_gops",
                                                 "sqrt_gops", "cos_gops", "atomic_gops_l2",
                                                 "atomic_gops_256mb")},
                # the reference's per-pair chain on every pair at these rates
                # (operation counts per stage of the chain x the measured
                # fraction of pairs reaching that stage): the time an
                # implementation of the plain chain cannot beat
                "reference_chain": {
                    "stage_counts_same": STAGE_COUNTS_SAME,
                    "stage_counts_mixed": STAGE_COUNTS_MIXED,
                    "survival": [round(x, 4) for x in fr],
                    "bound_ms_per_step": chain_s * 1e3,
                    "step_ms": t_step * 1e3,
                    "step_vs_bound": chain_s / t_step},
                # histogram updates of the same-event kernel: per binned pair
                # four FP64 sums (one 32-byte bin) and one u64 count, against
                # scattered FP64 atomic adds measured live on L2-resident data
                # (the atomic units) and on 256 MB (beyond L2)
                "l2_atomics": {
                    "achieved_gops": 5 * binned_same / t_same_all / 1e9,
                    "peak_gops": peaks["atomic_gops_l2"],
                    "frac": 5 * binned_same / t_same_all / 1e9 / peaks["atomic_gops_l2"],
                    "scattered_256mb_gops": peaks["atomic_gops_256mb"],
                    "peak_source": "measured live: scattered FP64 atomicAdd probe over 32 MB "
                                   "and 256 MB (lib/libhbt_probe.so)"}}

    # end to end through the host-buffer C ABI (pinned host arrays)
    e2e = None
    if not args.no_e2e:
        eng2 = E.Engine(device=local, precision=prec, kernel=kern, **p)
        eng2.set_tuning(order_items=args.order_items)
        # each group's columns packed in one pinned host array in the order
        # the batch stages them, every column a multiple of 32 doubles (the
        # layout the drop-in's HBT_correlation builds), so a step's inputs
        # cross in one copy
        pin = []
        for cols, mixed in groups:
            seq = list(cols) + [x for l1, l2 in mixed for x in list(l1) + list(l2)]
            sizes = [(x.size + 31) // 32 * 32 for x in seq]
            buf = torch.empty(sum(sizes), dtype=torch.float64).pin_memory().numpy()
            views, at = [], 0
            for x, sz in zip(seq, sizes):
                buf[at:at + x.size] = x
                views.append(buf[at:at + x.size])
                at += sz
            pc, k = views[:8], 8
            pm = []
            for l1, l2 in mixed:
                pm.append((views[k:k + 4], views[k + 4:k + 8]))
                k += 8
            pin.append((pc, pm))
        nb = eng2.L.hbt_n_bins(eng2.handle)
        # two pinned result sets: the histograms of step k copy to the host
        # (hbt_read_hist_async) while step k + 1 bins
        out = [[torch.empty(nb, dtype=torch.float64).pin_memory().numpy() for _ in range(6)]
               for _ in range(2)]

        def step_host(k):
            run_group(eng2, pin[k % len(pin)], batched, device=False)
            eng2._check(eng2.L.hbt_read_hist_async(
                eng2.handle, *[o.ctypes.data_as(E._PD) for o in out[k % 2]]))

        for k in range(args.warmup):
            step_host(k)
        eng2._check(eng2.L.hbt_read_hist_wait(eng2.handle))
        h2d = d2h = 0
        t0 = time.perf_counter()
        e2e_pairs = 0
        for k in range(args.steps):
            g = args.warmup + k
            step_host(g)
            pc, pm = pin[g % len(pin)]
            h2d += sum(c.nbytes for c in pc) + sum(x.nbytes for l1, l2 in pm for x in l1 + l2)
            d2h += 6 * nb * 8
            e2e_pairs += group_pairs(groups[g % len(groups)])
        eng2._check(eng2.L.hbt_read_hist_wait(eng2.handle))  # the last step's results
        t_e2e = time.perf_counter() - t0
        e2e = {"value": e2e_pairs / t_e2e, "unit": "pairs/s",
               "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps,
               "readback": "hbt_read_hist_async every step into pinned arrays (copies overlap "
                           "the next step), the last one waited for inside the timed region"}
        eng2.close()

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        cpu = cpu_baseline(groups[0], p)

    uneven = serving = ingest = average = None
    balance = fits = precision = None
    dropin = None
    if not args.no_ingest and rank == 0:
        ingest = ingest_leg()
        average = average_leg()
        dropin = dropin_leg()
    if not args.no_bf and rank == 0:
        balance = bf_leg()
    if not args.no_fit and rank == 0:
        fits = fit_leg()
    if not args.no_precision and rank == 0 and args.workload == "central":
        precision = precision_leg(E, groups, p, local)
    small = None
    if not args.no_uneven and rank == 0 and args.workload == "central":
        small = small_leg(E, torch, dev, stream, flush, local)
    capped = None
    if not args.no_capped and rank == 0 and args.workload == "central" and batched:
        capped = capped_leg(E, torch, dev, dgroups, groups, p, local, t_ms / args.steps)
    if not args.no_uneven:
        uneven = uneven_leg(E, torch, dev, stream, flush, local)
    if not args.no_serving:
        serving = serving_leg(E, local, n_jobs=args.serving_jobs)
        serving["steady_state"] = steady_serving_leg(E, local)

    if rank == 0:
        st = eng.stats()
        line = {"metric": "candidate pairs binned per second (same + mixed event)",
                "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": {"fp64": "f64", "fp32w": "f64 bins / f32 weights",
                          "df64": "f64 bins / double-float (2 x f32) values"}[args.precision],
                "data": "synthetic",
                "config": {"workload": args.workload,
                           "events": {"central": 1000, "medium": 300}.get(args.workload, 100),
                           "oversample": {"central": 100, "medium": 30}.get(args.workload, 10),
                           "particles_per_group": int(np.mean([g[0][0].size for g in groups])),
                           "mixed_partners": 5 if args.workload == "small" else 10,
                           "qnpts": p["qnpts"], "n_KT_bins": p["n_KT"] - 1,
                           "n_Kphi": p["n_Kphi"] if p["azimuthal_flag"] else 1,
                           "precision": args.precision, "kernel": args.kernel,
                           "order_items": args.order_items,
                           "l2": "flushed (256 MB write) between steps",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "pairs_per_step": pairs_all / args.steps / max(world, 1),
                "binned_same_fraction": round(fr[4], 4),
                "gpu_launches": launches,
                "replica_reduction_binned_pairs": reduced_bins,
                "clocks": clk.summary(),
                "roofline": roofline,
                "plain_kernel": dict(plain, frac_of_reference_chain_bound=(
                    roofline["reference_chain"]["bound_ms_per_step"] / plain["ms_per_step"]))
                if plain else None,
                "speedup_vs_plain": (value / plain["value"]) if plain else None,
                # each form against the plain kernel and against the best
                # batched FP64 form (the headline) on the same GPU
                "variants": {k: dict(v, speedup_vs_plain=(v["value"] / plain["value"])
                                     if plain else None,
                                     speedup_vs_batched_fp64=v["value"] / value)
                             for k, v in variants.items()},
                "e2e": e2e,
                "cpu_baseline": cpu,
                "small_config": small,
                "capped": capped,
                "dropin": dropin,
                "uneven": uneven,
                "serving": serving,
                "ingest": ingest,
                "average": average,
                "balance_function": balance,
                "radii_fit": fits,
                "precision_vs_oracle": precision,
                "stats": st}
        print(json.dumps(line))
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
