"""Balance-function pair binning on the GPU (include/hbt_bf.h) against the
oracle's restatement of the reference's loops, histogram by histogram:
counts must be identical (an FP32 screen with rigorous bounds decides most
pairs; the rest are binned in FP64 in the reference's operation order).  Inputs: the golden balance-function cases with their
species lists, and hand-made lists whose differences sit on bin edges."""
import math

import numpy as np
import pytest

import oracle_lib

pytestmark = pytest.mark.gpu


def _lists_of(buf, kin, prm, ptmin, ptmax):
    """Species lists a, abar, b, bbar of a buffer with the pT cut applied:
    (offsets, phi, y) each, plus the raw per-event arrays for the oracle."""
    a, b = int(prm["particle_alpha"]), int(prm["particle_beta"])
    yv = kin["eta"] if int(prm["rap_type"]) == 0 else kin["y"]
    out = []
    for mon in (a, -a, b, -b):
        keep = (buf.monval == mon) & ~((kin["pT"] < ptmin) | (kin["pT"] > ptmax))
        evid = np.repeat(np.arange(buf.n_events), buf.multiplicities())
        mult = np.bincount(evid[keep], minlength=buf.n_events)
        off = np.zeros(buf.n_events + 1, np.int64)
        np.cumsum(mult, out=off[1:])
        out.append((off, kin["phi"][keep], yv[keep], kin["pT"][keep]))
    return out


@pytest.mark.parametrize("name", ["pions", "kaon_pion_eta", "oscar_real_mixed"])
def test_bf_histograms_match_oracle(name):
    from hadronic_afterburner_toolkit_gb300 import bf, synth
    prm, ev, mixed = oracle_lib.bf_golden_case(name)
    p = oracle_lib.bf_params_from(prm)
    shift = prm.get("rapidity_shift", 0.0)
    eng = bf.BfEngine(p["Bnpts"], p["Brap_max"])
    orc = oracle_lib.BfOracle(**p)
    L = oracle_lib._bf_lib()
    rng = np.random.default_rng(7)
    size = int(prm["event_buffer_size"])
    rs = oracle_lib.buffer_ranges(ev.multiplicities(), size)
    rm = oracle_lib.buffer_ranges(mixed.multiplicities(), size) if mixed is not None else None
    pairs = {0: (0, 2), 1: (1, 3), 2: (0, 3), 3: (1, 2)}
    for k, (s, e) in enumerate(rs):
        buf = synth.subset(ev, s, e)
        same = _lists_of(buf, oracle_lib.bf_boost(buf, shift), prm, p["BpT_min"], p["BpT_max"])
        if mixed is not None:
            mbuf = synth.subset(mixed, *rm[k])
            pool = _lists_of(mbuf, oracle_lib.bf_boost(mbuf, shift), prm, p["BpT_min"],
                             p["BpT_max"])
        else:
            pool = same
        lists = [x[:3] for x in same] + [x[:3] for x in pool]
        jobs = []
        for h, (la, lb) in pairs.items():
            for ev_i in range(buf.n_events):
                jobs.append((h, la, ev_i, lb, ev_i, 0, 0.0))
                partner = int(rng.integers(len(pool[0][0]) - 1))
                rot = float(rng.uniform(0, 2 * math.pi))
                jobs.append((4 + h, la, ev_i, 4 + lb, partner, 1, rot))
        eng.bin(lists, jobs)
        for (h, la, ea, lb, eb, mx, rot) in jobs:
            A = lists[la]
            Bl = lists[lb]
            a0, a1 = A[0][ea], A[0][ea + 1]
            b0, b1 = Bl[0][eb], Bl[0][eb + 1]
            pa = np.ascontiguousarray(same[la][3][a0:a1] if la < 4 else pool[la - 4][3][a0:a1])
            pb = np.ascontiguousarray((same + pool)[lb][3][b0:b1])
            cols = [np.ascontiguousarray(x) for x in
                    (pa, A[1][a0:a1], A[2][a0:a1], pb, Bl[1][b0:b1], Bl[2][b0:b1])]
            L.orc_bf_bin(orc._h, h, a1 - a0, *[oracle_lib._pd(c) for c in cols[:3]],
                         b1 - b0, *[oracle_lib._pd(c) for c in cols[3:]], mx, rot)
    total = 0
    for h in range(8):
        g, o = eng.hist(h), orc.hist(h)
        assert np.array_equal(g, o), "histogram %d differs at %s" % (h, np.argwhere(g != o)[:5])
        total += o.sum()
    assert total > 1000


def test_bf_bin_edges_and_tiles():
    """Differences exactly on Delta y and Delta phi edges, |Delta y| below
    1e-10 (identical particles), rotations that wrap the azimuth, an event
    pair of more than one 128-particle tile, empty lists."""
    from hadronic_afterburner_toolkit_gb300 import bf
    Bnpts, Brap_max = 9, 1.0
    drap = 2.0 * Brap_max / (Bnpts - 1)
    ymin = -Brap_max - 0.5 * drap
    dphi = 2.0 * math.pi / 20
    rng = np.random.default_rng(3)
    edges_y = np.array([ymin + k * drap for k in range(Bnpts + 1)])
    edges_p = np.array([-math.pi / 2 + k * dphi for k in range(21)])
    # event 0: b at the origin, a on every edge combination (plus neighbours)
    ya = np.concatenate([edges_y, np.nextafter(edges_y, 5), np.nextafter(edges_y, -5),
                         rng.uniform(-2, 2, 40), [0.0, 1e-11, -5e-11]])
    pa = np.concatenate([np.resize(edges_p, ya.size - 3), [0.0, 0.0, 0.0]])
    yb = np.array([0.0, 1e-12, 0.3, -0.7])
    pb = np.array([0.0, 0.0, 1.1, -2.9])
    # event 1: 300 x 200 random particles (several tiles)
    ya1, pa1 = rng.uniform(-1.5, 1.5, 300), rng.uniform(-math.pi, math.pi, 300)
    yb1, pb1 = rng.uniform(-1.5, 1.5, 200), rng.uniform(-math.pi, math.pi, 200)
    A = (np.array([0, ya.size, ya.size + 300, ya.size + 300], np.int64),
         np.concatenate([pa, pa1]), np.concatenate([ya, ya1]))
    B = (np.array([0, 4, 204, 204], np.int64), np.concatenate([pb, pb1]),
         np.concatenate([yb, yb1]))
    jobs = []
    for ev_i in range(3):
        jobs.append((0, 0, ev_i, 1, ev_i, 0, 0.0))
        for r, rot in enumerate([0.0, 2 * math.pi - 1e-12, 5.5, -edges_p[3]]):
            jobs.append((4 + r, 0, ev_i, 1, ev_i, 1, rot))
    eng = bf.BfEngine(Bnpts, Brap_max)
    eng.bin([A, B], jobs)
    orc = oracle_lib.BfOracle(particle_alpha=1, particle_beta=2, BpT_min=-1.0, BpT_max=10.0,
                              Bnpts=Bnpts, Brap_max=Brap_max, rap_type=1, seed=1)
    L = oracle_lib._bf_lib()
    for (h, la, ea, lb, eb, mx, rot) in jobs:
        a0, a1 = A[0][ea], A[0][ea + 1]
        b0, b1 = B[0][eb], B[0][eb + 1]
        cols = [np.ascontiguousarray(x) for x in
                (np.ones(a1 - a0), A[1][a0:a1], A[2][a0:a1],
                 np.ones(b1 - b0), B[1][b0:b1], B[2][b0:b1])]
        L.orc_bf_bin(orc._h, h, a1 - a0, *[oracle_lib._pd(c) for c in cols[:3]], b1 - b0,
                     *[oracle_lib._pd(c) for c in cols[3:]], mx, rot)
    for h in range(5):
        assert np.array_equal(eng.hist(h), orc.hist(h)), h
    assert eng.hist(0).sum() > 30000  # most of the 300 x 200 tile pairs fall in the Delta y window


def test_bf_rejects_bad_jobs():
    from hadronic_afterburner_toolkit_gb300 import bf, engine
    eng = bf.BfEngine(5, 1.0)
    A = (np.array([0, 2], np.int64), np.zeros(2), np.zeros(2))
    with pytest.raises(engine.HbtError, match="HBT_ERR_INVALID"):
        eng.bin([A], [(0, 0, 1, 0, 0, 0, 0.0)])
    with pytest.raises(engine.HbtError, match="HBT_ERR_INVALID"):
        eng.bin([A], [(8, 0, 0, 0, 0, 0, 0.0)])


@pytest.mark.parametrize("name", ["pions", "kaon_pion_eta", "oscar_real_mixed"])
def test_bf_dropin_matches_reference_files(name, tmp_path):
    """The drop-in executable on a golden balance-function case writes the
    reference's three files (same partner and rotation draws, same bins)."""
    import os
    import shutil
    import subprocess
    import tarfile
    import parity
    src = os.path.join(oracle_lib.GOLDEN_BF, name)
    res = tmp_path / "results"
    res.mkdir()
    for fn in os.listdir(src):
        if fn == "parameters.dat":
            shutil.copy(os.path.join(src, fn), tmp_path)
        elif (fn.endswith(".gz") and fn != "outputs.tar.gz") or fn.endswith(".DAT"):
            shutil.copy(os.path.join(src, fn), res)
    exe = os.path.join(oracle_lib.REPO, "hadronic_afterburner_toolkit_gb300", "lib",
                       "hbt_afterburner.e")
    proc = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-2000:]
    with tarfile.open(os.path.join(src, "outputs.tar.gz")) as tar:
        want = {m.name: tar.extractfile(m).read() for m in tar.getmembers()}
    for f in want:
        parity.same_output_file(open(res / f, "rb").read(), want[f], f)


def test_bf_fp32_screen_near_edges():
    """Differences a few FP32 ulps either side of every Delta y and Delta
    phi edge and of the Delta y cuts, at rapidities and angles of several
    magnitudes: the FP32 screen must hand every pair it cannot decide to
    the FP64 expressions, so the counts stay the oracle's."""
    from hadronic_afterburner_toolkit_gb300 import bf
    Bnpts, Brap_max = 41, 2.0
    drap = 2.0 * Brap_max / (Bnpts - 1)
    ymin = -Brap_max - 0.5 * drap
    dphi = 2.0 * math.pi / 20
    rng = np.random.default_rng(11)
    edges_y = np.array([ymin + k * drap for k in range(Bnpts + 1)])
    edges_p = np.array([-math.pi / 2 + k * dphi for k in range(41)])
    offs = np.concatenate([[0.0], np.outer([1, -1], [1e-9, 3e-8, 1e-7, 4e-7, 2e-6]).ravel()])
    yb = np.array([0.0, 0.75, -3.2, 1e-11])
    pb = np.array([0.0, 1.3, -2.9, 3.1])
    ya, pa = [], []
    for y0, p0 in zip(yb, pb):
        for o in offs:
            ya.append(edges_y + y0 + o * (1.0 + abs(y0)))
            pa.append(np.resize(edges_p, edges_y.size) + p0 + o * (1.0 + abs(p0)))
    ya = np.concatenate(ya + [yb, yb + 1e-10, yb - 2e-10])
    pa = np.concatenate(pa + [pb, pb + 1e-7, pb - dphi])
    A = (np.array([0, ya.size], np.int64), pa, ya)
    B = (np.array([0, yb.size], np.int64), pb, yb)
    jobs = [(0, 0, 0, 1, 0, 0, 0.0)]
    for r, rot in enumerate([dphi, 2 * math.pi - dphi, 0.5 + 1e-8, 4 * dphi - 1e-9,
                             rng.uniform(0, 2 * math.pi), 1e-300, 6.0]):
        jobs.append((1 + r, 0, 0, 1, 0, 1, rot))
    eng = bf.BfEngine(Bnpts, Brap_max)
    eng.bin([A, B], bf.job_array(jobs))
    orc = oracle_lib.BfOracle(particle_alpha=1, particle_beta=2, BpT_min=-1.0, BpT_max=10.0,
                              Bnpts=Bnpts, Brap_max=Brap_max, rap_type=1, seed=1)
    L = oracle_lib._bf_lib()
    for (h, la, ea, lb, eb, mx, rot) in jobs:
        cols = [np.ascontiguousarray(x) for x in (np.ones(ya.size), pa, ya,
                                                   np.ones(yb.size), pb, yb)]
        L.orc_bf_bin(orc._h, h, ya.size, *[oracle_lib._pd(c) for c in cols[:3]], yb.size,
                     *[oracle_lib._pd(c) for c in cols[3:]], mx, rot)
    for h in range(len(jobs)):
        g, o = eng.hist(h), orc.hist(h)
        assert np.array_equal(g, o), "histogram %d differs at %s" % (h, np.argwhere(g != o)[:5])
    assert eng.hist(0).sum() > 1000
    st = eng.stats()
    assert st["pairs"] == len(jobs) * ya.size * yb.size
    assert 0 < st["fp64_pairs"] < st["pairs"]  # the edges reach the FP64 path
    assert st["kernel_ms"] > 0
    # a list passed twice with the same arrays is uploaded once
    eng.bin([A, B, A, B], [(0, 2, 0, 3, 0, 0, 0.0)])
    n_items = -(-ya.size // 128)
    assert eng.stats()["bytes_uploaded"] == 48 + 8 * n_items + 16 * (ya.size + yb.size)


def test_bf_many_rapidity_bins():
    """Bnpts = 600: the shared histogram (600 x 40 counts, 96 KB) needs the
    opt-in shared-memory size; random lists against the oracle."""
    from hadronic_afterburner_toolkit_gb300 import bf
    Bnpts, Brap_max = 600, 3.0
    rng = np.random.default_rng(19)
    na, nb = 700, 500
    A = (np.array([0, na], np.int64), rng.uniform(-np.pi, np.pi, na), rng.uniform(-2, 2, na))
    B = (np.array([0, nb], np.int64), rng.uniform(-np.pi, np.pi, nb), rng.uniform(-2, 2, nb))
    jobs = [(0, 0, 0, 1, 0, 0, 0.0), (5, 0, 0, 1, 0, 1, 2.1)]
    eng = bf.BfEngine(Bnpts, Brap_max)
    eng.bin([A, B], jobs)
    orc = oracle_lib.BfOracle(particle_alpha=1, particle_beta=2, BpT_min=-1.0, BpT_max=10.0,
                              Bnpts=Bnpts, Brap_max=Brap_max, rap_type=1, seed=1)
    L = oracle_lib._bf_lib()
    for (h, la, ea, lb, eb, mx, rot) in jobs:
        cols = [np.ascontiguousarray(x) for x in (np.ones(na), A[1], A[2], np.ones(nb), B[1], B[2])]
        L.orc_bf_bin(orc._h, h, na, *[oracle_lib._pd(c) for c in cols[:3]], nb,
                     *[oracle_lib._pd(c) for c in cols[3:]], mx, rot)
    for h in (0, 5):
        assert np.array_equal(eng.hist(h), orc.hist(h)), h
    assert eng.hist(0).sum() > 100000
