"""GPU parity of the C-ABI engine against the CPU oracle (FP64 form).

Counts, denominators and pair counters must be identical to the oracle's;
the FP64 sums agree to the tolerance stated in tests/parity.py.
"""
import numpy as np
import pytest

import oracle_lib
import parity

pytestmark = pytest.mark.gpu

BASIC = dict(qnpts=9, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=4,
             azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
             needed_number_of_pairs=1e18)
FULL = dict(BASIC, invariant_radius_flag=1, azimuthal_flag=1, n_Kphi=4, q_min=0.0, q_max=0.2,
            qnpts=11)
CUTS = dict(BASIC, KT_min=0.15, KT_max=0.55, long_comoving_boost=0, q_min=-0.1, q_max=0.2,
            qnpts=7, n_KT=4)
PARAMS = {"basic": BASIC, "full": FULL, "cuts": CUTS}


def _engine(**kw):
    from hadronic_afterburner_toolkit_gb300 import engine
    return engine.Engine(**kw)


def _oracle(**kw):
    kw = dict(kw)
    kw.pop("kphi_defer_tol", None)
    return oracle_lib.Oracle(**kw)


def _qscale(p):
    return max(abs(p["q_min"]), abs(p["q_max"])) + (p["q_max"] - p["q_min"]) / (p["qnpts"] - 1)


@pytest.mark.parametrize("name", sorted(PARAMS))
def test_same_event_matches_oracle(name):
    p = PARAMS[name]
    ev = parity.lists(seed=101)
    eng, orc = _engine(**p), _oracle(**p)
    eng.set_psi_ref(0.37)
    orc.set_psi_ref(0.37)
    c = parity.cols8(ev)
    eng.bin_same(c)
    orc.bin_same(c)
    h = orc.hist()
    assert h["count"].sum() > 100
    parity.compare(eng.hist(), h, _qscale(p))


@pytest.mark.parametrize("name", sorted(PARAMS))
def test_mixed_event_matches_oracle(name):
    p = PARAMS[name]
    ev = parity.lists(seed=202)
    eng, orc = _engine(**p), _oracle(**p)
    eng.set_psi_ref(-1.1)
    orc.set_psi_ref(-1.1)
    m = ev.multiplicities()
    o = ev.offsets
    for e in range(3):
        l1 = parity.rotated4(ev, 0.0, o[e], o[e + 1])
        l2 = [np.concatenate(x) for x in zip(*[parity.rotated4(ev, 0.3 + k, o[k], o[k + 1])
                                              for k in range(ev.n_events) if k != e])]
        eng.bin_mixed(l1, l2)
        orc.bin_mixed(l1, l2)
    h = orc.hist()
    assert h["den"].sum() > 100
    parity.compare(eng.hist(), h, _qscale(p))
    assert m.sum() > 0


def test_several_buffers_accumulate():
    p = dict(BASIC, invariant_radius_flag=1, q_min=0.0, q_max=0.2)
    eng, orc = _engine(**p), _oracle(**p)
    for seed in (1, 2, 3):
        ev = parity.lists(seed=seed, n_events=4)
        c = parity.cols8(ev)
        eng.bin_same(c)
        orc.bin_same(c)
        l1 = parity.rotated4(ev, 0.0, 0, ev.offsets[1])
        l2 = parity.rotated4(ev, 1.0, ev.offsets[1], None)
        eng.bin_mixed(l1, l2)
        orc.bin_mixed(l1, l2)
    parity.compare(eng.hist(), orc.hist(), _qscale(p))


@pytest.mark.parametrize("az", [0, 1])
def test_binding_caps_admit_pairs_in_reference_order(az):
    """needed_number_of_pairs binds inside launches: ordered admission."""
    p = dict(BASIC, invariant_radius_flag=1, azimuthal_flag=az, n_Kphi=3,
             needed_number_of_pairs=37)
    eng, orc = _engine(**p), _oracle(**p)
    eng.set_psi_ref(0.2)
    orc.set_psi_ref(0.2)
    for seed in (11, 12):
        ev = parity.lists(seed=seed, n_events=5)
        c = parity.cols8(ev)
        eng.bin_same(c)
        orc.bin_same(c)
        o = ev.offsets
        for e in range(ev.n_events):
            l1 = parity.rotated4(ev, 0.0, o[e], o[e + 1])
            l2 = parity.rotated4(ev, 0.7 * e, o[(e + 1) % ev.n_events],
                                 o[(e + 1) % ev.n_events + 1])
            eng.bin_mixed(l1, l2)
            orc.bin_mixed(l1, l2)
    h = orc.hist()
    assert (h["ctr_num"] == 38).any() and (h["ctr_den"] == 38).any()
    parity.compare(eng.hist(), h, _qscale(p))
    assert eng.stats()["ordered_passes"] > 0


@pytest.mark.parametrize("kernel", [0, 1])
def test_kphi_edge_pairs_decided_on_host(kernel):
    """A wide deferral zone sends many pairs through the host atan2 path
    (the screened kernels decide a K_phi bin in FP32 when its error bound
    allows and the pair lies outside the zone, and hand the rest to the
    reference chain, which defers the pairs inside the zone); bins must
    equal the oracle's exactly either way."""
    p = dict(FULL, kphi_defer_tol=0.05, kernel=kernel)
    eng, orc = _engine(**p), _oracle(**{k: v for k, v in p.items() if k != "kernel"})
    eng.set_psi_ref(0.11)
    orc.set_psi_ref(0.11)
    ev = parity.lists(seed=303)
    c = parity.cols8(ev)
    eng.bin_same(c)
    orc.bin_same(c)
    l1 = parity.rotated4(ev, 0.0, 0, ev.offsets[2])
    l2 = parity.rotated4(ev, 2.0, ev.offsets[2], None)
    eng.bin_mixed(l1, l2)
    orc.bin_mixed(l1, l2)
    h = eng.hist()
    assert eng.stats()["deferred_kphi"] > 100
    parity.compare(h, orc.hist(), _qscale(p))


def test_kphi_deferrals_with_binding_caps():
    p = dict(FULL, kphi_defer_tol=0.05, needed_number_of_pairs=15, n_Kphi=3)
    eng, orc = _engine(**p), _oracle(**p)
    eng.set_psi_ref(-0.4)
    orc.set_psi_ref(-0.4)
    ev = parity.lists(seed=404)
    c = parity.cols8(ev)
    eng.bin_same(c)
    orc.bin_same(c)
    l1 = parity.rotated4(ev, 0.0, 0, ev.offsets[2])
    l2 = parity.rotated4(ev, 2.0, ev.offsets[2], None)
    eng.bin_mixed(l1, l2)
    orc.bin_mixed(l1, l2)
    parity.compare(eng.hist(), orc.hist(), _qscale(p))


def _edge_pairs(p, seed=7, per_edge=25):
    """Pairs whose q_out / q_side / q_long sit within a few ulps of every bin
    edge and window bound (K along +x so q_out = q_x, q_side = q_y)."""
    rng = np.random.default_rng(seed)
    dq = (p["q_max"] - p["q_min"]) / (p["qnpts"] - 1)
    base = p["q_min"] - dq / 2.0
    edges = [base + k * dq for k in range(p["qnpts"] + 1)]
    edges += [p["q_min"] - dq / 2.0 + 1e-8, p["q_max"] + dq / 2.0 - 1e-8]
    rows = []
    for e in edges:
        for m in range(-per_edge, per_edge + 1):
            val = e + m * 2.0 ** -55
            px2 = rng.uniform(0.3, 0.6)
            py = 0.0  # K_y = 0 exactly, so cos(phi_K) = 1 and sin(phi_K) = 0
            pz2 = rng.uniform(-0.3, 0.3)
            which = m % 3
            qx = val if which == 0 else rng.uniform(-0.05, 0.05)
            qy = val if which == 1 else rng.uniform(-0.05, 0.05)
            qz = val if which == 2 else rng.uniform(-0.05, 0.05)
            p1 = (px2 + qx, py + qy / 2.0, pz2 + qz)
            p2 = (px2, py - qy / 2.0, pz2)
            for (x, y, z) in (p1, p2):
                E = np.sqrt(x * x + y * y + z * z + 0.13957 ** 2)
                rows.append((x, y, z, E))
    a = np.array(rows)
    n = a.shape[0]
    zeros = rng.normal(0, 1, size=(n, 4))
    return [a[:, 0].copy(), a[:, 1].copy(), a[:, 2].copy(), a[:, 3].copy(),
            zeros[:, 0].copy(), zeros[:, 1].copy(), zeros[:, 2].copy(), zeros[:, 3].copy()]


@pytest.mark.parametrize("boost", [0, 1])
def test_bin_edge_pairs_bit_exact(boost):
    p = dict(BASIC, long_comoving_boost=boost, KT_min=0.3, KT_max=0.6, qnpts=7)
    c = _edge_pairs(p)
    eng, orc = _engine(**p), _oracle(**p)
    eng.bin_same(c)
    orc.bin_same(c)
    eng.bin_mixed(c[:4], c[:4])
    orc.bin_mixed(c[:4], c[:4])
    h = orc.hist()
    assert h["count"].sum() > 1000
    parity.compare(eng.hist(), h, _qscale(p))


def test_empty_and_single_particle_lists():
    p = dict(BASIC, invariant_radius_flag=1)
    eng, orc = _engine(**p), _oracle(**p)
    ev = parity.lists(seed=5)
    for n in (0, 1):
        c = [x[:n] for x in parity.cols8(ev)]
        eng.bin_same(c)
        orc.bin_same(c)
        eng.bin_mixed(c[:4], parity.cols8(ev)[:4])
        orc.bin_mixed(c[:4], parity.cols8(ev)[:4])
    h = eng.hist()
    assert h["count"].sum() == 0
    parity.compare(h, orc.hist(), _qscale(p))
    assert h["pairs_mixed"] == 1 * ev.n_particles


def test_counts_repeatable_across_runs():
    ev = parity.lists(seed=9, n_events=8)
    c = parity.cols8(ev)
    hs = []
    for _ in range(3):
        eng = _engine(**BASIC)
        eng.bin_same(c)
        hs.append(eng.hist())
    for h in hs[1:]:
        assert np.array_equal(h["count"], hs[0]["count"])
        assert np.allclose(h["num"], hs[0]["num"], rtol=0, atol=1e-9)


def test_device_resident_entry_points():
    torch = pytest.importorskip("torch")
    ev = parity.lists(seed=77)
    c = parity.cols8(ev)
    eng_h, eng_d = _engine(**FULL), _engine(**FULL)
    for e in (eng_h, eng_d):
        e.set_psi_ref(0.5)
    eng_h.bin_same(c)
    dc = [torch.from_numpy(x).cuda() for x in c]
    eng_d.bin_same(dc, device=True)
    eng_h.bin_mixed(c[:4], c[:4])
    eng_d.bin_mixed(dc[:4], dc[:4], device=True)
    a, b = eng_h.hist(), eng_d.hist()
    for k in ("count", "den", "qinv_count", "qinv_den"):
        assert np.array_equal(a[k], b[k])


def test_sync_with_timeout_and_stats():
    eng = _engine(**BASIC)
    ev = parity.lists(seed=3)
    eng.bin_same(parity.cols8(ev))
    eng.sync(timeout_us=10_000_000)
    st = eng.stats()
    assert st["pairs_same"] == ev.n_particles * (ev.n_particles - 1) // 2
    assert st["launches"] >= 1


# ------------------------------------------------------------------ screen
# The default (screened) kernels decide most bins in FP32 with an error
# bound; these cases put many pairs where that bound matters.

def _hard_lists(seed, n=900):
    """Momenta up to several GeV (larger FP32 rounding) and a tight source."""
    from hadronic_afterburner_toolkit_gb300 import synth
    return synth.generate(3, n / 3.0, seed=seed, T=1.2, sigma_xy=1.0, tau_mean=1.0)


@pytest.mark.parametrize("az,boost", [(0, 1), (1, 1), (1, 0), (0, 0)])
def test_screened_and_reference_chain_kernels_agree(az, boost):
    p = dict(BASIC, azimuthal_flag=az, long_comoving_boost=boost, n_Kphi=8, qnpts=15,
             n_KT=9, KT_max=2.0)
    ev = _hard_lists(31 + az + 2 * boost)
    c = parity.cols8(ev)
    hs = []
    for kernel in (0, 1):
        eng = _engine(kernel=kernel, **p)
        eng.set_psi_ref(0.9)
        eng.bin_same(c)
        eng.bin_mixed(c[:4], [x[::-1].copy() for x in c[:4]])
        hs.append(eng.hist())
    orc = _oracle(**p)
    orc.set_psi_ref(0.9)
    orc.bin_same(c)
    orc.bin_mixed(c[:4], [x[::-1].copy() for x in c[:4]])
    h = orc.hist()
    assert h["count"].sum() > 500
    for eh in hs:
        parity.compare(eh, h, _qscale(p))


def test_screen_pairs_with_vanishing_pair_momentum():
    """p_T(2) ~ -p_T(1): K_perp near 0 makes the FP32 bounds unusable; such
    pairs must take the FP64 path (and K_perp == 0 exactly is an anomaly)."""
    rng = np.random.default_rng(5)
    n = 400
    px = rng.uniform(-0.3, 0.3, n)
    py = rng.uniform(-0.3, 0.3, n)
    eps = rng.choice([0.0, 1e-9, 1e-7, 1e-5, 1e-3], size=n)
    px2 = -px + eps
    py2 = -py - eps
    pz = rng.uniform(-0.2, 0.2, 2 * n)
    pxs = np.concatenate([px, px2])
    pys = np.concatenate([py, py2])
    E = np.sqrt(pxs ** 2 + pys ** 2 + pz ** 2 + 0.13957 ** 2)
    pos = rng.normal(0, 1, size=(4, 2 * n))
    c = [pxs, pys, pz, E, pos[0], pos[1], pos[2], pos[3]]
    p = dict(BASIC, q_min=-1.0, q_max=1.0, qnpts=11)
    eng, orc = _engine(**p), _oracle(**p)
    eng.bin_same(c)
    orc.bin_same(c)
    eng.bin_mixed(c[:4], [x[:n] for x in c[:4]])
    orc.bin_mixed(c[:4], [x[:n] for x in c[:4]])
    h = orc.hist()
    parity.compare(eng.hist(), h, 1.0)


def test_screen_kphi_edges():
    """K directions placed within float rounding of K_phi bin edges."""
    rng = np.random.default_rng(8)
    psi = 0.4
    n_kphi = 8
    rows = []
    for m in range(n_kphi):
        edge = psi + m * 2 * np.pi / n_kphi
        for k in range(-6, 7):
            ang = edge + k * 3e-8
            kt = rng.uniform(0.1, 0.6)
            q = rng.uniform(-0.05, 0.05, 3)
            K = np.array([kt * np.cos(ang), kt * np.sin(ang), rng.uniform(-0.2, 0.2)])
            for s in (+1, -1):
                v = K + s * q / 2
                rows.append((v[0], v[1], v[2], np.sqrt(v @ v + 0.13957 ** 2)))
    a = np.array(rows)
    pos = rng.normal(0, 1, size=(4, a.shape[0]))
    c = [a[:, 0].copy(), a[:, 1].copy(), a[:, 2].copy(), a[:, 3].copy()] + [x.copy() for x in pos]
    p = dict(BASIC, azimuthal_flag=1, n_Kphi=n_kphi, qnpts=11)
    eng, orc = _engine(**p), _oracle(**p)
    for x in (eng, orc):
        x.set_psi_ref(psi)
        x.bin_same(c)
        x.bin_mixed(c[:4], c[:4])
    h = orc.hist()
    assert h["count"].sum() > 50
    parity.compare(eng.hist(), h, _qscale(p))


def _qinv_edge_pairs(p, seed=13, per_edge=20):
    """Pairs whose q_inv, computed with the reference's FP64 expression
    sqrt(-(qE*qE - qx*qx - qy*qy - qz*qz)), lies within a few ulps of every
    q bin edge and window bound above 0: p1 = p2 + s v with s found by
    bisection, then s stepped by single ulps around it."""
    rng = np.random.default_rng(seed)
    m = 0.13957
    dq = (p["q_max"] - p["q_min"]) / (p["qnpts"] - 1)
    base = p["q_min"] - dq / 2.0
    edges = [base + k * dq for k in range(p["qnpts"] + 1)]
    edges += [p["q_min"] - dq / 2.0 + 1e-8, p["q_max"] + dq / 2.0 - 1e-8]
    edges = [e for e in edges if e > 1e-4]

    def qinv(p1, p2):
        e1 = np.sqrt(p1 @ p1 + m * m)
        e2 = np.sqrt(p2 @ p2 + m * m)
        qx, qy, qz, qE = p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2], e1 - e2
        return np.sqrt(-(qE * qE - qx * qx - qy * qy - qz * qz))

    rows = []
    for e in edges:
        p2 = np.array([rng.uniform(0.2, 0.5), rng.uniform(-0.2, 0.2), rng.uniform(-0.3, 0.3)])
        v = rng.normal(size=3)
        v /= np.sqrt(v @ v)
        lo, hi = 0.0, 1.0
        for _ in range(80):
            mid = 0.5 * (lo + hi)
            if qinv(p2 + mid * v, p2) < e:
                lo = mid
            else:
                hi = mid
        for k in range(-per_edge, per_edge + 1):
            s = np.nextafter(lo, np.inf if k > 0 else -np.inf) if k else lo
            for _ in range(abs(k) - 1):
                s = np.nextafter(s, np.inf if k > 0 else -np.inf)
            p1 = p2 + s * v
            for q in (p1, p2):
                rows.append((q[0], q[1], q[2], np.sqrt(q @ q + m * m)))
    a = np.array(rows)
    pos = rng.normal(0, 1, size=(a.shape[0], 4))
    return [np.ascontiguousarray(a[:, k]) for k in range(4)] + \
        [np.ascontiguousarray(pos[:, k]) for k in range(4)]


@pytest.mark.parametrize("kernel", [0, 1])
def test_qinv_edge_pairs_bit_exact(kernel):
    """q_inv histograms on pairs at every q_inv bin edge (same-event and
    mixed-event): the batched kernels' FP32 q_inv screen hands every pair it
    cannot decide to the reference chain, so counts equal the oracle's."""
    p = dict(BASIC, invariant_radius_flag=1, qnpts=11, q_min=0.0, q_max=0.2, KT_min=0.0)
    c = _qinv_edge_pairs(p)
    eng, orc = _engine(kernel=kernel, **p), _oracle(**p)
    eng.bin_same(c)
    orc.bin_same(c)
    eng.bin_mixed(c[:4], c[:4])
    orc.bin_mixed(c[:4], c[:4])
    h = orc.hist()
    assert h["qinv_count"].sum() > 1000 and h["qinv_den"].sum() > 1000
    parity.compare(eng.hist(), h, _qscale(p))


def test_async_readback_applies_host_decided_kphi_edges():
    """hbt_read_hist_async decides the deferred K_phi edges in the stream's
    order (a host function queued after the binning) without waiting for the
    binning: with a wide deferral zone on the reference chain, many pairs
    take that path, and the snapshot equals the oracle's binning."""
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(FULL, kphi_defer_tol=0.05, kernel=1)
    eng, orc = _engine(**p), _oracle(**{k: v for k, v in p.items() if k != "kernel"})
    for x in (eng, orc):
        x.set_psi_ref(-0.2)
    ev = parity.lists(seed=404)
    c = parity.cols8(ev)
    l1 = parity.rotated4(ev, 0.0, 0, ev.offsets[2])
    l2 = parity.rotated4(ev, 1.3, ev.offsets[2], None)
    for x in (eng, orc):
        x.bin_same(c)
        x.bin_mixed(l1, l2)
    n = int(eng.L.hbt_n_bins(eng.handle))
    snap = [np.full(n, -1.0) for _ in range(6)]
    eng._check(eng.L.hbt_read_hist_async(eng.handle, *[a.ctypes.data_as(E._PD) for a in snap]))
    eng._check(eng.L.hbt_read_hist_wait(eng.handle))
    assert eng.stats()["deferred_kphi"] > 100
    o = orc.hist()
    got = dict(zip(("count", "q_out", "q_side", "q_long", "num", "den"), snap))
    for k in ("count", "den"):
        assert np.array_equal(got[k], o[k]), k
    for k in ("q_out", "q_side", "q_long", "num"):
        bound = parity.RTOL * np.maximum(o["count"], 1.0) * (1.0 if k == "num" else _qscale(p))
        assert (np.abs(got[k] - o[k]) <= bound).all(), k
    # a second read (nothing new deferred) leaves the histograms as they are
    again = [np.zeros(n) for _ in range(6)]
    eng._check(eng.L.hbt_read_hist_async(eng.handle, *[a.ctypes.data_as(E._PD) for a in again]))
    eng._check(eng.L.hbt_read_hist_wait(eng.handle))
    for a, b in zip(again, snap):
        np.testing.assert_array_equal(a, b)
