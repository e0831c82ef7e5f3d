"""Serving loop (include/hbt_server.h): requests of different analyses
(q grids, K_T / K_phi bins, boost, precision) batched into shared persistent
launches must give, for every request, the result it gets alone, and that
result must equal the oracle's run of the reference's buffer loop
(orc_process_buffer: event-plane angle, oversampled same-event pairs,
seeded partner draws and rotations, mixed pairs).

Tolerances: counts, denominators and pair counters identical; FP64 sums
within tests/parity.py's RTOL (1e-12 per count); FP32-weight sums within
RTOL32 = 1e-5 per count against the FP64 oracle and between runs;
double-float sums within RTOL_DF = 1e-11 per count.
"""
import numpy as np
import pytest

import oracle_lib
import parity

pytestmark = pytest.mark.gpu

RTOL32 = 1e-5
RTOL_DF = 1e-11  # the double-float form's stated bound (test_precision_gpu.py)
FP32W = 1
DF64 = 2

# name -> request: analysis parameters and the buffer's shape
REQUESTS = {
    "fp64_boost": dict(params=dict(qnpts=13, n_KT=4), n_events=6, mu=80.0, partners=3, seed=11),
    "fp64_noboost_wide": dict(params=dict(qnpts=11, q_min=-0.2, q_max=0.2, n_KT=3,
                                          long_comoving_boost=0),
                              n_events=5, mu=120.0, partners=2, seed=12),
    "kphi": dict(params=dict(qnpts=9, n_KT=3, azimuthal_flag=1, n_Kphi=4), n_events=4,
                 mu=150.0, partners=2, seed=13),
    "fp32w": dict(params=dict(qnpts=13, n_KT=4, precision=FP32W), n_events=6, mu=100.0,
                  partners=2, seed=14),
    "df64": dict(params=dict(qnpts=13, n_KT=4, precision=DF64), n_events=6, mu=100.0,
                 partners=2, seed=20),
    "cap_solo": dict(params=dict(qnpts=11, n_KT=3, needed_number_of_pairs=1500), n_events=4,
                     mu=60.0, partners=2, seed=15),
    "qinv_solo": dict(params=dict(qnpts=11, n_KT=3, invariant_radius_flag=1), n_events=3,
                      mu=60.0, partners=2, seed=16),
    "one_event": dict(params=dict(qnpts=11, n_KT=3), n_events=1, mu=50.0, partners=1, seed=17),
    "tiny_events": dict(params=dict(qnpts=11, n_KT=3), n_events=4, mu=[0, 1, 2, 40],
                        partners=2, seed=18),
    "kaon_default_partners": dict(params=dict(qnpts=9, n_KT=2, KT_min=0.1, KT_max=0.9),
                                  n_events=5, mu=70.0, partners=0, seed=19, kaon=True),
}


def _buffer(req):
    from hadronic_afterburner_toolkit_gb300 import synth
    kw = dict(seed=1000 + req["seed"], sigma_xy=2.0, tau_mean=3.0)
    if req.get("kaon"):
        kw.update(mass=synth.KAON_MASS, T=0.30)
    return synth.generate(req["n_events"], req["mu"], **kw)


def _full_params(req):
    from hadronic_afterburner_toolkit_gb300 import server
    return server.default_params(**req["params"])


def _qscale(p):
    return max(abs(p["q_min"]), abs(p["q_max"])) + (p["q_max"] - p["q_min"]) / (p["qnpts"] - 1)


def _submit(srv, req, ev, **kw):
    return srv.submit(parity.cols8(ev), ev.offsets, req["params"],
                      mixed_partners=req["partners"], seed=req["seed"], **kw)


def _oracle_buffer(req, ev):
    """The reference's buffer loop on the CPU: the mixed pool is the buffer."""
    p = _full_params(req)
    keep = ("qnpts", "q_min", "q_max", "n_KT", "KT_min", "KT_max", "n_Kphi", "azimuthal_flag",
            "invariant_radius_flag", "long_comoving_boost", "needed_number_of_pairs")
    orc = oracle_lib.Oracle(**{k: p[k] for k in keep}, HBTrap_min=-1.0, HBTrap_max=1.0,
                            number_of_mixed_events=req["partners"], seed=req["seed"])
    orc.process_buffer(ev)
    return orc.hist()


def _check(res, ref, p, what):
    rtol = {FP32W: RTOL32, DF64: RTOL_DF}.get(p["precision"], parity.RTOL)
    try:
        return parity.compare(res, ref, _qscale(p), rtol=rtol)
    except AssertionError as e:
        raise AssertionError("%s: %s" % (what, e))


@pytest.fixture(scope="module")
def buffers():
    return {name: _buffer(req) for name, req in REQUESTS.items()}


@pytest.fixture(scope="module")
def alone(buffers):
    """Each request run with nothing else on the server."""
    from hadronic_afterburner_toolkit_gb300 import server
    out = {}
    with server.Server() as srv:
        for name, req in REQUESTS.items():
            j = _submit(srv, req, buffers[name])
            srv.wait(j)
            out[name] = (srv.result(j), srv.info(j))
    return out


@pytest.mark.parametrize("name", list(REQUESTS))
def test_request_matches_oracle_buffer_loop(name, buffers, alone):
    req = REQUESTS[name]
    res, info = alone[name]
    assert info["solo"] == (1 if name.endswith("solo") else 0)
    ref = _oracle_buffer(req, buffers[name])
    _check(res, ref, _full_params(req), name)


def test_results_same_alone_and_in_the_mix(buffers, alone):
    from hadronic_afterburner_toolkit_gb300 import server
    # a small round budget splits each request over several rounds and puts
    # the work of several requests into each round
    with server.Server(round_tile_pairs=12, max_in_flight=3) as srv:
        jobs = {name: _submit(srv, req, buffers[name]) for name, req in REQUESTS.items()}
        for j in jobs.values():
            srv.wait(j)
        infos = {name: srv.info(j) for name, j in jobs.items()}
        st = srv.stats()
        for name, j in jobs.items():
            _check(srv.result(j), alone[name][0], _full_params(REQUESTS[name]),
                   name + " mixed vs alone")
    batched = [i for i in infos.values() if not i["solo"]]
    assert all(i["state"] == server.JOB_DONE for i in infos.values())
    assert max(i["rounds"] for i in batched) > 1          # requests split over rounds
    assert sum(i["rounds"] for i in batched) > st["rounds"]  # rounds shared by requests
    assert st["completed"] == len(REQUESTS) and st["failed"] == 0
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert st["bytes_in_use"] == 0 and st["active"] == 0


def test_oversample_groups_match_oracle(buffers):
    """Same-event lists of `oversample` consecutive events; partners and
    rotations as the server drew them."""
    from hadronic_afterburner_toolkit_gb300 import server
    req = dict(params=dict(qnpts=13, n_KT=4, azimuthal_flag=1, n_Kphi=3), n_events=7,
               mu=90.0, partners=2, seed=21)
    ev = _buffer(req)
    with server.Server(round_tile_pairs=8) as srv:
        j = _submit(srv, req, ev, oversample=3)
        srv.wait(j)
        res, info = srv.result(j), srv.info(j)
        P, partners, cphi, sphi = srv.mixing(j, ev.n_events)
    p = _full_params(req)
    keep = ("qnpts", "q_min", "q_max", "n_KT", "KT_min", "KT_max", "n_Kphi", "azimuthal_flag",
            "invariant_radius_flag", "long_comoving_boost", "needed_number_of_pairs")
    orc = oracle_lib.Oracle(**{k: p[k] for k in keep})
    psi = oracle_lib.event_plane_angle(ev.px, ev.py, 2)
    assert info["psi_ref"] == psi
    orc.set_psi_ref(psi)
    o = ev.offsets
    cols = parity.cols8(ev)
    ratio = ev.pz / ev.E
    cut = (ratio > np.tanh(-1.0)) & (ratio < np.tanh(1.0))
    for g0 in range(0, ev.n_events, 3):
        g1 = min(g0 + 3, ev.n_events)
        sel = np.zeros(ev.px.size, bool)
        sel[o[g0]:o[g1]] = True
        sel &= cut
        orc.bin_same([c[sel] for c in cols])
    for e in range(ev.n_events):
        s1 = np.zeros(ev.px.size, bool)
        s1[o[e]:o[e + 1]] = True
        s1 &= cut
        l2 = [[], [], [], []]
        for k in range(P):
            m = partners[e, k]
            s2 = np.zeros(ev.px.size, bool)
            s2[o[m]:o[m + 1]] = True
            s2 &= cut
            px, py = ev.px[s2], ev.py[s2]
            l2[0].append(px * cphi[e, k] - py * sphi[e, k])
            l2[1].append(px * sphi[e, k] + py * cphi[e, k])
            l2[2].append(ev.pz[s2])
            l2[3].append(ev.E[s2])
        orc.bin_mixed([c[s1] for c in cols[:4]], [np.concatenate(c) for c in l2])
    _check(res, orc.hist(), p, "oversample=3")


def test_memory_admission_holds_one_request_at_a_time(buffers):
    from hadronic_afterburner_toolkit_gb300 import server
    names = ["fp64_boost", "fp64_noboost_wide", "fp32w", "one_event"]
    with server.Server() as probe:
        sizes = {}
        for n in names:
            j = _submit(probe, REQUESTS[n], buffers[n])
            sizes[n] = probe.info(j)["device_bytes"]
            probe.wait(j)
    budget = max(sizes.values())  # no two requests fit together
    with server.Server(memory_budget=budget) as srv:
        jobs = [_submit(srv, REQUESTS[n], buffers[n]) for n in names]
        for j in jobs:
            srv.wait(j)
        st = srv.stats()
        infos = [srv.info(j) for j in jobs]
    assert st["peak_active"] == 1
    assert st["peak_bytes"] <= budget
    assert st["completed"] == len(names)
    # each later request was admitted only after the one before it finished
    for a, b in zip(infos, infos[1:]):
        assert b["queue_ms"] >= 0.0 and a["state"] == b["state"] == server.JOB_DONE


def test_rejections(buffers):
    from hadronic_afterburner_toolkit_gb300 import engine, server
    ev = buffers["fp64_boost"]
    req = REQUESTS["fp64_boost"]
    with server.Server(memory_budget=1 << 20) as srv:
        with pytest.raises(engine.HbtError, match="HBT_ERR_NOMEM"):
            _submit(srv, req, ev)
    with server.Server() as srv:
        with pytest.raises(engine.HbtError, match="HBT_ERR_INVALID"):
            srv.submit(parity.cols8(ev), ev.offsets, dict(qnpts=1))
        bad = np.array(ev.offsets)
        bad[2] = bad[1] - 1
        with pytest.raises(engine.HbtError, match="HBT_ERR_INVALID"):
            srv.submit(parity.cols8(ev), bad, req["params"])
        with pytest.raises(engine.HbtError, match="HBT_ERR_INVALID"):
            srv.submit(parity.cols8(ev), ev.offsets, req["params"], seed=-1)
        # reading a request that is not done, releasing, then reading again
        j = _submit(srv, req, ev)
        srv.wait(j)
        srv.release(j)
        with pytest.raises(engine.HbtError):
            srv.info(j)
