"""Deterministic synthetic correlation tables in the eight-column layout the
reference's radii fit reads (ebe_scripts/fit_HBT_radii.py:60-67: columns
0-2 the pair-averaged q_out, q_side, q_long, column 6 the correlation C - 1,
column 7 its error; columns 3-5 are pair counts and sums the fit ignores).

The noise comes from a splitmix64 stream through Box-Muller in plain Python
floats, so a table is the same on every machine and numpy version up to the
last bits of libm's log and cos, which the fit tolerances absorb.
"""
from __future__ import annotations

import math

import numpy as np

HBARC = 0.19733
KT_CUTS = ["0_0.2", "0.2_0.4", "0.4_0.6", "0.6_0.8"]
M64 = (1 << 64) - 1


def _splitmix(state):
    state = (state + 0x9E3779B97F4A7C15) & M64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return state, z ^ (z >> 31)


def normals(seed: int, n: int) -> np.ndarray:
    out = np.empty(n)
    s = seed & M64
    for i in range(0, n, 2):
        s, a = _splitmix(s)
        s, b = _splitmix(s)
        u1 = ((a >> 11) + 1) * 2.0 ** -53
        u2 = (b >> 11) * 2.0 ** -53
        r = math.sqrt(-2.0 * math.log(u1))
        out[i] = r * math.cos(2.0 * math.pi * u2)
        if i + 1 < n:
            out[i + 1] = r * math.sin(2.0 * math.pi * u2)
    return out


def model(qo, qs, ql, p):
    """lambda exp(-(R_out q_out)^2 - ... - 2 q_out q_long R_ol^2), radii in fm."""
    lam, ro, rs, rl, ros, rol = [float(x) for x in p]
    ao, as_, al, aos, aol = (ro / HBARC, rs / HBARC, rl / HBARC, ros / HBARC, rol / HBARC)
    return lam * np.exp(-((ao * qo) ** 2 + (as_ * qs) ** 2 + (al * ql) ** 2
                          + 2.0 * qo * qs * aos ** 2 + 2.0 * qo * ql * aol ** 2))


def make_table(seed: int, params, nq: int = 21, q_max: float = 0.15, noise: float = 0.03,
               floor: float = 0.004, blank_every: int = 0,
               blank_beyond: float = 0.16) -> np.ndarray:
    """An (nq^3, 8) table: grid q in [-q_max, q_max] (q_long outer, q_out,
    q_side inner, the writer's order), each q shifted by up to a tenth of a
    bin as a pair average would be; C from the model plus Gaussian noise of
    floor + noise * C; with `blank_every`, every such row beyond
    |q| = `blank_beyond` has C and its error NaN (an empty bin), which the
    script's nan_to_num turns into zeros."""
    q = np.linspace(-q_max, q_max, nq)
    dq = q[1] - q[0]
    ql, qo, qs = [a.ravel() for a in np.meshgrid(q, q, q, indexing="ij")]
    n = ql.size
    z = normals(seed, 4 * n)
    qo = qo + 0.1 * dq * np.tanh(z[:n])
    qs = qs + 0.1 * dq * np.tanh(z[n:2 * n])
    ql = ql + 0.1 * dq * np.tanh(z[2 * n:3 * n])
    c0 = model(qo, qs, ql, params)
    err = floor + noise * c0
    c = c0 + err * z[3 * n:]
    t = np.zeros((n, 8))
    t[:, 0], t[:, 1], t[:, 2] = qo, qs, ql
    t[:, 3] = 1000.0
    t[:, 4] = c * 1000.0
    t[:, 5] = 1000.0
    t[:, 6], t[:, 7] = c, err
    if blank_every:
        far = np.sqrt(qo ** 2 + qs ** 2 + ql ** 2) > blank_beyond
        rows = np.flatnonzero(far)[::blank_every]
        t[rows, 6:] = np.nan
    return t


# Events of the fixture database: seed, source parameters per K_T bin.
EVENTS = {
    "event_1": (11, [(0.55, 6.0, 5.2, 6.5, 1.5, 1.1), (0.6, 5.2, 4.8, 5.0, 1.2, 0.9),
                     (0.62, 4.6, 4.3, 4.0, 1.0, 0.7), (0.65, 4.1, 3.9, 3.3, 0.9, 0.6)]),
    "event_2": (23, [(0.4, 7.5, 6.0, 8.0, 2.0, 1.5), (0.45, 6.5, 5.5, 6.5, 1.6, 1.3),
                     (0.5, 5.5, 5.0, 5.5, 1.3, 1.1), (0.5, 4.8, 4.6, 4.6, 1.1, 0.9)]),
}


def database():
    """{event: {file name: table}} of the fixture."""
    out = {}
    for ev, (seed, plist) in EVENTS.items():
        out[ev] = {}
        for k, (cut, p) in enumerate(zip(KT_CUTS, plist)):
            out[ev]["HBT_correlation_function_KT_%s.dat" % cut] = make_table(
                seed * 10 + k, p, blank_every=7 if k == 3 else 0)
    return out


def random_database(seed: int, n_events: int = 2) -> dict:
    """A database in the fixture's layout with source parameters, noise,
    grid size and empty bins drawn from a seeded generator (the live
    comparison with the reference script uses it)."""
    rng = np.random.default_rng(seed)
    out = {}
    for e in range(n_events):
        ev = "event_%d" % (e + 1)
        out[ev] = {}
        nq = int(rng.choice([15, 21, 25]))
        for k, cut in enumerate(KT_CUTS):
            p = (float(rng.uniform(0.3, 0.8)), float(rng.uniform(2.5, 8.5)),
                 float(rng.uniform(2.5, 8.0)), float(rng.uniform(2.0, 9.0)),
                 float(rng.uniform(0.0, 2.0)), float(rng.uniform(0.0, 1.6)))
            out[ev]["HBT_correlation_function_KT_%s.dat" % cut] = make_table(
                int(rng.integers(1, 1 << 30)), p, nq=nq,
                noise=float(rng.uniform(0.01, 0.06)),
                blank_every=int(rng.choice([0, 0, 5, 9])))
    return out
