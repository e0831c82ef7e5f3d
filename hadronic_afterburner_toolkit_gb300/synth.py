"""Seeded synthetic particle samples in the toolkit's input formats.

No public dataset exists for the HBT path; events are drawn from a simple
emission-source model with the shapes the benchmark configurations name:

* momentum: pT ~ Exp(slope T), azimuth ~ U[0, 2pi), rapidity y ~ U(-y_max, y_max),
  mT = sqrt(pT^2 + m^2), E = mT cosh y, pz = mT sinh y;
* position: x, y ~ N(0, sigma_xy), eta_s ~ U(-1, 1), tau ~ Exp(mean tau0),
  t = tau cosh eta_s, z = tau sinh eta_s.

Writers produce the two text formats the drop-in reads:

* ``read_in_mode = 10`` (iSS gzip): per event one line ``n``, then ``n`` lines
  ``monval mass t x y z E px py pz``
  (reference: src/particleSamples.cpp:1247-1286);
* ``read_in_mode = 0`` (OSCAR): three header lines, then per event
  ``event_id n 0 0`` and ``n`` lines ``idx monval px py pz E mass x y z t``
  (reference: src/particleSamples.cpp:680-714).

Doubles are printed with 17 significant digits, so the text round-trips to
the exact binary values.
"""
from __future__ import annotations

import dataclasses
import gzip
from typing import Optional, Sequence

import numpy as np

PION_MASS = 0.13957
KAON_MASS = 0.49368


@dataclasses.dataclass
class Events:
    """A flat particle table with per-event offsets (CSR layout)."""

    offsets: np.ndarray  # int64 [n_events + 1]
    monval: np.ndarray  # int32
    mass: np.ndarray
    t: np.ndarray
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    E: np.ndarray
    px: np.ndarray
    py: np.ndarray
    pz: np.ndarray

    @property
    def n_events(self) -> int:
        return int(self.offsets.size - 1)

    @property
    def n_particles(self) -> int:
        return int(self.offsets[-1])

    def multiplicities(self) -> np.ndarray:
        return np.diff(self.offsets)

    def event(self, i: int) -> dict:
        a, b = int(self.offsets[i]), int(self.offsets[i + 1])
        return {k: getattr(self, k)[a:b] for k in
                ("monval", "mass", "t", "x", "y", "z", "E", "px", "py", "pz")}

    @staticmethod
    def concat(parts: Sequence["Events"]) -> "Events":
        fields = ("monval", "mass", "t", "x", "y", "z", "E", "px", "py", "pz")
        mult = np.concatenate([p.multiplicities() for p in parts])
        offsets = np.zeros(mult.size + 1, dtype=np.int64)
        np.cumsum(mult, out=offsets[1:])
        return Events(offsets, *[np.concatenate([getattr(p, f) for p in parts])
                                 for f in fields])


def generate(n_events: int,
             multiplicity,
             *,
             seed: int,
             mass: float = PION_MASS,
             monval: int = 211,
             T: float = 0.25,
             y_max: float = 1.0,
             sigma_xy: float = 5.0,
             tau_mean: float = 10.0,
             sigma_xy_of_n=None) -> Events:
    """Draw ``n_events`` events.

    ``multiplicity`` is either a float (Poisson mean), an int array of
    explicit per-event multiplicities, or a callable ``rng -> int array``.
    ``sigma_xy_of_n`` optionally maps each event's multiplicity to its
    transverse source size (the uneven-multiplicity workload uses
    1.2 * N^(1/3) fm).
    """
    rng = np.random.default_rng(seed)
    if callable(multiplicity):
        mult = np.asarray(multiplicity(rng), dtype=np.int64)
    elif np.ndim(multiplicity) == 0:
        mult = rng.poisson(float(multiplicity), size=n_events).astype(np.int64)
    else:
        mult = np.asarray(multiplicity, dtype=np.int64)
    assert mult.size == n_events
    n = int(mult.sum())
    offsets = np.zeros(n_events + 1, dtype=np.int64)
    np.cumsum(mult, out=offsets[1:])

    pT = rng.exponential(T, size=n)
    phi = rng.uniform(0.0, 2.0 * np.pi, size=n)
    rap = rng.uniform(-y_max, y_max, size=n)
    mT = np.sqrt(pT * pT + mass * mass)
    E = mT * np.cosh(rap)
    pz = mT * np.sinh(rap)
    px = pT * np.cos(phi)
    py = pT * np.sin(phi)

    if sigma_xy_of_n is not None:
        sig = np.repeat(np.asarray([sigma_xy_of_n(int(m)) for m in mult]), mult)
    else:
        sig = np.full(n, float(sigma_xy))
    x = rng.normal(0.0, 1.0, size=n) * sig
    y = rng.normal(0.0, 1.0, size=n) * sig
    eta_s = rng.uniform(-1.0, 1.0, size=n)
    tau = rng.exponential(tau_mean, size=n)
    t = tau * np.cosh(eta_s)
    z = tau * np.sinh(eta_s)
    return Events(offsets, np.full(n, monval, dtype=np.int32),
                  np.full(n, mass), t, x, y, z, E, px, py, pz)


def _g17(a: np.ndarray):
    return ["%.17g" % v for v in a.tolist()]


def write_mode10(path: str, ev: Events, compresslevel: int = 1) -> None:
    """Write ``ev`` as an iSS gzip sample file (``read_in_mode = 10``)."""
    with gzip.open(path, "wt", compresslevel=compresslevel, newline="\n") as f:
        cols = [_g17(getattr(ev, k)) for k in
                ("mass", "t", "x", "y", "z", "E", "px", "py", "pz")]
        mon = [str(int(v)) for v in ev.monval.tolist()]
        for e in range(ev.n_events):
            a, b = int(ev.offsets[e]), int(ev.offsets[e + 1])
            f.write("%d\n" % (b - a))
            for k in range(a, b):
                f.write(mon[k] + " " + " ".join(c[k] for c in cols) + "\n")


def write_oscar(path: str, ev: Events) -> None:
    """Write ``ev`` as an OSCAR text file (``read_in_mode = 0``)."""
    with open(path, "w", newline="\n") as f:
        f.write("OSC1997A\nfinal_id_p_x\n synthetic emission source\n")
        cols = [_g17(getattr(ev, k)) for k in
                ("px", "py", "pz", "E", "mass", "x", "y", "z", "t")]
        mon = [str(int(v)) for v in ev.monval.tolist()]
        for e in range(ev.n_events):
            a, b = int(ev.offsets[e]), int(ev.offsets[e + 1])
            f.write("%d %d 0 0\n" % (e + 1, b - a))
            for i, k in enumerate(range(a, b)):
                f.write("%d %s %s\n" % (i + 1, mon[k], " ".join(c[k] for c in cols)))


def buffers(ev: Events, event_buffer_size: int):
    """Split events into the reader's buffers (oversample groups).

    Whole events are taken until the running particle count reaches
    ``event_buffer_size`` (src/particleSamples.cpp:1256-1283).  Returns a
    list of ``(first_event, last_event_exclusive)``.
    """
    out = []
    e = 0
    mult = ev.multiplicities()
    while e < ev.n_events:
        start = e
        count = 0
        while count < event_buffer_size and e < ev.n_events:
            count += int(mult[e])
            e += 1
        out.append((start, e))
    return out


def subset(ev: Events, first: int, last: int) -> Events:
    a, b = int(ev.offsets[first]), int(ev.offsets[last])
    fields = ("monval", "mass", "t", "x", "y", "z", "E", "px", "py", "pz")
    return Events(ev.offsets[first:last + 1] - a,
                  *[getattr(ev, f)[a:b] for f in fields])


# Named workloads --------------------------------------------------------

def small_pions(n_events: int = 100, mu: float = 500.0, seed: int = 1) -> Events:
    """100 pi+ events, Poisson(500), T=0.25 GeV, sigma_xy=5 fm, tau0=10 fm/c."""
    return generate(n_events, mu, seed=seed, sigma_xy=5.0, tau_mean=10.0)


def central_pions(n_events: int = 1000, mu: float = 1500.0, seed: int = 1) -> Events:
    """1000 pi+ events, Poisson(1500), sigma_xy=7 fm, tau0=12 fm/c."""
    return generate(n_events, mu, seed=seed, sigma_xy=7.0, tau_mean=12.0)


def central_kaons(n_events: int = 1000, mu: float = 250.0, seed: int = 2) -> Events:
    """K+ events, Poisson(250), T=0.30 GeV, same source as central pions."""
    return generate(n_events, mu, seed=seed, mass=KAON_MASS, monval=321,
                    T=0.30, sigma_xy=7.0, tau_mean=12.0)


def uneven_pions(n_events: int = 4096, lo: int = 20, hi: int = 3000,
                 seed: int = 3) -> Events:
    """Log-uniform multiplicities in [lo, hi]; sigma_xy = 1.2 N^(1/3) fm."""
    def mult(rng):
        u = rng.uniform(np.log(lo), np.log(hi), size=n_events)
        return np.floor(np.exp(u)).astype(np.int64)
    return generate(n_events, mult, seed=seed, tau_mean=10.0,
                    sigma_xy_of_n=lambda m: 1.2 * max(m, 1) ** (1.0 / 3.0))
