"""Helpers shared by the GPU parity tests: seeded particle lists and the
engine-versus-oracle comparison.

Tolerances (FP64 form): pair counts, denominators and pair counters must be
identical.  The q sums and the cos(q.dx) numerator are FP64 sums whose order
differs from the oracle's (and the device cos differs from glibc's in the
last ulps), so per bin |engine - oracle| <= RTOL * count * scale with
RTOL = 1e-12 and scale = max|q| of the window (q sums) or 1 (cos sums).
"""
import numpy as np

RTOL = 1e-12


def lists(seed, n_events=6, mu=60.0, sigma_xy=2.0, tau=3.0, mass=0.13957):
    from hadronic_afterburner_toolkit_gb300 import synth
    ev = synth.generate(n_events, mu, seed=seed, sigma_xy=sigma_xy, tau_mean=tau, mass=mass)
    return ev


def cols8(ev, a=None, b=None):
    sl = slice(a, b)
    return [np.ascontiguousarray(getattr(ev, k)[sl]) for k in
            ("px", "py", "pz", "E", "x", "y", "z", "t")]


def rotated4(ev, angle, a=None, b=None):
    sl = slice(a, b)
    c, s = np.cos(angle), np.sin(angle)
    px, py = ev.px[sl], ev.py[sl]
    return [np.ascontiguousarray(px * c - py * s), np.ascontiguousarray(px * s + py * c),
            np.ascontiguousarray(ev.pz[sl]), np.ascontiguousarray(ev.E[sl])]


def compare(eng_h, orc_h, q_scale, rtol=RTOL, exact_sums=False):
    """Asserts parity; returns the worst relative sum errors seen."""
    for k in ("count", "den", "qinv_count", "qinv_den", "ctr_num", "ctr_den",
              "ctr_num_qinv", "ctr_den_qinv"):
        a, b = np.asarray(eng_h[k]), np.asarray(orc_h[k])
        assert a.shape == b.shape, k
        bad = np.nonzero(a != b)[0]
        assert bad.size == 0, "%s differs at %d bins, first %s: %s vs %s" % (
            k, bad.size, bad[:5], a[bad[:5]], b[bad[:5]])
    assert eng_h["pairs_same"] == orc_h["pairs_same"]
    assert eng_h["pairs_mixed"] == orc_h["pairs_mixed"]
    assert eng_h["anomalies"] == orc_h["anomalies"]
    worst = {}
    for k, cnt, scale in (("q_out", "count", q_scale), ("q_side", "count", q_scale),
                          ("q_long", "count", q_scale), ("num", "count", 1.0),
                          ("qinv_sum", "qinv_count", q_scale), ("qinv_num", "qinv_count", 1.0)):
        a, b = np.asarray(eng_h[k]), np.asarray(orc_h[k])
        bound = rtol * np.maximum(orc_h[cnt], 1.0) * scale
        err = np.abs(a - b)
        if exact_sums:
            assert np.array_equal(a, b), k
        assert (err <= bound).all(), "%s: max err %g (bound %g)" % (
            k, err.max(), bound[np.argmax(err - bound)])
        denom = np.maximum(orc_h[cnt] * scale, 1e-300)
        worst[k] = float((err / denom).max()) if err.size else 0.0
    return worst


def _parse_table(text):
    rows = []
    for line in text.strip().split("\n"):
        if line.lstrip().startswith("#"):
            continue
        rows.append([float("nan") if "nan" in tok else float(tok) for tok in line.split()])
    return np.array(rows)


def same_output_file(got: bytes, want: bytes, fname: str) -> None:
    """Asserts that an HBT_correlation_function file matches the reference's.

    The golden files were written by the reference built on x86-64.  On an
    x86-64 host the oracle and the writer reproduce them byte for byte.  On
    another architecture glibc's cos / atan2 may differ in the last ulp, which
    can change the last printed digit or the sign of a sum that is zero up to
    rounding; there the denominator column must still be identical and every
    other column must agree to 2e-8 relative (the printed precision) or 1e-9
    absolute."""
    import platform
    if platform.machine() in ("x86_64", "AMD64"):
        assert got == want, "%s differs from the reference" % fname
        return
    g, w = _parse_table(got.decode()), _parse_table(want.decode())
    assert g.shape == w.shape, fname
    assert np.array_equal(g[:, -1], w[:, -1], equal_nan=True), fname
    for col in range(g.shape[1] - 1):
        ok = np.isclose(g[:, col], w[:, col], rtol=2e-8, atol=1e-9, equal_nan=True)
        assert ok.all(), "%s: column %d rows %s" % (fname, col, np.nonzero(~ok)[0][:5])
