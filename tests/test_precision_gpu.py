"""FP32-weight (hbt_precision = 1) and double-float (2) forms against the
FP64 oracle.

Bins and every count stay exact: the FP32 screen decides bins with error
bounds and the reference chain decides the rest, as in the FP64 form.  The
summed values change precision: q_out / q_side / q_long are the FP32 screen
values (relative error < 1e-6) and cos(q.dx / hbarC) is evaluated in FP32
after an FP64 phase and range reduction (absolute error < 2e-7).  They are
accumulated into FP32 partial bins, merged into the FP64 bins with Kahan
compensation every 8192 same-event tile pairs (pairs of even and odd
warps in two partial arrays).  Stated per-bin bound checked here:
|sum - oracle| <= 1e-5 * count * scale (scale = max|q| of the window, or 1
for the cos numerator).
"""
import numpy as np
import pytest

import oracle_lib
import parity

pytestmark = pytest.mark.gpu

P = dict(qnpts=15, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=4,
         azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
         needed_number_of_pairs=1e18)
RTOL32 = 1e-5


def _qscale(p):
    return max(abs(p["q_min"]), abs(p["q_max"])) + (p["q_max"] - p["q_min"]) / (p["qnpts"] - 1)


@pytest.mark.parametrize("az", [0, 1])
def test_fp32w_counts_exact_sums_within_bound(az):
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(P, azimuthal_flag=az)
    ev = parity.lists(seed=606, n_events=8, mu=90.0)
    c = parity.cols8(ev)
    eng = E.Engine(precision=E.PRECISION_FP32W, **p)
    orc = oracle_lib.Oracle(**p)
    for x in (eng, orc):
        x.set_psi_ref(0.25)
        x.bin_same(c)
        x.bin_mixed(c[:4], [v[::-1].copy() for v in c[:4]])
    h = orc.hist()
    assert h["count"].sum() > 1000
    worst = parity.compare(eng.hist(), h, _qscale(p), rtol=RTOL32)
    # the error is far below the stated bound in practice
    assert worst["num"] < 1e-6 and worst["q_out"] < 1e-6


def test_fp32w_and_fp64_forms_bin_identically():
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(P, azimuthal_flag=1, n_Kphi=8)
    ev = parity.lists(seed=707, n_events=10, mu=80.0)
    c = parity.cols8(ev)
    hs = []
    for prec in (E.PRECISION_FP64, E.PRECISION_FP32W):
        eng = E.Engine(precision=prec, **p)
        eng.set_psi_ref(-0.6)
        eng.bin_same(c)
        eng.bin_same(c)  # twice: partials merged into accumulated bins
        hs.append(eng.hist())
    for k in ("count", "ctr_num"):
        assert np.array_equal(hs[0][k], hs[1][k])
    m = hs[0]["count"] > 0
    rel = np.abs(hs[0]["num"][m] - hs[1]["num"][m]) / hs[0]["count"][m]
    assert rel.max() < 1e-6


# Double-float form (hbt_precision = 2): the same-event q sums and cos(q.dx)
# are computed in double-float arithmetic (hi + lo FP32 pairs: 48
# significant bits per input, momenta split relative to each tile's first
# row; about 2^-46 relative per operation chain) and added to the FP64 bins.
# A pair's phase error is then about 2^-46 times the phase plus the
# splitting errors of the inputs times their partners in q.dx, e.g. 1e-12 at
# a phase of 60 rad with emission times of 140 fm/c.  Stated per-bin bound:
# |sum - oracle| <= 1e-11 * count * scale (scale as for the FP32 form).
RTOL_DF = 1e-11


@pytest.mark.parametrize("az,boost", [(0, 1), (1, 1), (0, 0)])
def test_df64_counts_exact_sums_within_fp64_bound(az, boost):
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(P, azimuthal_flag=az, long_comoving_boost=boost)
    ev = parity.lists(seed=808 + az + 2 * boost, n_events=8, mu=90.0)
    c = parity.cols8(ev)
    eng = E.Engine(precision=E.PRECISION_DF64, **p)
    orc = oracle_lib.Oracle(**p)
    for x in (eng, orc):
        x.set_psi_ref(0.25)
        x.bin_same(c)
        x.bin_mixed(c[:4], [v[::-1].copy() for v in c[:4]])
    h = orc.hist()
    assert h["count"].sum() > 1000
    parity.compare(eng.hist(), h, _qscale(p), rtol=RTOL_DF)


@pytest.mark.parametrize("kernel", [0, 2])
def test_df64_large_source_against_oracle(kernel):
    """A source of 8 fm and emission times of 12 fm/c on average, up to
    140 fm/c (phases up to about 100 rad), through the batched path (kernel
    0) and the screened grid (kernel 2)."""
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(P, q_min=-0.25, q_max=0.25)
    ev = parity.lists(seed=909, n_events=6, mu=120.0, sigma_xy=8.0, tau=12.0)
    c = parity.cols8(ev)
    eng = E.Engine(precision=E.PRECISION_DF64, kernel=kernel, **p)
    orc = oracle_lib.Oracle(**p)
    for x in (eng, orc):
        x.set_psi_ref(0.0)
        x.bin_same(c)
    h = orc.hist()
    assert h["count"].sum() > 1000
    parity.compare(eng.hist(), h, _qscale(p), rtol=RTOL_DF)


def test_df64_and_fp64_forms_bin_identically():
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(P, azimuthal_flag=1, n_Kphi=8)
    ev = parity.lists(seed=1010, n_events=10, mu=80.0)
    c = parity.cols8(ev)
    hs = []
    for prec in (E.PRECISION_FP64, E.PRECISION_DF64):
        eng = E.Engine(precision=prec, **p)
        eng.set_psi_ref(-0.6)
        eng.bin_same(c)
        hs.append(eng.hist())
    for k in ("count", "ctr_num"):
        assert np.array_equal(hs[0][k], hs[1][k])
    m = hs[0]["count"] > 0
    rel = np.abs(hs[0]["num"][m] - hs[1]["num"][m]) / hs[0]["count"][m]
    assert rel.max() < RTOL_DF
