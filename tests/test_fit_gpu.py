"""Batched radii fits on the GPU (include/hbt_fit.h) against the rows the
reference's own fit script stored for the fixture database
(tests/golden_fit/expected.json) and against the scipy oracle
(oracle/fit_radii.py).

Both sides minimise the same chi^2. scipy stops when an iteration lowers
chi^2 by less than ftol = 1.49e-8 of it, which leaves each parameter up to
sqrt(ftol chi^2) standard errors (0.004 to 0.02 here) from the minimum, and
it differentiates by finite differences; the GPU iterates to a 1e-14
relative change with the analytic Jacobian. The tolerance is 1e-3 of each
parameter's error for the parameters (measured: at most 1.3e-4). scipy's
covariance comes from the Jacobian at the iterate before its last step,
up to 0.02 standard errors away; R_os and R_ol enter squared, so their
errors scale with 1 / R and move by that fraction times sigma / R: the
errors' tolerance is 1e-4 + 0.02 sigma / |p| relative."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden_fit"))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

pytestmark = pytest.mark.gpu


def _close(got, want):
    p, e = got[..., 1::2], got[..., 2::2]
    pw, ew = want[..., 1::2], want[..., 2::2]
    assert np.all(np.abs(p - pw) <= 1e-3 * ew + 1e-9 * np.abs(pw)), np.max(np.abs(p - pw) / ew)
    rtol = 1e-4 + 0.02 * ew / np.abs(pw)
    assert np.all(np.abs(e - ew) <= rtol * ew), np.max(np.abs(e - ew) / ew)


def _fixture():
    import tables
    expected = json.load(open(os.path.join(HERE, "golden_fit", "expected.json")))
    db = tables.database()
    keys, tabs, want = [], [], []
    for ev, per_kt in expected["fits"].items():
        for kt, rows in per_kt.items():
            keys.append((ev, kt))
            tabs.append(db[ev]["HBT_correlation_function_KT_%s.dat" % kt])
            want.append(rows)
    return keys, tabs, np.array(want)


def test_fits_match_reference_script():
    from hadronic_afterburner_toolkit_gb300 import radii
    keys, tabs, want = _fixture()
    f = radii.Fitter()
    got = f.fit(tabs)
    assert got.shape == want.shape == (len(tabs), 5, 13)
    np.testing.assert_array_equal(got[..., 0], want[..., 0])
    _close(got, want)
    assert np.all(f.last["status"] == 0)
    st = f.stats()
    assert st["fits"] == len(tabs) * 5 and st["passes"] >= st["fits"]
    assert st["points"] == int(f.last["n_points"].sum())


def test_batching_and_layouts_do_not_change_results():
    """One call for all tables equals one call per table bit for bit; a
    table with extra columns (stride 11) and the same table as five
    separate column arrays (stride 1, packed on the host) fit the same; the
    cut list in another order gives the same fit per cut."""
    from hadronic_afterburner_toolkit_gb300 import radii
    _, tabs, _ = _fixture()
    f = radii.Fitter()
    together = f.fit(tabs)
    for k, t in enumerate(tabs[:3]):
        np.testing.assert_array_equal(f.fit([t])[0], together[k])
    wide = np.concatenate([tabs[0], np.zeros((tabs[0].shape[0], 3))], axis=1)
    np.testing.assert_array_equal(f.fit([wide])[0], together[0])
    t = tabs[1]
    cols = (t[:, 0].copy(), t[:, 1].copy(), t[:, 2].copy(), t[:, 6].copy(), t[:, 7].copy())
    mixed = f.fit([cols, tabs[0]])
    np.testing.assert_array_equal(mixed[0], together[1])
    np.testing.assert_array_equal(mixed[1], together[0])
    cuts = [0.125, 0.05, 0.15, 0.1, 0.075]
    perm = f.fit(tabs[:2], q_cut_max_list=cuts)
    for j, c in enumerate(cuts):
        k = list(radii.Q_CUT_MAX_LIST).index(c)
        np.testing.assert_array_equal(perm[:, j], together[:2, k])


def test_lower_cut_empty_and_degenerate_tables():
    """q_cut_min > 0 against the oracle; a cut with fewer than six rows
    reports too-few with NaN; NaN rows inside the cuts become zeros with
    weight 1e15, which pins lambda to 0 in both (the script's nan_to_num
    behaviour)."""
    import fit_radii
    import tables
    from hadronic_afterburner_toolkit_gb300 import radii
    f = radii.Fitter()
    t = tables.make_table(5, (0.5, 5.0, 4.5, 5.5, 1.0, 0.7))
    got = f.fit([t], q_cut_min=0.03)
    _close(got[0], fit_radii.fit_table(t, q_cut_min=0.03))
    tiny = f.fit([t], q_cut_max_list=[0.001, 0.1])
    assert f.last["status"][0, 0] == 3 and np.isnan(tiny[0, 0, 1:]).all()
    _close(tiny[0, 1:], fit_radii.fit_table(t, q_cut_max_list=[0.1]))
    holes = tables.make_table(6, (0.5, 5.0, 4.5, 5.5, 1.0, 0.7), blank_every=3,
                              blank_beyond=0.0)
    g = f.fit([holes], q_cut_max_list=[0.1])
    o = fit_radii.fit_table(holes, q_cut_max_list=[0.1])
    assert abs(g[0, 0, 1]) < 1e-6 and abs(o[0, 1]) < 1e-6


def test_many_tables_against_oracle():
    """Forty tables of varied sources and noise, two launches' worth of
    fits, against the oracle."""
    import fit_radii
    import tables
    from hadronic_afterburner_toolkit_gb300 import radii
    rng = np.random.default_rng(3)
    tabs = []
    for k in range(40):
        p = (rng.uniform(0.3, 0.9), rng.uniform(3, 8), rng.uniform(3, 7), rng.uniform(3, 9),
             rng.uniform(0.6, 2.0), rng.uniform(0.5, 1.6))
        tabs.append(tables.make_table(100 + k, p, noise=rng.uniform(0.01, 0.05)))
    got = radii.Fitter().fit(tabs)
    for k in range(0, 40, 5):
        _close(got[k], fit_radii.fit_table(tabs[k]))


def test_dropin_writes_radii_beside_the_tables(tmp_path):
    import tables
    from hadronic_afterburner_toolkit_gb300 import radii
    keys, tabs, want = _fixture()
    for (ev, kt), t in zip(keys, tabs):
        d = tmp_path / ev
        d.mkdir(exist_ok=True)
        np.savetxt(d / ("HBT_correlation_function_KT_%s.dat" % kt), t, fmt="%.17g")
    assert radii.fit_database(str(tmp_path), verbose=False) == len(keys)
    for (ev, kt), w in zip(keys, want):
        path = tmp_path / ev / ("HBT_radii_KT_%s.dat" % kt)
        assert open(path).readline().rstrip("\n") == radii.HEADER
        _close(np.loadtxt(path), w)


def test_empty_calls_and_tables():
    """No tables; a table of no rows and one of five rows (too few for six
    parameters) beside a normal one; a fit limited to two iterations
    reports the iteration limit with the best point found."""
    import tables
    from hadronic_afterburner_toolkit_gb300 import radii
    f = radii.Fitter()
    assert f.fit([]).shape == (0, 5, 13)
    t = tables.make_table(9, (0.5, 5.0, 4.5, 5.5, 1.0, 0.7))
    rows = f.fit([np.zeros((0, 8)), t[:5], t])
    assert (f.last["status"][0] == 3).all() and (f.last["status"][1] == 3).all()
    assert np.isnan(rows[0, :, 1:]).all() and np.isnan(rows[1, :, 1:]).all()
    assert (f.last["status"][2] == 0).all()
    np.testing.assert_array_equal(rows[2], f.fit([t])[0])
    f.fit([t], max_iterations=2)
    assert (f.last["status"] == 1).all() and (f.last["iterations"] == 2).all()
