"""The radii-fit oracle (oracle/fit_radii.py) against the reference's own
script (ebe_scripts/fit_HBT_radii.py), run live where the reference
checkout is on this machine (through the h5py stand-in of
tests/golden_fit/make_golden_fit.py):

* the committed fixture rows (tests/golden_fit/expected.json) are what the
  script stores for the fixture database now;
* on four random databases (tests/golden_fit/tables.random_database: source
  parameters, noise, grid size and empty bins drawn from a seed) the
  oracle's rows agree with the script's: the q cuts exactly, the parameters
  to 1e-6 of their errors, the errors to 1e-6 relative.

Skipped where there is no reference checkout.
"""
import json
import os
import sys

import numpy as np
import pytest

import oracle_lib

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden_fit"))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

pytest.importorskip("scipy")
REF_ROOT = oracle_lib.reference_checkout()
pytestmark = [
    pytest.mark.slow,
    pytest.mark.skipif(not REF_ROOT or not os.path.exists(
        os.path.join(REF_ROOT, "ebe_scripts", "fit_HBT_radii.py")),
        reason="no reference checkout"),
]


def _compare(got, want, where):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape == (5, 13), where
    np.testing.assert_array_equal(got[:, 0], want[:, 0])
    p, e = got[:, 1::2], got[:, 2::2]
    pw, ew = want[:, 1::2], want[:, 2::2]
    assert np.all(np.abs(p - pw) <= 1e-6 * ew + 1e-12 * np.abs(pw)), where
    np.testing.assert_allclose(e, ew, rtol=1e-6, err_msg=str(where))


def test_committed_fit_fixture_is_the_reference_output():
    import make_golden_fit
    import tables
    header, fits = make_golden_fit.reference_fits(REF_ROOT, tables.database())
    expected = json.load(open(os.path.join(HERE, "golden_fit", "expected.json")))
    assert header.decode() == expected["header"]
    assert sorted(fits) == sorted(expected["fits"])
    for ev in fits:
        for cut in fits[ev]:
            _compare(fits[ev][cut], expected["fits"][ev][cut], (ev, cut))


# some random tables make both the script's and the oracle's model overflow
# in exp while the fit wanders, or leave a covariance that cannot be
# estimated (infinite errors); both warn the same way and store the same rows
@pytest.mark.filterwarnings("ignore::RuntimeWarning")
@pytest.mark.filterwarnings("ignore::scipy.optimize.OptimizeWarning")
@pytest.mark.parametrize("seed", range(4))
def test_fit_oracle_matches_reference_script_on_random_databases(seed):
    import fit_radii
    import make_golden_fit
    import tables
    db = tables.random_database(100 + seed)
    header, fits = make_golden_fit.reference_fits(REF_ROOT, db)
    assert header.decode() == fit_radii.HEADER
    for ev, per_cut in fits.items():
        for cut, rows in per_cut.items():
            got = fit_radii.fit_table(db[ev]["HBT_correlation_function_KT_%s.dat" % cut])
            _compare(got, rows, (seed, ev, cut))
