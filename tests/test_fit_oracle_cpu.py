"""The radii-fit oracle (oracle/fit_radii.py) against the rows the
reference's own script stored for the fixture database
(tests/golden_fit/expected.json, made by tests/golden_fit/make_golden_fit.py).
Same scipy algorithm on the same tables: the parameters agree to a small
fraction of their errors, the errors to 1e-6 relative."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden_fit"))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

pytest.importorskip("scipy")


def test_oracle_matches_reference_script():
    import fit_radii
    import tables
    expected = json.load(open(os.path.join(HERE, "golden_fit", "expected.json")))
    assert expected["header"] == fit_radii.HEADER
    db = tables.database()
    for ev, per_kt in expected["fits"].items():
        for kt, rows in per_kt.items():
            got = fit_radii.fit_table(db[ev]["HBT_correlation_function_KT_%s.dat" % kt])
            want = np.array(rows)
            assert got.shape == want.shape == (5, 13)
            np.testing.assert_array_equal(got[:, 0], want[:, 0])
            p, e = got[:, 1::2], got[:, 2::2]
            pw, ew = want[:, 1::2], want[:, 2::2]
            assert np.all(np.abs(p - pw) <= 1e-6 * ew + 1e-12 * np.abs(pw)), (ev, kt)
            np.testing.assert_allclose(e, ew, rtol=1e-6)
