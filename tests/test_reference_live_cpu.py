"""The oracle against the reference itself, run live on this machine.

Where the reference checkout is present, the build step compiles the
unmodified reference into oracle/_ref (oracle/Makefile, from its own
sources).  Then:

* every committed golden case is regenerated with that binary from the
  same seeded inputs, and its output files and logged pair counts equal the
  committed ones (the fixtures are the reference's own outputs);
* two cases that are not among the fixtures (K_phi bins with q_inv
  histograms and binding caps; no longitudinal boost with a rapidity shift,
  K_T and rapidity cuts and an asymmetric q grid), and a seeded sweep of 24
  random parameter sets (make_golden.random_case) plus 8 on the OSCAR
  reader with mixed species (random_oscar_case), run through the
  reference binary and through the oracle: every output file byte-identical
  (x86-64; to the printed precision elsewhere) and the same logged pair
  totals;
* the balance-function path likewise: every committed balance-function
  fixture regenerated, and a seeded sweep of 16 random balance-function
  parameter sets (make_golden_bf.random_case: species pairs, rapidity or
  pseudorapidity, Delta y grids, p_T windows, shifts, buffer sizes, both
  readers, real mixed events) through the reference and the balance-function
  oracle, byte-identical.

Skipped where there is no reference checkout (the GPU machine).
"""
import os
import sys
import tarfile

import numpy as np
import pytest

import oracle_lib
import parity

sys.path.insert(0, os.path.join(oracle_lib.REPO, "tests", "golden"))
sys.path.insert(0, os.path.join(oracle_lib.REPO, "tests", "golden_bf"))
import make_golden  # noqa: E402
import make_golden_bf  # noqa: E402

REF_ROOT = oracle_lib.reference_checkout()
pytestmark = [
    pytest.mark.slow,
    pytest.mark.skipif(not REF_ROOT or not os.path.exists(make_golden.REF_BIN),
                       reason="no reference checkout or no oracle/_ref binary"),
]

LIVE_CASES = {
    "live_kphi_qinv_cap": dict(
        events=lambda: make_golden._events_basic(seed=77, n_events=28, mu=55.0),
        params={"azimuthal_flag": 1, "n_Kphi": 5, "invariant_radius_flag": 1,
                "needed_number_of_pairs": 30, "qnpts": 9, "event_buffer_size": 160}),
    "live_noboost_cuts": dict(
        events=lambda: make_golden._events_basic(seed=78, n_events=20, mu=45.0),
        params={"long_comoving_boost": 0, "rapidity_shift": -0.2, "KT_min": 0.1,
                "KT_max": 0.8, "n_KT": 6, "HBTrap_min": -0.7, "HBTrap_max": 0.6,
                "q_min": -0.12, "q_max": 0.18, "qnpts": 13}),
}


def _outputs(case_dir):
    out = {}
    with tarfile.open(os.path.join(case_dir, "outputs.tar.gz")) as tar:
        for m in tar.getmembers():
            out[m.name] = tar.extractfile(m).read()
    return out


def _pair_totals(case_dir):
    lines = open(os.path.join(case_dir, "pairs.txt")).read().split("\n")
    same = sum(int(l.split(":")[1]) for l in lines if l.startswith("pairs:"))
    mixed = sum(int(l.split(":")[1]) for l in lines if l.startswith("mixed pairs:"))
    return same, mixed


@pytest.mark.parametrize("name", sorted(make_golden.CASES))
def test_committed_fixture_is_the_reference_output(name, tmp_path):
    make_golden.run_case(name, make_golden.CASES[name], REF_ROOT, out_root=str(tmp_path))
    fresh = os.path.join(str(tmp_path), name)
    committed = os.path.join(oracle_lib.GOLDEN, name)
    assert _outputs(fresh) == _outputs(committed)
    assert (open(os.path.join(fresh, "pairs.txt")).read()
            == open(os.path.join(committed, "pairs.txt")).read())


@pytest.mark.parametrize("name", sorted(LIVE_CASES))
def test_oracle_matches_reference_on_a_new_case(name, tmp_path):
    make_golden.run_case(name, LIVE_CASES[name], REF_ROOT, out_root=str(tmp_path))
    case_dir = os.path.join(str(tmp_path), name)
    want = _outputs(case_dir)
    out_dir = os.path.join(str(tmp_path), "oracle_out")
    os.makedirs(out_dir)
    orc = oracle_lib.run_golden_case_through_oracle(name, out_dir, root=str(tmp_path))
    got = {f: open(os.path.join(out_dir, f), "rb").read() for f in os.listdir(out_dir)}
    assert sorted(got) == sorted(want) and want
    for f in want:
        parity.same_output_file(got[f], want[f], f)
    h = orc.hist()
    assert (h["pairs_same"], h["pairs_mixed"]) == _pair_totals(case_dir)
    cap = LIVE_CASES[name]["params"].get("needed_number_of_pairs")
    if cap is not None:
        # the cap binds: some slot's counter ran one past it
        assert (np.asarray(h["ctr_num"]) == cap + 1).any()


@pytest.mark.parametrize("kind,k", [("mode10", k) for k in range(24)] +
                         [("oscar", k) for k in range(8)])
def test_oracle_matches_reference_on_random_parameter_sets(kind, k, tmp_path):
    """A seeded sweep of parameter sets through the reference binary and
    the oracle: byte-identical files and the same pair totals.  "oscar":
    the OSCAR reader with mixed species and, in some cases, a real
    mixed-event file."""
    name = "sweep_%s_%02d" % (kind, k)
    case = make_golden.random_case(k) if kind == "mode10" else make_golden.random_oscar_case(k)
    make_golden.run_case(name, case, REF_ROOT, out_root=str(tmp_path))
    case_dir = os.path.join(str(tmp_path), name)
    want = _outputs(case_dir)
    out_dir = os.path.join(str(tmp_path), "oracle_out")
    os.makedirs(out_dir)
    orc = oracle_lib.run_golden_case_through_oracle(name, out_dir, root=str(tmp_path))
    got = {f: open(os.path.join(out_dir, f), "rb").read() for f in os.listdir(out_dir)}
    assert sorted(got) == sorted(want) and want
    for f in want:
        parity.same_output_file(got[f], want[f], f)
    h = orc.hist()
    assert (h["pairs_same"], h["pairs_mixed"]) == _pair_totals(case_dir)


def _bf_outputs(case_dir):
    return _outputs(case_dir)


@pytest.mark.parametrize("name", sorted(make_golden_bf.CASES))
def test_committed_bf_fixture_is_the_reference_output(name, tmp_path):
    make_golden_bf.run_case(name, make_golden_bf.CASES[name], REF_ROOT, out_root=str(tmp_path))
    assert (_bf_outputs(os.path.join(str(tmp_path), name))
            == _bf_outputs(os.path.join(oracle_lib.GOLDEN_BF, name)))


@pytest.mark.parametrize("k", range(16))
def test_bf_oracle_matches_reference_on_random_parameter_sets(k, tmp_path):
    name = "bfsweep%02d" % k
    make_golden_bf.run_case(name, make_golden_bf.random_case(k), REF_ROOT,
                            out_root=str(tmp_path))
    want = _bf_outputs(os.path.join(str(tmp_path), name))
    out_dir = os.path.join(str(tmp_path), "oracle_out")
    os.makedirs(out_dir)
    oracle_lib.run_bf_golden_case_through_oracle(name, out_dir, root=str(tmp_path))
    got = {f: open(os.path.join(out_dir, f), "rb").read() for f in os.listdir(out_dir)}
    assert sorted(got) == sorted(want) and len(want) == 3
    for f in want:
        parity.same_output_file(got[f], want[f], f)
