"""Pin the CPU oracle to the reference: byte-identical output files.

Every golden case (tests/golden/<case>/) holds the input and parameters the
reference binary was run on and every HBT_correlation_function_*.dat it
wrote.  The oracle, replayed over the same input, must reproduce each file
byte for byte on x86-64 (same pair loops, same cap order, same RNG draws for
the mixed-event partners and rotations, same glibc cos/atan2, same writer);
on another architecture to the printed precision (parity.same_output_file).
"""
import os
import tarfile

import pytest

import oracle_lib
import parity

CASES = sorted(d for d in os.listdir(oracle_lib.GOLDEN)
               if os.path.exists(os.path.join(oracle_lib.GOLDEN, d, "parameters.dat")))


def _golden_files(name):
    out = {}
    with tarfile.open(os.path.join(oracle_lib.GOLDEN, name, "outputs.tar.gz")) as tar:
        for m in tar.getmembers():
            out[m.name] = tar.extractfile(m).read()
    return out


def _pair_lines(name):
    return open(os.path.join(oracle_lib.GOLDEN, name, "pairs.txt")).read().split("\n")


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_files(name, tmp_path):
    orc = oracle_lib.run_golden_case_through_oracle(name, str(tmp_path))
    want = _golden_files(name)
    got = {f: open(os.path.join(tmp_path, f), "rb").read() for f in os.listdir(tmp_path)}
    assert sorted(got) == sorted(want)
    for f in want:
        parity.same_output_file(got[f], want[f], f)
    # the logged candidate-pair totals agree too
    lines = _pair_lines(name)
    same = sum(int(l.split(":")[1]) for l in lines if l.startswith("pairs:"))
    mixed = sum(int(l.split(":")[1]) for l in lines if l.startswith("mixed pairs:"))
    h = orc.hist()
    assert h["pairs_same"] == same
    assert h["pairs_mixed"] == mixed
    assert h["anomalies"] == 0


def test_caps_bind_in_cap_cases():
    """The cap fixtures really exercise order-dependent admission."""
    for name in ("cap", "cap_kphi"):
        prm, _, _ = oracle_lib.golden_case(name)
        import tempfile
        with tempfile.TemporaryDirectory() as d:
            h = oracle_lib.run_golden_case_through_oracle(name, d).hist()
        cap = int(prm["needed_number_of_pairs"])
        assert (h["ctr_num"] == cap + 1).any()
        assert (h["ctr_den"] == cap + 1).any()
