"""Pin the balance-function oracle to the reference: its three output files
are the reference binary's (tests/golden_bf/, made by make_golden_bf.py),
byte for byte on x86-64 (parity.same_output_file)."""
import os
import tarfile

import pytest

import oracle_lib
import parity

CASES = sorted(d for d in os.listdir(oracle_lib.GOLDEN_BF)
               if os.path.exists(os.path.join(oracle_lib.GOLDEN_BF, d, "parameters.dat")))


@pytest.mark.parametrize("name", CASES)
def test_bf_oracle_reproduces_reference_files(name, tmp_path):
    oracle_lib.run_bf_golden_case_through_oracle(name, str(tmp_path))
    with tarfile.open(os.path.join(oracle_lib.GOLDEN_BF, name, "outputs.tar.gz")) as tar:
        want = {m.name: tar.extractfile(m).read() for m in tar.getmembers()}
    got = {f: open(os.path.join(tmp_path, f), "rb").read() for f in os.listdir(tmp_path)}
    assert sorted(got) == sorted(want) and len(want) == 3
    for f in want:
        parity.same_output_file(got[f], want[f], f)
