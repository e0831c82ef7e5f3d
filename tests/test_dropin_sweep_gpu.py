"""The drop-in executable on the GPU against the oracle over a seeded sweep
of parameter sets.

make_golden.random_case(k) draws case k: grid size (odd and even),
symmetric or asymmetric q window (one without q = 0), K_T edges and range,
longitudinal boost, K_phi bins, q_inv histograms, a pair cap that binds or
not, buffer size (down to one event per buffer), rapidity window and shift,
the mixing seed; and 8 cases on the OSCAR reader with mixed species, a
random analysed species and, in some, a real mixed-event file
(random_oscar_case).  On the CPU the same cases run through the reference
binary and the oracle with byte-identical output files
(tests/test_reference_live_cpu.py); here lib/hbt_afterburner.e (reader,
HBT_correlation, the batched GPU kernels, writer) runs each case and every
file it writes is compared with the oracle's: same file set, denominator
column identical, mean q and numerators to the last printed digits
(test_dropin_gpu.compare_files), and the logged pair totals equal.

The reference path: src/HBT_correlation.cpp:177-218 (buffer driver),
:291-461 and :563-689 (pair loops), :694-855 (writers).
"""
import os
import shutil
import subprocess
import sys

import pytest

import oracle_lib

sys.path.insert(0, os.path.join(oracle_lib.REPO, "tests", "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu

EXE = os.path.join(oracle_lib.REPO, "hadronic_afterburner_toolkit_gb300", "lib",
                   "hbt_afterburner.e")


def _logged_totals(stdout):
    same = mixed = 0
    for line in stdout.splitlines():
        if "number of pairs:" in line:
            same += int(line.rsplit(":", 1)[1])
        elif "number of mixed pairs:" in line:
            mixed += int(line.rsplit(":", 1)[1])
    return same, mixed


@pytest.mark.parametrize("kind,k", [("mode10", k) for k in range(24)] +
                         [("oscar", k) for k in range(8)])
def test_dropin_matches_oracle_on_random_parameter_sets(kind, k, tmp_path):
    from test_dropin_gpu import compare_files
    name = "sweep_%s_%02d" % (kind, k)
    case = make_golden.random_case(k) if kind == "mode10" else make_golden.random_oscar_case(k)
    case_dir = make_golden.write_case(name, case, str(tmp_path))
    work = os.path.join(str(tmp_path), "work")
    res = os.path.join(work, "results")
    os.makedirs(res)
    shutil.copy(os.path.join(case_dir, "parameters.dat"), work)
    for fn in make_golden.input_files(case_dir):
        shutil.copy(os.path.join(case_dir, fn), res)
    proc = subprocess.run([EXE], cwd=work, capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-2000:]

    want_dir = os.path.join(str(tmp_path), "oracle_out")
    os.makedirs(want_dir)
    orc = oracle_lib.run_golden_case_through_oracle(name, want_dir, root=str(tmp_path))
    want = sorted(f for f in os.listdir(want_dir) if f.startswith("HBT_correlation"))
    got = sorted(f for f in os.listdir(res) if f.startswith("HBT_correlation"))
    assert got == want and want
    for f in want:
        compare_files(open(os.path.join(res, f)).read(),
                      open(os.path.join(want_dir, f)).read(), f)
    h = orc.hist()
    assert _logged_totals(proc.stdout) == (h["pairs_same"], h["pairs_mixed"])
