"""Event averaging of the HBT files (hbt_host_average_events, hbt_average.e)
against the reference's ebe_scripts/average_event_HBT_correlation_function.py
run on the same folders (tests/golden_average/case.tar.gz, made by
make_golden_average.py).  The script sums the folders in directory order;
on another filesystem that order may differ, so values are compared to
1e-14 relative (a few ulps of the 10-digit print), NaN where NaN."""
import ctypes
import os
import subprocess
import tarfile

import numpy as np
import pytest

from hadronic_afterburner_toolkit_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = tmp_path_factory.mktemp("avg")
    with tarfile.open(os.path.join(HERE, "golden_average", "case.tar.gz")) as tar:
        tar.extractall(d, filter="data")
    return str(d)


def _table(path):
    return np.array([[float(t) for t in l.split()] for l in open(path) if l.strip()])


def _check(got_dir, want_dir):
    want = sorted(os.listdir(want_dir))
    assert sorted(os.listdir(got_dir)) == want and len(want) == 4
    for f in want:
        g, w = _table(os.path.join(got_dir, f)), _table(os.path.join(want_dir, f))
        assert g.shape == w.shape, f
        assert np.allclose(g, w, rtol=1e-14, atol=0.0, equal_nan=True), f
        # the reference's layout: "%.10e" fields joined by two blanks
        first = open(os.path.join(got_dir, f)).readline().rstrip("\n").split("  ")
        assert all(len(t.split("e")[0].split(".")[-1]) == 10 for t in first if t != "nan"), f


def test_library_average_matches_reference_script(case, tmp_path):
    build.build_gpu()
    L = ctypes.CDLL(build.build_host())
    L.hbt_host_average_events.restype = ctypes.c_int
    L.hbt_host_average_events.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32]
    for threads in (1, 3, 0):
        out = tmp_path / ("avg%d" % threads)
        n = L.hbt_host_average_events(os.path.join(case, "work").encode(), str(out).encode(),
                                      threads)
        assert n == 4
        _check(str(out), os.path.join(case, "avg"))


def test_cli_matches_reference_script(case, tmp_path):
    build.build_host()
    exe = os.path.join(os.path.dirname(build.build_host()), "hbt_average.e")
    proc = subprocess.run([exe, os.path.join(case, "work"), str(tmp_path / "o")],
                          capture_output=True, text=True, timeout=120)
    assert proc.returncode == 0, proc.stderr
    assert "Analysis is done." in proc.stdout
    _check(str(tmp_path / "o"), os.path.join(case, "avg"))


def test_ragged_or_missing_inputs_fail(case, tmp_path):
    import shutil
    L = ctypes.CDLL(build.build_host())
    L.hbt_host_average_events.restype = ctypes.c_int
    L.hbt_host_average_events.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32]
    work = tmp_path / "work"
    shutil.copytree(os.path.join(case, "work"), work)
    victim = work / "UrQMDev_3" / "UrQMD_results" / "HBT_correlation_function_KT_0_0.2.dat"
    lines = open(victim).read().split("\n")
    lines[7] = " ".join(lines[7].split()[:-1])
    open(victim, "w").write("\n".join(lines))
    assert L.hbt_host_average_events(str(work).encode(), str(tmp_path / "o").encode(), 0) == -1
    assert L.hbt_host_average_events(str(tmp_path / "none").encode(),
                                     str(tmp_path / "o2").encode(), 0) == -1


@pytest.mark.slow
@pytest.mark.parametrize("seed,n_ev,q", [(7, 3, 4), (8, 9, 7), (9, 2, 9), (10, 12, 5)])
def test_average_matches_reference_script_live(seed, n_ev, q, tmp_path):
    """Where the reference checkout is on this machine: random working
    folders (event count, grid size, pair counts, empty bins and, from three
    events on, a NaN q_inv row drawn from a seed) through the reference's
    averaging script and through the library call and the CLI."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden_average"))
    import make_golden_average
    import oracle_lib
    ref = oracle_lib.reference_checkout()
    if not ref or not os.path.exists(os.path.join(
            ref, "ebe_scripts", "average_event_HBT_correlation_function.py")):
        pytest.skip("no reference checkout")
    work, want = str(tmp_path / "work"), str(tmp_path / "want")
    make_golden_average.write_work(work, seed=seed, n_ev=n_ev, q=q)
    make_golden_average.run_script(ref, work, want)
    L = ctypes.CDLL(build.build_host())
    L.hbt_host_average_events.restype = ctypes.c_int
    L.hbt_host_average_events.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32]
    assert L.hbt_host_average_events(work.encode(), str(tmp_path / "lib").encode(), 0) == 4
    _check(str(tmp_path / "lib"), want)
    exe = os.path.join(os.path.dirname(build.build_host()), "hbt_average.e")
    proc = subprocess.run([exe, work, str(tmp_path / "cli")], capture_output=True, text=True,
                          timeout=120)
    assert proc.returncode == 0, proc.stderr
    _check(str(tmp_path / "cli"), want)


@pytest.mark.slow
def test_committed_average_fixture_is_the_reference_output(case, tmp_path):
    """Where the reference checkout is on this machine: the fixture's inputs
    come from make_golden_average.write_work (byte for byte) and the
    reference script still writes its averages for them."""
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden_average"))
    import make_golden_average
    import oracle_lib
    ref = oracle_lib.reference_checkout()
    if not ref or not os.path.exists(os.path.join(
            ref, "ebe_scripts", "average_event_HBT_correlation_function.py")):
        pytest.skip("no reference checkout")
    work, want = str(tmp_path / "work"), str(tmp_path / "want")
    make_golden_average.write_work(work)
    for root, _, files in os.walk(os.path.join(case, "work")):
        for f in files:
            rel = os.path.relpath(os.path.join(root, f), os.path.join(case, "work"))
            assert (open(os.path.join(work, rel), "rb").read()
                    == open(os.path.join(root, f), "rb").read()), rel
    make_golden_average.run_script(ref, work, want)
    _check(want, os.path.join(case, "avg"))
