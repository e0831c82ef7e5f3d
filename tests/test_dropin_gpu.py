"""End-to-end drop-in runs on the GPU against the reference's own outputs.

The C++ drop-in executable (lib/hbt_afterburner.e: ParameterReader,
particleSamples, HBT_correlation on libhbt_gpu.so) is run on every golden
case's parameters.dat and input file, exactly as the reference binary was,
and each HBT_correlation_function_*.dat it writes is compared with the file
the reference wrote:
  - same file set, same line count, same grid columns where a bin has fewer
    than 2 pairs;
  - the denominator column (normalised pair counts) identical;
  - mean q and the cos(q.dx) numerator within 2e-8 relative (the last printed
    digit of "%.8e" may flip because the GPU sums in a different order) or
    1e-9 absolute (numerators that cancel to ~0).
"""
import os
import shutil
import subprocess
import tarfile

import numpy as np
import pytest

import oracle_lib

pytestmark = pytest.mark.gpu

EXE = os.path.join(oracle_lib.REPO, "hadronic_afterburner_toolkit_gb300", "lib",
                   "hbt_afterburner.e")
CASES = sorted(d for d in os.listdir(oracle_lib.GOLDEN)
               if os.path.exists(os.path.join(oracle_lib.GOLDEN, d, "parameters.dat")))


def _parse(text):
    rows = []
    for line in text.strip().split("\n"):
        rows.append([float("nan") if "nan" in tok else float(tok) for tok in line.split()])
    return np.array(rows)


def _golden(name):
    out = {}
    with tarfile.open(os.path.join(oracle_lib.GOLDEN, name, "outputs.tar.gz")) as tar:
        for m in tar.getmembers():
            out[m.name] = tar.extractfile(m).read().decode()
    return out


def run_dropin(name, workdir, extra_args=()):
    src = os.path.join(oracle_lib.GOLDEN, name)
    res = os.path.join(workdir, "results")
    os.makedirs(res)
    for fn in os.listdir(src):
        if fn in ("parameters.dat",):
            shutil.copy(os.path.join(src, fn), workdir)
        elif fn.endswith(".gz") and fn != "outputs.tar.gz" or fn.endswith(".DAT"):
            shutil.copy(os.path.join(src, fn), res)
    proc = subprocess.run([EXE] + list(extra_args), cwd=workdir, capture_output=True, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stdout[-2000:] + proc.stderr[-2000:]
    return res, proc.stdout


def compare_files(got_text, want_text, fname):
    g, w = _parse(got_text), _parse(want_text)
    assert g.shape == w.shape, fname
    # denominator column: exact
    assert np.array_equal(g[:, -1], w[:, -1], equal_nan=True), fname
    num_g, num_w = g[:, -2], w[:, -2]
    ok = np.isclose(num_g, num_w, rtol=2e-8, atol=1e-9, equal_nan=True)
    assert ok.all(), "%s: numerator rows %s" % (fname, np.nonzero(~ok)[0][:5])
    if g.shape[1] > 2:
        for col in range(g.shape[1] - 2):
            ok = np.isclose(g[:, col], w[:, col], rtol=2e-8, atol=1e-12, equal_nan=True)
            assert ok.all(), "%s: column %d rows %s" % (fname, col, np.nonzero(~ok)[0][:5])


@pytest.mark.parametrize("name", CASES)
def test_dropin_matches_reference_outputs(name, tmp_path):
    res, log = run_dropin(name, str(tmp_path))
    want = _golden(name)
    got = {f: open(os.path.join(res, f)).read() for f in os.listdir(res)
           if f.startswith("HBT_correlation")}
    assert sorted(got) == sorted(want)
    same = 0
    for f in want:
        compare_files(got[f], want[f], f)
        same += got[f] == want[f]
    # most files come out byte-identical
    assert same >= len(want) // 2, "only %d of %d files byte-identical" % (same, len(want))


@pytest.mark.parametrize("name", ["basic", "kphi"])
def test_dropin_reference_chain_kernel(name, tmp_path):
    """hbt_kernel=1 (FP64 reference chain on every pair) gives the same files."""
    res, _ = run_dropin(name, str(tmp_path), ["hbt_kernel=1"])
    want = _golden(name)
    for f in want:
        compare_files(open(os.path.join(res, f)).read(), want[f], f)


@pytest.mark.parametrize("name", ["basic", "kphi"])
def test_dropin_double_float_precision(name, tmp_path):
    """hbt_precision=2 (same-event values in double-float arithmetic, at most
    1e-11 per pair from the FP64 sums) gives the same files within the
    printed precision."""
    res, _ = run_dropin(name, str(tmp_path), ["hbt_precision=2"])
    want = _golden(name)
    got = sorted(f for f in os.listdir(res) if f.startswith("HBT_correlation"))
    assert got == sorted(want)
    for f in want:
        compare_files(open(os.path.join(res, f)).read(), want[f], f)


def test_dropin_missing_key_is_a_parameter_error(tmp_path):
    name = "basic"
    src = os.path.join(oracle_lib.GOLDEN, name)
    res = os.path.join(str(tmp_path), "results")
    os.makedirs(res)
    shutil.copy(os.path.join(src, "particle_samples.gz"), res)
    lines = [l for l in open(os.path.join(src, "parameters.dat"))
             if not l.startswith("qnpts")]
    open(os.path.join(str(tmp_path), "parameters.dat"), "w").writelines(lines)
    proc = subprocess.run([EXE], cwd=str(tmp_path), capture_output=True, text=True, timeout=120)
    assert proc.returncode == 255
    assert "parameter with name qnpts not found" in proc.stdout
