"""Error paths of the engine and the drop-in, each made without faulting the
GPU: a wait that runs out of budget, the device's own error flag raised by a
full K_phi deferral buffer, an allocation failure injected on the host, and
a truncated input file.  After each, the context (or the next run) must work
and agree with the oracle.

The reference stops the process with exit() on its error paths
(src/particleSamples.cpp:164-195, src/ParameterReader.cpp:142-151); the
engine returns a status instead and keeps the context usable.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle_lib
import parity
from hadronic_afterburner_toolkit_gb300 import engine, synth

pytestmark = pytest.mark.gpu

BASIC = dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=4,
             azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
             needed_number_of_pairs=1e18)
HBT_ERR_NOMEM, HBT_ERR_TIMEOUT, HBT_ERR_DEVICE = 3, 4, 5


def _cols(ev):
    return [np.ascontiguousarray(getattr(ev, k)) for k in
            ("px", "py", "pz", "E", "x", "y", "z", "t")]


def test_sync_budget_runs_out_then_a_full_wait_succeeds():
    """hbt_sync with a 1 us budget on a launch of ~1e9 pairs returns
    HBT_ERR_TIMEOUT while the work runs; hbt_sync without a limit then
    returns HBT_OK and the result equals a second, waited-for binning."""
    ev = synth.generate(30, 1500.0, seed=81, sigma_xy=7.0, tau_mean=12.0)
    c = _cols(ev)
    eng = engine.Engine(**BASIC)
    L = eng.L
    eng.bin_same(c)
    rc = L.hbt_sync(eng.handle, 1)
    assert rc == HBT_ERR_TIMEOUT, engine.STATUS.get(rc)
    assert b"still running" in L.hbt_last_error(eng.handle)
    assert L.hbt_sync(eng.handle, 0) == 0
    a = eng.hist()
    eng.reset()
    eng.bin_same(c)
    eng.sync()
    b = eng.hist()
    assert a["count"].sum() > 1e6
    assert np.array_equal(a["count"], b["count"])


def test_full_deferral_buffer_raises_the_device_error_flag():
    """With the reference-chain kernel and a 1 rad K_phi edge zone every
    binned pair is handed to the host; more than the 65,536 records the
    buffer holds make the kernel raise its error flag (no write past the
    buffer): hbt_sync and the histogram read return HBT_ERR_DEVICE.  After
    hbt_reset the same context bins a smaller list exactly as the oracle."""
    p = dict(BASIC, qnpts=11, azimuthal_flag=1, kernel=engine.KERNEL_REFERENCE_CHAIN)
    ev = synth.generate(3, 1000.0, seed=82, sigma_xy=1.0, tau_mean=1.0)
    eng = engine.Engine(kphi_defer_tol=1.0, **p)
    eng.set_psi_ref(0.4)
    eng.bin_same(_cols(ev))
    rc = eng.L.hbt_sync(eng.handle, 0)
    assert rc == HBT_ERR_DEVICE, engine.STATUS.get(rc)
    with pytest.raises(engine.HbtError, match="HBT_ERR_DEVICE"):
        eng.hist()
    eng.reset()
    small = synth.generate(2, 150.0, seed=83, sigma_xy=2.0, tau_mean=3.0)
    eng.bin_same(_cols(small))
    h = eng.hist()
    orc = oracle_lib.Oracle(**{k: v for k, v in p.items() if k != "kernel"})
    orc.set_psi_ref(0.4)
    orc.bin_same(_cols(small))
    o = orc.hist()
    assert 0 < o["count"].sum() < 65536
    parity.compare(h, o, q_scale=0.15)
    assert eng.stats()["deferred_kphi"] == o["count"].sum()


def test_injected_allocation_failure_leaves_the_context_usable():
    """An allocation failure injected into the engine's device allocator:
    the staging of a list fails with HBT_ERR_NOMEM and bins nothing; the
    next call works.  A failure in the histogram read-back leaves the
    histograms intact for the next read."""
    ev = synth.generate(4, 400.0, seed=84, sigma_xy=3.0, tau_mean=4.0)
    c = _cols(ev)
    eng = engine.Engine(**BASIC)
    L = eng.L
    assert L.hbt_inject_alloc_failure(eng.handle, -2) == 1  # invalid
    assert L.hbt_inject_alloc_failure(eng.handle, 0) == 0
    with pytest.raises(engine.HbtError, match="HBT_ERR_NOMEM"):
        eng.bin_same(c)
    assert eng.stats()["pairs_same"] == 0
    eng.bin_same(c)  # the injection fired once and switched itself off
    orc = oracle_lib.Oracle(**BASIC)
    orc.bin_same(c)
    o = orc.hist()
    # the read-back buffer is this context's next allocation
    assert L.hbt_inject_alloc_failure(eng.handle, 0) == 0
    with pytest.raises(engine.HbtError, match="HBT_ERR_NOMEM"):
        eng.hist()
    parity.compare(eng.hist(), o, q_scale=0.15)


def test_drop_in_reports_a_truncated_sample_file(tmp_path):
    """The drop-in executable on a particle_samples.gz cut short exits with
    status 1 and names the problem; the intact file runs to the end."""
    exe = os.path.join(oracle_lib.REPO, "hadronic_afterburner_toolkit_gb300", "lib",
                       "hbt_afterburner.e")
    src = os.path.join(oracle_lib.GOLDEN, "basic")
    data = open(os.path.join(src, "particle_samples.gz"), "rb").read()
    for cut, want_rc in ((len(data), 0), (len(data) - 8, 1), (len(data) // 2, 1)):
        work = tmp_path / ("cut%d" % cut)
        (work / "results").mkdir(parents=True)
        shutil.copy(os.path.join(src, "parameters.dat"), str(work))
        (work / "results" / "particle_samples.gz").write_bytes(data[:cut])
        proc = subprocess.run([exe], cwd=str(work), capture_output=True, text=True, timeout=300)
        assert proc.returncode == want_rc, (cut, proc.stdout[-500:], proc.stderr[-500:])
        if want_rc:
            assert "gzip stream ends early" in proc.stderr
