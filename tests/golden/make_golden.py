"""Regenerate the golden HBT fixtures from the compiled reference.

Run in a container that has the reference sources (the recipe in
``oracle/Makefile`` builds ``oracle/_ref/hadronic_afterburner_tools.e`` from
them):

    make -C oracle ref
    python tests/golden/make_golden.py [REFERENCE_ROOT]

For every case below it writes a seeded synthetic input, a full
``parameters.dat`` and runs the unmodified reference binary in a scratch
directory.  Committed per case under ``tests/golden/<case>/``:

* ``parameters.dat``        the exact parameter file the reference read;
* ``particle_samples.gz`` or ``OSCAR.DAT`` (+ mixed-event file) - the input;
* ``outputs.tar.gz``        every ``HBT_correlation_function_*.dat`` written;
* ``pairs.txt``             the reference's logged candidate-pair counts
                            ("number of pairs" / "number of mixed pairs").

The fixtures pin the oracle restatement (byte-identical output files) and the
drop-in's host logic; the GPU path is then checked against the oracle.
"""
from __future__ import annotations

import io
import os
import re
import shutil
import subprocess
import sys
import tarfile
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from hadronic_afterburner_toolkit_gb300 import synth  # noqa: E402

REF_BIN = os.path.join(REPO, "oracle", "_ref", "hadronic_afterburner_tools.e")

BASE_PARAMS = {
    "echo_level": 9,
    "read_in_mode": 10,
    "ecoOutput": 0,
    "analyze_flow": 0,
    "analyze_HBT": 1,
    "analyze_balance_function": 0,
    "analyze_ebe_yield": 0,
    "randomSeed": 1,
    "read_in_real_mixed_events": 0,
    "particle_monval": 211,
    "distinguish_isospin": 1,
    "resonance_weak_feed_down_flag": 0,
    "resonance_feed_down_flag": 0,
    "select_resonances_flag": 0,
    "net_particle_flag": 0,
    "flag_charge_dependence": 0,
    "event_buffer_size": 120,
    "rapidity_shift": 0.0,
    "readRapidityShiftFromFile": 0,
    "long_comoving_boost": 1,
    "needed_number_of_pairs": 30000000,
    "invariant_radius_flag": 0,
    "azimuthal_flag": 0,
    "n_KT": 5,
    "KT_min": 0.0,
    "KT_max": 1.0,
    "n_Kphi": 4,
    "HBTrap_min": -1.0,
    "HBTrap_max": 1.0,
    "qnpts": 9,
    "q_min": -0.15,
    "q_max": 0.15,
}


def _events_basic(seed=11, n_events=24, mu=40.0):
    return synth.generate(n_events, mu, seed=seed, sigma_xy=2.0, tau_mean=3.0)


def _events_mixed_species(seed):
    """pi+, pi- and K+ in every event: the species filter must pick pi+."""
    a = synth.generate(10, 35.0, seed=seed, sigma_xy=2.0, tau_mean=3.0)
    b = synth.generate(10, 20.0, seed=seed + 1, monval=-211, sigma_xy=2.0, tau_mean=3.0)
    c = synth.generate(10, 10.0, seed=seed + 2, mass=synth.KAON_MASS, monval=321,
                       sigma_xy=2.0, tau_mean=3.0)
    parts = []
    for e in range(10):
        sub = [synth.subset(x, e, e + 1) for x in (a, b, c)]
        ev = synth.Events.concat(sub)
        order = np.random.default_rng(seed + 100 + e).permutation(ev.n_particles)
        fields = ("monval", "mass", "t", "x", "y", "z", "E", "px", "py", "pz")
        parts.append(synth.Events(np.array([0, ev.n_particles], dtype=np.int64),
                                  *[getattr(ev, f)[order] for f in fields]))
    return synth.Events.concat(parts)


def _events_ragged(seed=5):
    """Ragged multiplicities, including empty and one-particle events."""
    mult = np.array([30, 0, 1, 25, 2, 0, 40, 1, 33, 17, 0, 28], dtype=np.int64)
    return synth.generate(mult.size, mult, seed=seed, sigma_xy=2.0, tau_mean=3.0)


CASES = {
    # plain 3-D, cap not binding
    "basic": dict(events=lambda: _events_basic(), params={}),
    # 1-D q_inv histograms as well
    "qinv": dict(events=lambda: _events_basic(seed=12),
                 params={"invariant_radius_flag": 1, "q_min": 0.0, "q_max": 0.2,
                         "qnpts": 11}),
    # K_phi-differential bins (psi_ref from the buffer's v2 plane)
    "kphi": dict(events=lambda: _events_basic(seed=13),
                 params={"azimuthal_flag": 1, "n_Kphi": 4, "qnpts": 7,
                         "invariant_radius_flag": 1}),
    # order-dependent caps bind (3-D cap 40, q_inv cap 50*40)
    "cap": dict(events=lambda: _events_basic(seed=14, n_events=30, mu=60.0),
                params={"needed_number_of_pairs": 40, "invariant_radius_flag": 1,
                        "event_buffer_size": 200}),
    "cap_kphi": dict(events=lambda: _events_basic(seed=15, n_events=30, mu=60.0),
                     params={"needed_number_of_pairs": 25, "azimuthal_flag": 1,
                             "n_Kphi": 3, "qnpts": 7, "event_buffer_size": 200}),
    # K_T and rapidity cuts active, no longitudinal boost, asymmetric q grid,
    # rapidity shift, compact output
    "cuts": dict(events=lambda: _events_basic(seed=16),
                 params={"KT_min": 0.15, "KT_max": 0.55, "HBTrap_min": -0.5,
                         "HBTrap_max": 0.5, "long_comoving_boost": 0,
                         "q_min": -0.1, "q_max": 0.2, "qnpts": 7,
                         "rapidity_shift": 0.3, "ecoOutput": 1, "n_KT": 4}),
    # OSCAR input with a species mix and a separate real mixed-event file
    "oscar_mixed": dict(events=lambda: _events_mixed_species(21),
                        mixed=lambda: _events_mixed_species(31),
                        params={"read_in_mode": 0, "read_in_real_mixed_events": 1,
                                "event_buffer_size": 100}),
    # one event per buffer (the mixed partner is the event itself), empty
    # and one-particle events
    "ragged": dict(events=lambda: _events_ragged(),
                   params={"event_buffer_size": 1, "invariant_radius_flag": 1}),
}


def param_text(p: dict) -> str:
    lines = ["# golden-fixture parameters (HBT drop-in)"]
    for k, v in p.items():
        lines.append("%s = %s" % (k, repr(v) if isinstance(v, float) else v))
    return "\n".join(lines) + "\n"


def random_case(k: int) -> dict:
    """Case k of a seeded sweep of parameter sets and inputs: grid size (odd
    and even), symmetric or asymmetric window (one without q = 0), K_T edges
    and range, boost, K_phi bins, q_inv histograms, a cap that binds or not,
    buffer size (down to one event), rapidity window and shift, the mixing
    seed."""
    rng = np.random.default_rng(4000 + k)
    q_max = round(float(rng.uniform(0.06, 0.3)), 4)
    q_min = -q_max if rng.random() < 0.6 else round(float(rng.uniform(-q_max, 0.02)), 4)
    kt_min = round(float(rng.choice([0.0, rng.uniform(0.0, 0.3)])), 4)
    params = {
        "qnpts": int(rng.choice([4, 5, 7, 8, 11, 15])),
        "q_min": q_min, "q_max": q_max,
        "n_KT": int(rng.integers(2, 7)),
        "KT_min": kt_min, "KT_max": round(kt_min + float(rng.uniform(0.3, 1.2)), 4),
        "long_comoving_boost": int(rng.integers(0, 2)),
        "azimuthal_flag": int(rng.integers(0, 2)),
        "n_Kphi": int(rng.integers(2, 7)),
        "invariant_radius_flag": int(rng.integers(0, 2)),
        "needed_number_of_pairs": int(rng.choice([20, 300, 30000000])),
        "event_buffer_size": int(rng.choice([1, 50, 120, 400])),
        "HBTrap_min": round(-float(rng.uniform(0.4, 1.2)), 4),
        "HBTrap_max": round(float(rng.uniform(0.4, 1.2)), 4),
        "rapidity_shift": round(float(rng.choice([0.0, rng.uniform(-0.3, 0.3)])), 4),
        "randomSeed": int(rng.integers(1, 10000)),
    }
    n_events = int(rng.integers(8, 30))
    mu = float(rng.uniform(15.0, 70.0))
    return dict(events=lambda: _events_basic(seed=5000 + k, n_events=n_events, mu=mu),
                params=params)


def random_oscar_case(k: int) -> dict:
    """Case k of a seeded sweep over the OSCAR reader (read_in_mode 0):
    events holding pi+, pi- and K+ in shuffled order, the analysed species
    drawn among them, a separate real mixed-event file or not, and the
    parameters of random_case."""
    rng = np.random.default_rng(6000 + k)
    case = random_case(1000 + k)
    params = dict(case["params"])
    params["read_in_mode"] = 0
    params["particle_monval"] = int(rng.choice([211, -211, 321]))
    real_mixed = bool(rng.integers(0, 2))
    params["read_in_real_mixed_events"] = int(real_mixed)
    params["event_buffer_size"] = int(rng.choice([1, 40, 100, 300]))
    out = dict(events=lambda: _events_mixed_species(7000 + k), params=params)
    if real_mixed:
        out["mixed"] = lambda: _events_mixed_species(8000 + k)
    return out


def write_case(name: str, case: dict, out_root: str = HERE) -> str:
    """Writes one case's parameters.dat and input files into out_root/name
    (no run); returns that folder."""
    out_dir = os.path.join(out_root, name)
    os.makedirs(out_dir, exist_ok=True)
    params = dict(BASE_PARAMS)
    params.update(case["params"])
    ev = case["events"]()
    mixed = case["mixed"]() if "mixed" in case else None
    if params["read_in_mode"] == 10:
        inputs = {"particle_samples.gz": ev}
        if mixed is not None:
            inputs["particle_samples_mixed_event.gz"] = mixed
        for fn, e in inputs.items():
            synth.write_mode10(os.path.join(out_dir, fn), e)
    else:
        inputs = {"OSCAR.DAT": ev}
        if mixed is not None:
            inputs["OSCAR_mixed_event.DAT"] = mixed
        for fn, e in inputs.items():
            synth.write_oscar(os.path.join(out_dir, fn), e)
    with open(os.path.join(out_dir, "parameters.dat"), "w") as f:
        f.write(param_text(params))
    return out_dir


def input_files(case_dir: str) -> list:
    """The input files of a case folder (what goes into results/)."""
    return sorted(fn for fn in os.listdir(case_dir)
                  if (fn.endswith(".gz") and fn != "outputs.tar.gz") or fn.endswith(".DAT"))


def run_case(name: str, case: dict, ref_root: str, out_root: str = HERE) -> None:
    """Runs the reference binary on one case and writes the case's files
    into out_root/name (tests/golden/<name> for the committed fixtures)."""
    out_dir = write_case(name, case, out_root)
    inputs = input_files(out_dir)

    with tempfile.TemporaryDirectory() as tmp:
        res = os.path.join(tmp, "results")
        os.makedirs(res)
        os.symlink(os.path.join(ref_root, "EOS"), os.path.join(tmp, "EOS"))
        for fn in inputs:
            shutil.copy(os.path.join(out_dir, fn), res)
        shutil.copy(os.path.join(out_dir, "parameters.dat"), tmp)
        proc = subprocess.run([REF_BIN], cwd=tmp, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("reference failed on %s:\n%s" % (name, proc.stdout[-2000:]))
        pairs = [ln.split("number of ")[-1] for ln in proc.stdout.splitlines()
                 if "number of pairs" in ln or "number of mixed pairs" in ln]
        pairs = [re.sub(r"\x1b\[[0-9;]*m", "", p).strip() for p in pairs]
        with open(os.path.join(out_dir, "pairs.txt"), "w") as f:
            f.write("\n".join(pairs) + "\n")
        outs = sorted(fn for fn in os.listdir(res) if fn.startswith("HBT_correlation"))
        with tarfile.open(os.path.join(out_dir, "outputs.tar.gz"), "w:gz") as tar:
            for fn in outs:
                data = open(os.path.join(res, fn), "rb").read()
                info = tarfile.TarInfo(fn)
                info.size = len(data)
                info.mtime = 0
                tar.addfile(info, io.BytesIO(data))
        print("%-12s %3d output files, %d pair-count lines" % (name, len(outs), len(pairs)))


def main(argv):
    ref_root = argv[1] if len(argv) > 1 else os.environ.get("HBT_REFERENCE_ROOT")
    if not ref_root:
        raise SystemExit("usage: %s <reference checkout> (or set HBT_REFERENCE_ROOT)" % argv[0])
    if not os.path.exists(REF_BIN):
        raise SystemExit("build the reference first: make -C oracle ref")
    for name, case in CASES.items():
        run_case(name, case, ref_root)


if __name__ == "__main__":
    main(sys.argv)
