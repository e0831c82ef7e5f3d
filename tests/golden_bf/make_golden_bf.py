"""Regenerate the balance-function fixtures from the compiled reference.

    make -C oracle ref
    python tests/golden_bf/make_golden_bf.py [REFERENCE_ROOT]

For every case: a seeded synthetic input with a mix of species, a full
parameters.dat (analyze_balance_function = 1), and the three files the
unmodified reference binary writes (Balance_function_*_Delta_y.dat,
*_Delta_phi.dat, Correlation_function_*_2D.dat) in outputs.tar.gz.
"""
from __future__ import annotations

import io
import os
import shutil
import subprocess
import sys
import tarfile
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
from hadronic_afterburner_toolkit_gb300 import synth  # noqa: E402
from make_golden import BASE_PARAMS, REF_BIN, param_text  # noqa: E402

BF_PARAMS = dict(BASE_PARAMS, analyze_HBT=0, analyze_balance_function=1,
                 particle_alpha=211, particle_beta=-211, BpT_min=0.2, BpT_max=2.0,
                 Bnpts=21, Brap_max=1.0, rap_type=1, event_buffer_size=150)


def species_mix(seed, n_events, mu=(30.0, 28.0, 8.0, 7.0)):
    """pi+, pi-, K+, K- in every event, shuffled."""
    kinds = [(211, synth.PION_MASS, 0.25), (-211, synth.PION_MASS, 0.25),
             (321, synth.KAON_MASS, 0.30), (-321, synth.KAON_MASS, 0.30)]
    gens = [synth.generate(n_events, m, seed=seed + k, mass=mass, monval=mon, T=T,
                           sigma_xy=2.0, tau_mean=3.0)
            for k, ((mon, mass, T), m) in enumerate(zip(kinds, mu))]
    parts = []
    for e in range(n_events):
        ev = synth.Events.concat([synth.subset(g, e, e + 1) for g in gens])
        order = np.random.default_rng(seed + 1000 + e).permutation(ev.n_particles)
        fields = ("monval", "mass", "t", "x", "y", "z", "E", "px", "py", "pz")
        parts.append(synth.Events(np.array([0, ev.n_particles], dtype=np.int64),
                                  *[getattr(ev, f)[order] for f in fields]))
    return synth.Events.concat(parts)


CASES = {
    "pions": dict(events=lambda: species_mix(41, 12), params={}),
    "kaon_pion_eta": dict(events=lambda: species_mix(51, 10),
                          params={"particle_alpha": 321, "particle_beta": -211, "rap_type": 0,
                                  "Bnpts": 11, "Brap_max": 1.5, "rapidity_shift": 0.2,
                                  "BpT_min": 0.0, "BpT_max": 3.0, "event_buffer_size": 100}),
    "oscar_real_mixed": dict(events=lambda: species_mix(61, 8), mixed=lambda: species_mix(71, 9),
                             params={"read_in_mode": 0, "read_in_real_mixed_events": 1,
                                     "Bnpts": 15, "Brap_max": 0.8, "event_buffer_size": 120}),
}


def random_case(k: int) -> dict:
    """Case k of a seeded sweep: the alpha / beta species among pi+-, K+-
    (alpha == beta included), rapidity or pseudorapidity, the Delta y grid
    (odd and even Bnpts) and range, the p_T window, a rapidity shift, the
    buffer size, mode-10 or OSCAR input with or without a real mixed-event
    file, the mixing seed."""
    rng = np.random.default_rng(9000 + k)
    species = [211, -211, 321, -321]
    params = {
        "particle_alpha": int(rng.choice(species)),
        "particle_beta": int(rng.choice(species)),
        "rap_type": int(rng.integers(0, 2)),
        "Bnpts": int(rng.choice([6, 9, 11, 20, 21, 41])),
        "Brap_max": round(float(rng.uniform(0.4, 2.0)), 4),
        "BpT_min": round(float(rng.choice([0.0, rng.uniform(0.0, 0.4)])), 4),
        "BpT_max": round(float(rng.uniform(1.0, 3.0)), 4),
        "rapidity_shift": round(float(rng.choice([0.0, rng.uniform(-0.3, 0.3)])), 4),
        "event_buffer_size": int(rng.choice([1, 80, 150, 400])),
        "read_in_mode": int(rng.choice([10, 0])),
        "randomSeed": int(rng.integers(1, 10000)),
    }
    real_mixed = bool(rng.integers(0, 2))
    params["read_in_real_mixed_events"] = int(real_mixed)
    n_events = int(rng.integers(5, 14))
    case = dict(events=lambda: species_mix(9500 + 10 * k, n_events), params=params)
    if real_mixed:
        case["mixed"] = lambda: species_mix(9700 + 10 * k, n_events + 1)
    return case


def run_case(name, case, ref_root, out_root=HERE):
    """Runs the reference binary on one case and writes the case's files
    into out_root/name (tests/golden_bf/<name> for the committed fixtures)."""
    out_dir = os.path.join(out_root, name)
    os.makedirs(out_dir, exist_ok=True)
    params = dict(BF_PARAMS)
    params.update(case["params"])
    ev = case["events"]()
    mixed = case["mixed"]() if "mixed" in case else None
    with tempfile.TemporaryDirectory() as tmp:
        res = os.path.join(tmp, "results")
        os.makedirs(res)
        os.symlink(os.path.join(ref_root, "EOS"), os.path.join(tmp, "EOS"))
        if params["read_in_mode"] == 10:
            inputs = {"particle_samples.gz": ev}
            if mixed is not None:
                inputs["particle_samples_mixed_event.gz"] = mixed
            for fn, e in inputs.items():
                synth.write_mode10(os.path.join(res, fn), e)
        else:
            inputs = {"OSCAR.DAT": ev}
            if mixed is not None:
                inputs["OSCAR_mixed_event.DAT"] = mixed
            for fn, e in inputs.items():
                synth.write_oscar(os.path.join(res, fn), e)
        with open(os.path.join(tmp, "parameters.dat"), "w") as f:
            f.write(param_text(params).replace("HBT drop-in", "balance function"))
        proc = subprocess.run([REF_BIN], cwd=tmp, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError("reference failed on %s:\n%s" % (name, proc.stdout[-2000:]))
        for fn in inputs:
            shutil.copy(os.path.join(res, fn), os.path.join(out_dir, fn))
        shutil.copy(os.path.join(tmp, "parameters.dat"), out_dir)
        outs = sorted(fn for fn in os.listdir(res)
                      if fn.startswith("Balance_function") or fn.startswith("Correlation_function"))
        with tarfile.open(os.path.join(out_dir, "outputs.tar.gz"), "w:gz") as tar:
            for fn in outs:
                data = open(os.path.join(res, fn), "rb").read()
                info = tarfile.TarInfo(fn)
                info.size = len(data)
                info.mtime = 0
                tar.addfile(info, io.BytesIO(data))
        print("%-18s %d output files" % (name, len(outs)))


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
