"""Generates the event-averaging fixture: a working folder of UrQMD* event
folders holding HBT correlation files in the writer's format, and the
averages the reference's ebe_scripts/average_event_HBT_correlation_function.py
writes for them (run from the reference checkout given as argv[1]).

    python tests/golden_average/make_golden_average.py <reference checkout>

Writes tests/golden_average/case.tar.gz with work/ (inputs) and avg/
(the reference script's outputs).
"""
import os
import shutil
import subprocess
import sys
import tarfile
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def row5(v):
    return "%18.8e    %.8e    %.8e    %.8e    %.8e" % tuple(v)


def write_work(work, seed=2024, n_ev=5, q=5):
    """A working folder of n_ev UrQMD* event folders, each holding two 3-D
    files, one compact (eco) file and one q_inv file on a q^3 (q) grid;
    bins below 40 pairs carry a zero numerator, one q_inv row a NaN."""
    rng = np.random.default_rng(seed)
    grid = np.linspace(-0.1, 0.1, q)
    for ev in range(n_ev):
        res = os.path.join(work, "UrQMDev_%d" % ev, "UrQMD_results")
        os.makedirs(res)
        # two 3-D files (5 columns), one compact file (2 columns), one q_inv file
        for kt in ("0_0.2", "0.2_0.4"):
            lines = []
            for il in range(q):
                for io in range(q):
                    for is_ in range(q):
                        den = float(rng.integers(0, 400))
                        if den < 40:
                            v = (grid[io], grid[is_], grid[il], 0.0, den)
                        else:
                            v = (grid[io] + rng.normal(0, 0.005), grid[is_] + rng.normal(0, 0.005),
                                 grid[il] + rng.normal(0, 0.005), den * rng.uniform(0.9, 1.3),
                                 den * rng.uniform(0.9, 1.1))
                        lines.append(row5(v))
            with open(os.path.join(res, "HBT_correlation_function_KT_%s.dat" % kt), "w") as f:
                f.write("\n".join(lines) + "\n")
        with open(os.path.join(res, "HBT_correlation_function_KT_0.4_0.6_eco.dat"), "w") as f:
            for k in range(q ** 3):
                f.write("%18.8e    %.8e\n" % (rng.normal(10, 3), rng.integers(0, 100)))
        with open(os.path.join(res, "HBT_correlation_function_inv_KT_0_0.2.dat"), "w") as f:
            for k in range(q):
                qm = "-nan" if (ev == 2 and k == 0) else "%.8e" % rng.uniform(0, 0.1)
                f.write("%18s    %.8e    %.8e\n" % (qm, rng.normal(50, 5), rng.normal(45, 5)))


def run_script(ref, work, avg):
    """The reference's averaging script on `work`, writing into `avg`."""
    script = os.path.join(ref, "ebe_scripts", "average_event_HBT_correlation_function.py")
    subprocess.run([sys.executable, script, work, avg], check=True, capture_output=True)


def main(ref):
    tmp = tempfile.mkdtemp()
    work = os.path.join(tmp, "work")
    write_work(work)
    avg = os.path.join(tmp, "avg")
    run_script(ref, work, avg)
    out = os.path.join(HERE, "case.tar.gz")
    with tarfile.open(out, "w:gz") as tar:
        tar.add(work, arcname="work")
        tar.add(avg, arcname="avg")
    shutil.rmtree(tmp)
    print("wrote", out)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HBT_REFERENCE_ROOT")
    if not ref:
        raise SystemExit("usage: %s <reference checkout> (or set HBT_REFERENCE_ROOT)" % sys.argv[0])
    main(ref)
