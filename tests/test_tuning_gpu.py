"""Launch-shape tuning of the batched path (hbt_set_tuning,
hbt_autotune_batch) and its CUDA-graph launches: every tuning and every
graph re-launch gives the oracle's bins and counts exactly and sums within
tests/parity.py's tolerance; the autotuner leaves the histograms untouched."""
import numpy as np
import pytest

import oracle_lib
import parity
from test_batch_gpu import BASE, _qscale, _run_oracle, _uneven_jobs

pytestmark = pytest.mark.gpu


def _device_jobs(jobs):
    torch = pytest.importorskip("torch")
    out = []
    for j in jobs:
        if j[0] == "same":
            out.append(("same", [torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in j[1]]))
        else:
            out.append(("mixed", [torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in j[1]],
                        [torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in j[2]]))
    return out


@pytest.mark.parametrize("tuning", [
    dict(cell_pt=0.01, cell_y=0.025),
    dict(cell_pt=0.04, cell_y=0.1),
    dict(cell_pt=0.5, cell_y=2.0),
    dict(blocks_per_sm=1),
    dict(blocks_per_sm=3, use_graph=0),
])
def test_every_tuning_matches_oracle(tuning):
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE, azimuthal_flag=1)
    jobs = _uneven_jobs(seed=51, n_groups=3)
    eng = E.Engine(**p)
    eng.set_tuning(**tuning)
    eng.set_psi_ref(0.4)
    eng.bin_batch(jobs)
    parity.compare(eng.hist(), _run_oracle(p, jobs, psi=0.4), _qscale(p))


def test_graph_capture_and_relaunch():
    """The same batch three times: a direct launch, a capture, a re-launch of
    the cached graph; the histograms are three times the oracle's."""
    from hadronic_afterburner_toolkit_gb300 import engine as E
    jobs = _uneven_jobs(seed=61, n_groups=2)
    djobs = _device_jobs(jobs)
    eng = E.Engine(**BASE)
    eng.set_tuning(use_graph=1)
    for _ in range(3):
        eng.bin_batch(djobs, device=True)
    st = eng.stats()
    assert st["graph_captures"] == 1 and st["graph_replays"] == 1
    # the cull's statistics of the last batch
    assert 0 < st["tiles_same_kept"] <= st["tiles_same"]
    assert 0 < st["tiles_mixed_kept"] <= st["tiles_mixed"]
    orc = oracle_lib.Oracle(**BASE)
    for _ in range(3):
        for j in jobs:
            if j[0] == "same":
                orc.bin_same(j[1])
            else:
                orc.bin_mixed(j[1], j[2])
    parity.compare(eng.hist(), orc.hist(), _qscale(BASE))
    # a smaller batch of another shape runs directly (no buffer grows), and
    # the first shape then re-launches the cached graph
    eng.bin_batch(djobs[:3], device=True)
    eng.bin_batch(djobs, device=True)
    st = eng.stats()
    assert st["graph_captures"] == 1 and st["graph_replays"] == 2


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_keeps_histograms_and_results(precision):
    from hadronic_afterburner_toolkit_gb300 import engine as E
    p = dict(BASE)
    jobs = _uneven_jobs(seed=71, n_groups=3)
    djobs = _device_jobs(jobs)
    eng = E.Engine(precision=precision, **p)
    best, ms = eng.autotune(djobs)
    assert ms > 0.0
    assert best["cell_pt"] > 0 and best["cell_y"] > 0
    assert eng.tuning() == best
    h0 = eng.hist()
    assert not h0["count"].any() and not h0["den"].any() and eng.stats()["pairs_same"] == 0
    eng.bin_batch(djobs, device=True)
    rtol = 1e-5 if precision else parity.RTOL
    parity.compare(eng.hist(), _run_oracle(p, jobs), _qscale(p), rtol=rtol)


def test_invalid_tuning_rejected():
    from hadronic_afterburner_toolkit_gb300 import engine as E
    eng = E.Engine(**BASE)
    for bad in (dict(merge_chunk=20000), dict(blocks_per_sm=-1), dict(use_graph=2),
                dict(cell_pt=-0.1)):
        with pytest.raises(E.HbtError, match="HBT_ERR_INVALID"):
            eng.set_tuning(**bad)
