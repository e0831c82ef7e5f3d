"""Host side of the drop-in on CPU (no GPU calls): the event reader and the
reference-format writer of libhbt_host.so, checked on the golden cases."""
import ctypes
import os
import tarfile

import numpy as np
import pytest

import oracle_lib
from hadronic_afterburner_toolkit_gb300 import build, engine, synth

CASES = sorted(d for d in os.listdir(oracle_lib.GOLDEN)
               if os.path.isdir(os.path.join(oracle_lib.GOLDEN, d)))
_PD = ctypes.POINTER(ctypes.c_double)
_PU = ctypes.POINTER(ctypes.c_uint64)


@pytest.fixture(scope="module")
def host():
    build.build_gpu()
    lib = build.build_host()
    L = ctypes.CDLL(lib)
    L.hbt_host_scan_buffers.restype = ctypes.c_int
    L.hbt_host_scan_buffers.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int64),
                                        ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int64)]
    L.hbt_host_write.restype = ctypes.c_int
    L.hbt_host_write.argtypes = [ctypes.POINTER(engine.HbtParams), ctypes.c_char_p,
                                 ctypes.c_int32] + [_PD] * 10 + [_PU] * 4
    return L


def _stage(name, tmp):
    src = os.path.join(oracle_lib.GOLDEN, name)
    res = os.path.join(tmp, "results")
    os.makedirs(res, exist_ok=True)
    for fn in os.listdir(src):
        if (fn.endswith(".gz") and fn != "outputs.tar.gz") or fn.endswith(".DAT"):
            os.symlink(os.path.join(src, fn), os.path.join(res, fn))
    return os.path.join(src, "parameters.dat"), res


@pytest.mark.parametrize("name", CASES)
def test_reader_buffers_match_reference_rule(host, name, tmp_path):
    pfile, res = _stage(name, str(tmp_path))
    cap = 256
    nev = (ctypes.c_int32 * cap)()
    npart = (ctypes.c_int64 * cap)()
    mnev = (ctypes.c_int32 * cap)()
    mpart = (ctypes.c_int64 * cap)()
    nb = host.hbt_host_scan_buffers(pfile.encode(), res.encode(), cap, nev, npart, mnev, mpart)
    assert nb > 0
    prm, ev, mixed = oracle_lib.golden_case(name)
    size = int(prm["event_buffer_size"])
    mon = int(prm["particle_monval"])
    want = oracle_lib.buffer_ranges(ev.multiplicities(), size)
    # the reader sees one trailing empty buffer when the last buffer ended
    # exactly at the end of the file without touching EOF
    assert nb in (len(want), len(want) + 1)
    for b, (s, e) in enumerate(want):
        buf = oracle_lib.filter_species(synth.subset(ev, s, e), mon)
        assert nev[b] == buf.n_events
        assert npart[b] == buf.n_particles
        if mixed is None:
            assert mnev[b] == buf.n_events and mpart[b] == buf.n_particles
    if mixed is not None:
        mwant = oracle_lib.buffer_ranges(mixed.multiplicities(), size)
        for b, (s, e) in enumerate(mwant[:len(want)]):
            mb = oracle_lib.filter_species(synth.subset(mixed, s, e), mon)
            assert mnev[b] == mb.n_events and mpart[b] == mb.n_particles


@pytest.mark.parametrize("name", CASES)
def test_writer_reproduces_reference_files(host, name, tmp_path):
    """Oracle histograms written by the drop-in writer == reference files."""
    orc = oracle_lib.run_golden_case_through_oracle(name, str(tmp_path))
    h = orc.hist()
    out = tmp_path / "w"
    out.mkdir()
    p = orc.p
    hp = engine.HbtParams(qnpts=p["qnpts"], q_min=p["q_min"], q_max=p["q_max"], n_KT=p["n_KT"],
                          KT_min=p["KT_min"], KT_max=p["KT_max"], n_Kphi=p["n_Kphi"],
                          azimuthal_flag=p["azimuthal_flag"],
                          invariant_radius_flag=p["invariant_radius_flag"])
    prm, _, _ = oracle_lib.golden_case(name)
    arrs = [np.ascontiguousarray(h[k]) for k in
            ("count", "q_out", "q_side", "q_long", "num", "den",
             "qinv_sum", "qinv_num", "qinv_count", "qinv_den")]
    ctr = [np.ascontiguousarray(h[k]) for k in
           ("ctr_num", "ctr_den", "ctr_num_qinv", "ctr_den_qinv")]
    rc = host.hbt_host_write(ctypes.byref(hp), str(out).encode(), int(prm.get("ecooutput", 0)),
                             *[a.ctypes.data_as(_PD) for a in arrs],
                             *[c.ctypes.data_as(_PU) for c in ctr])
    assert rc == 0
    with tarfile.open(os.path.join(oracle_lib.GOLDEN, name, "outputs.tar.gz")) as tar:
        want = {m.name: tar.extractfile(m).read() for m in tar.getmembers()}
    got = {f: open(os.path.join(out, f), "rb").read() for f in os.listdir(out)}
    assert sorted(got) == sorted(want)
    for f in want:
        assert got[f] == want[f], f
