"""The drop-in host side against the known answers of the reference's own
unit tests, on the reference's own fixture files (read where the reference
source tree is; skipped where it is absent, e.g. on a machine that only has
this repository).

* unit_tests/particleSamples_unittest.cc:60-100: the OSCAR reader
  (read_in_mode 0) keeps 31 and 27 pi+ in the two events of
  test_reader_files/OSCAR.DAT, same-event list and mixed-event pool.
* unit_tests/HBT_unittest.cc:23-47: psi_ref of
  calculate_flow_event_plane_angle(1, 2, 3) over the pi+ of
  test_gzip_reader/particle_list.dat is -1.6751628499713109,
  -0.85236384292521539 and 0.06674083818478263 (to 1e-8). That file is in
  the zipped UrQMD format (read_in_mode 2), whose reader is not part of the
  drop-in: the test parses it (pi+ = UrQMD ityp 101 with 2 I_3 = 2) and
  feeds px, py to the drop-in's event-plane sums (hbt_host_event_plane_angle,
  the code HBT_correlation::calculate_flow_event_plane_angle runs).
"""
import ctypes
import gzip
import os

import numpy as np
import pytest

import oracle_lib
from hadronic_afterburner_toolkit_gb300 import build

# the reference checkout whose unit-test fixtures are read in place
REF = oracle_lib.reference_checkout()
UNIT = os.path.join(REF, "unit_tests") if REF else ""
pytestmark = pytest.mark.skipif(not UNIT or not os.path.isdir(UNIT),
                                reason="no reference checkout (HBT_REFERENCE_ROOT)")


@pytest.fixture(scope="module")
def host():
    build.build_gpu()
    L = ctypes.CDLL(build.build_host())
    L.hbt_host_scan_buffers.restype = ctypes.c_int
    L.hbt_host_scan_buffers.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int64),
                                        ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int64)]
    L.hbt_host_event_plane_angle.restype = ctypes.c_double
    L.hbt_host_event_plane_angle.argtypes = [ctypes.c_int64, ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(ctypes.c_double), ctypes.c_int32]
    return L


def test_oscar_reader_counts(host, tmp_path):
    """One event per buffer (event_buffer_size = 1: whole events are read
    until the count reaches it), so the buffers' counts are the events'.
    The fixture's parameters.dat predates the read_in_real_mixed_events key,
    which today's reader requires (the reference exits without it); the
    mixed-event pool is read from OSCAR_mixed_event.DAT (a link to the same
    file), as the reference's mixed-event test reads it."""
    text = open(os.path.join(UNIT, "parameters.dat")).read()
    pfile = tmp_path / "parameters.dat"
    pfile.write_text(text + "\nread_in_mode = 0\nparticle_monval = 211\n"
                            "event_buffer_size = 1\nrun_mode = 1\n"
                            "read_in_real_mixed_events = 1\n")
    cap = 8
    nev = (ctypes.c_int32 * cap)()
    npart = (ctypes.c_int64 * cap)()
    mnev = (ctypes.c_int32 * cap)()
    mpart = (ctypes.c_int64 * cap)()
    nb = host.hbt_host_scan_buffers(str(pfile).encode(),
                                    os.path.join(UNIT, "test_reader_files").encode(),
                                    cap, nev, npart, mnev, mpart)
    # the read that meets the end of the file gives a last, empty buffer, as
    # the reference's buffer loop does
    assert nb == 3 and nev[2] == 0 and npart[2] == 0
    assert list(nev[:2]) == [1, 1] and list(mnev[:2]) == [1, 1]
    assert list(npart[:2]) == [31, 27]
    assert list(mpart[:2]) == [31, 27]


def _urqmd_pi_plus(path):
    """px, py of the pi+ of a zipped UrQMD particle list, in file order:
    per event a count line, one skipped line, then one line per particle
    (ityp, 2 I_3, charge, two fields, parent process, mass, t, x, y, z, E,
    px, py, pz; src/particleSamples.cpp:910-964)."""
    px, py = [], []
    with gzip.open(path, "rt") as f:
        lines = f.read().split("\n")
    i = 0
    while i < len(lines) and lines[i].strip():
        n = int(lines[i].split()[0])
        for line in lines[i + 2:i + 2 + n]:
            v = line.split()
            if int(v[0]) == 101 and int(v[1]) == 2:
                px.append(float(v[12]))
                py.append(float(v[13]))
        i += 2 + n
    return np.array(px), np.array(py)


def test_psi_ref_known_answers(host):
    px, py = _urqmd_pi_plus(os.path.join(UNIT, "test_gzip_reader", "particle_list.dat"))
    assert px.size > 0
    pd = ctypes.POINTER(ctypes.c_double)
    want = {1: -1.6751628499713109, 2: -0.85236384292521539, 3: 0.06674083818478263}
    for n, psi in want.items():
        got = host.hbt_host_event_plane_angle(px.size, px.ctypes.data_as(pd),
                                              py.ctypes.data_as(pd), n)
        assert abs(got - psi) < 1e-8, (n, got, psi)

