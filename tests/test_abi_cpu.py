"""The C ABI library builds for sm_103a, loads without a GPU and exports
every entry point include/hbt_gpu.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

from hadronic_afterburner_toolkit_gb300 import build, engine

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
HEADER = os.path.join(INCLUDE, "hbt_gpu.h")
SERVER_HEADER = os.path.join(INCLUDE, "hbt_server.h")
BF_HEADER = os.path.join(INCLUDE, "hbt_bf.h")
FIT_HEADER = os.path.join(INCLUDE, "hbt_fit.h")
CHECK_HEADER = os.path.join(INCLUDE, "hbt_check.h")


def _declared_functions(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(hbt_[a-z_0-9]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    build.build_gpu()
    return ctypes.CDLL(engine.LIB_PATH)


def test_header_declares_the_engine_api():
    names = _declared_functions(HEADER)
    assert "hbt_create" in names and "hbt_bin_same" in names and "hbt_bin_mixed" in names
    # the Python mirror binds exactly what the header declares
    assert sorted(engine.exported_symbols()) == names


def test_library_exports_every_declared_symbol(lib):
    for name in (_declared_functions(HEADER) + _declared_functions(SERVER_HEADER) +
                 _declared_functions(BF_HEADER) + _declared_functions(FIT_HEADER) +
                 _declared_functions(CHECK_HEADER)):
        assert hasattr(lib, name), name


def test_bf_header_matches_its_binding(lib):
    from hadronic_afterburner_toolkit_gb300 import bf
    names = _declared_functions(BF_HEADER)
    assert "hbt_bf_bin" in names and "hbt_bf_read" in names
    assert sorted(bf.exported_symbols()) == names


def test_fit_header_matches_its_binding(lib):
    from hadronic_afterburner_toolkit_gb300 import radii
    names = _declared_functions(FIT_HEADER)
    assert "hbt_fit_radii" in names and "hbt_fit_create" in names
    assert sorted(radii.exported_symbols()) == names
    # the ctypes mirrors have the C structs' sizes
    assert ctypes.sizeof(radii.HbtFitResult) == 8 * 14 + 16
    assert ctypes.sizeof(radii.HbtFitTable) == 8 * 7


def test_fit_rejects_bad_options_without_a_device_call(lib):
    from hadronic_afterburner_toolkit_gb300 import radii
    L = radii.load()
    assert L.hbt_fit_radii(None, 0, None, None, None) == 1
    assert L.hbt_fit_last_error(None) == b"null context"


def test_server_header_matches_its_binding(lib):
    from hadronic_afterburner_toolkit_gb300 import server
    names = _declared_functions(SERVER_HEADER)
    assert "hbt_server_submit" in names and "hbt_server_wait" in names
    assert sorted(server.exported_symbols()) == names


def test_server_create_reports_errors_without_crashing(lib):
    """Without a GPU hbt_server_create returns HBT_ERR_CUDA; with one it
    starts and stops cleanly."""
    from hadronic_afterburner_toolkit_gb300 import server
    L = server.load()
    cfg = server.HbtServerConfig(device=0)
    h = ctypes.c_void_p()
    rc = L.hbt_server_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc in (0, 2)
    if rc == 0:
        L.hbt_server_destroy(h)
    assert L.hbt_server_last_error(None) == b"null server"


def test_binding_loads_without_gpu(lib):
    L = engine.load()
    assert L.hbt_n_bins(None) == 0
    assert L.hbt_last_error(None) == b"null context"


def test_invalid_parameters_rejected_before_any_device_call(lib):
    L = engine.load()
    p = engine.HbtParams(qnpts=1, q_min=-0.1, q_max=0.1, n_KT=5, KT_min=0, KT_max=1,
                         n_Kphi=4, needed_number_of_pairs=1e18)
    h = ctypes.c_void_p()
    assert L.hbt_create(ctypes.byref(p), 0, ctypes.byref(h)) == 1  # HBT_ERR_INVALID
    p.qnpts = 11
    p.precision = 7
    assert L.hbt_create(ctypes.byref(p), 0, ctypes.byref(h)) == 1


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(engine.HbtError):
        engine.load(str(tmp_path / "libhbt_gpu.so"))


def test_check_math_rejects_unknown_functions_without_a_device_call(lib):
    """hbt_check_math validates `which` (cos, exp, double-float cos, cos at
    the pair scale) and its arrays before touching a device."""
    L = engine.load()
    L.hbt_check_math.restype = ctypes.c_int32
    L.hbt_check_math.argtypes = [ctypes.c_int, ctypes.c_int32, ctypes.c_int64,
                                 ctypes.c_void_p, ctypes.c_void_p]
    x = (ctypes.c_double * 1)(0.5)
    out = (ctypes.c_double * 1)()
    assert L.hbt_check_math(0, 4, 1, x, out) == 1           # HBT_ERR_INVALID
    assert L.hbt_check_math(0, -1, 1, x, out) == 1
    assert L.hbt_check_math(0, 2, 1, None, out) == 1        # missing input
    assert L.hbt_check_math(0, 2, 0, None, None) == 0       # nothing to do
    text = open(CHECK_HEADER).read()
    assert "#define HBT_CHECK_DFCOS 2" in text
    assert "#define HBT_CHECK_COS_PHASE 3" in text
