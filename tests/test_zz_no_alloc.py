"""hbt_bin_mixed_rotated_noalloc: the entry point for callers that cannot
allocate device memory (their framework owns the device memory through its
own pool, or their loop cannot afford an allocation's synchronisation).

Every array here is allocated by the test, standing in for such a caller;
the entry point itself allocates nothing.  Its denominator counts must equal
those of the existing entry point (hbt_bin_mixed on the same rotated partner
list) exactly - the tolerance the tests use for counts - over two calls in a
row that add into the same caller-owned histogram.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = dict(qnpts=11, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=4,
              azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
              needed_number_of_pairs=1e18)
COLS = ("px", "py", "pz", "E")


def _params(E, **over):
    p = dict(PARAMS, **over)
    return E.HbtParams(**p, precision=E.PRECISION_FP64, kphi_defer_tol=0.0,
                       kernel=E.KERNEL_SCREENED)


def test_noalloc_matches_existing_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    from hadronic_afterburner_toolkit_gb300 import engine as E
    from hadronic_afterburner_toolkit_gb300 import synth

    L = E.load()
    hp = _params(E)
    ref = E.Engine(**PARAMS)  # existing entry point
    nb = int(L.hbt_n_bins(ref.handle))
    den = torch.zeros(nb, dtype=torch.int64, device="cuda")  # caller-owned output
    stream = torch.cuda.current_stream().cuda_stream
    err = ctypes.create_string_buffer(256)
    for seed, angle in ((41, 0.7), (42, 2.9)):
        ev = synth.generate(4, 300.0, seed=seed, sigma_xy=2.0, tau_mean=3.0)
        cut = int(ev.offsets[1])
        l1_np = [np.ascontiguousarray(getattr(ev, k)[:cut]) for k in COLS]
        pool_np = [np.ascontiguousarray(getattr(ev, k)[cut:]) for k in COLS]
        l1 = [torch.from_numpy(x).cuda() for x in l1_np]
        pool = [torch.from_numpy(x).cuda() for x in pool_np]
        c, s = float(np.cos(angle)), float(np.sin(angle))
        a = E.HbtSoa4(*[t.data_ptr() for t in l1])
        b = E.HbtSoa4(*[t.data_ptr() for t in pool])
        rc = L.hbt_bin_mixed_rotated_noalloc(ctypes.byref(hp), l1[0].numel(), ctypes.byref(a),
                                             pool[0].numel(), ctypes.byref(b), c, s,
                                             ctypes.c_void_p(den.data_ptr()),
                                             ctypes.c_void_p(stream), err, len(err))
        assert rc == E.HBT_OK, err.value
        # the existing entry point on the same list, rotated on the host
        rot = [pool_np[0] * c - pool_np[1] * s, pool_np[0] * s + pool_np[1] * c,
               pool_np[2], pool_np[3]]
        ref.bin_mixed(l1_np, rot)
        torch.cuda.synchronize()
        want = ref.hist()["den"]
        got = den.cpu().numpy().astype(np.float64)
        assert want.sum() > 100
        assert np.array_equal(got, want)


def test_noalloc_rejects_oversized_pool_and_unsupported_flags():
    from hadronic_afterburner_toolkit_gb300 import engine as E
    L = E.load()
    err = ctypes.create_string_buffer(256)
    dummy = E.HbtSoa4(1, 1, 1, 1)
    rc = L.hbt_bin_mixed_rotated_noalloc(ctypes.byref(_params(E)), 10, ctypes.byref(dummy),
                                         65537, ctypes.byref(dummy), 1.0, 0.0,
                                         ctypes.c_void_p(1), None, err, len(err))
    assert rc == 1 and b"HBT_NOALLOC_MAX_POOL" in err.value
    rc = L.hbt_bin_mixed_rotated_noalloc(ctypes.byref(_params(E, azimuthal_flag=1)), 10,
                                         ctypes.byref(dummy), 10, ctypes.byref(dummy), 1.0, 0.0,
                                         ctypes.c_void_p(1), None, err, len(err))
    assert rc == 1 and b"azimuthal_flag" in err.value
