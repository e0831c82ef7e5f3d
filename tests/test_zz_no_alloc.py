"""hbt_bin_mixed_rotated_noalloc: the entry point for callers that cannot
allocate device memory (their framework owns the device memory through its
own pool, or their loop cannot afford an allocation's synchronisation).

Every array here is allocated by the test, standing in for such a caller;
the entry point itself allocates nothing.  Its denominator counts must equal
those of the existing entry point (hbt_bin_mixed on the same rotated partner
list) exactly - the tolerance the tests use for counts - over two calls in a
row that add into the same caller-owned histogram; they must also equal the
CPU oracle's on pairs placed within a few ulps of every bin edge of a
41-point grid and on a pool of exactly HBT_NOALLOC_MAX_POOL particles, and
the device's free memory must not change across calls.
"""
import ctypes
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = dict(qnpts=11, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0, KT_max=1.0, n_Kphi=4,
              azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
              needed_number_of_pairs=1e18)
COLS = ("px", "py", "pz", "E")
MAX_POOL = 65536  # HBT_NOALLOC_MAX_POOL of include/hbt_gpu.h


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


_RT = []


def _default_pool_used_bytes():
    """Bytes in use in the device's default stream-ordered memory pool (the
    pool cudaMallocAsync draws from), or None when no CUDA runtime library
    can be loaded here to ask."""
    import torch
    if not _RT:
        names = [os.path.join(os.path.dirname(torch.__file__), "lib", "libcudart.so"),
                 "libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"]
        for name in names:
            try:
                _RT.append(ctypes.CDLL(name))
                break
            except OSError:
                continue
        else:
            _RT.append(None)
    rt = _RT[0]
    if rt is None:
        return None
    pool = ctypes.c_void_p()
    if rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), 0) != 0:
        return None
    used = ctypes.c_uint64()
    # cudaMemPoolAttrUsedMemCurrent = 0x7
    if rt.cudaMemPoolGetAttribute(pool, 7, ctypes.byref(used)) != 0:
        return None
    return int(used.value)


def _device_memory():
    """(free device bytes, default-pool bytes in use)."""
    import torch
    torch.cuda.synchronize()
    used = _default_pool_used_bytes()
    return torch.cuda.mem_get_info()[0], used


def _call(L, E, hp, l1, pool, c, s, den, stream, err):
    a = E.HbtSoa4(*[t.data_ptr() for t in l1])
    b = E.HbtSoa4(*[t.data_ptr() for t in pool])
    return L.hbt_bin_mixed_rotated_noalloc(ctypes.byref(hp), l1[0].numel(), ctypes.byref(a),
                                           pool[0].numel(), ctypes.byref(b), c, s,
                                           ctypes.c_void_p(den.data_ptr()),
                                           ctypes.c_void_p(stream), err, len(err))


def _edge_list(p, seed=11, per_edge=12):
    """Particles in pairs whose q_out / q_side / q_long lie within a few ulps
    of every bin edge and window bound of p's grid (K along +x, so q_out =
    q_x and q_side = q_y)."""
    rng = np.random.default_rng(seed)
    dq = (p["q_max"] - p["q_min"]) / (p["qnpts"] - 1)
    base = p["q_min"] - dq / 2.0
    edges = [base + k * dq for k in range(p["qnpts"] + 1)]
    edges += [p["q_min"] - dq / 2.0 + 1e-8, p["q_max"] + dq / 2.0 - 1e-8]
    rows = []
    for e in edges:
        for m in range(-per_edge, per_edge + 1):
            val = e + m * 2.0 ** -55
            px2, pz2 = rng.uniform(0.3, 0.6), rng.uniform(-0.3, 0.3)
            which = m % 3
            qx = val if which == 0 else rng.uniform(-0.05, 0.05)
            qy = val if which == 1 else rng.uniform(-0.05, 0.05)
            qz = val if which == 2 else rng.uniform(-0.05, 0.05)
            for (x, y, z) in ((px2 + qx, qy / 2.0, pz2 + qz), (px2, -qy / 2.0, pz2)):
                rows.append((x, y, z, math.sqrt(x * x + y * y + z * z + 0.13957 ** 2)))
    a = np.array(rows)
    return [np.ascontiguousarray(a[:, k]) for k in range(4)]


def test_noalloc_matches_oracle_on_edge_pairs_and_a_full_pool():
    """Against the CPU oracle (the reference's mixed-event loop,
    src/HBT_correlation.cpp:563-689) on a 41-point grid: bin-edge pairs
    unrotated and rotated, then a pool of exactly HBT_NOALLOC_MAX_POOL
    particles, all added into one caller-owned histogram; after the first
    call no further call changes the device's free memory or the default
    memory pool's use."""
    torch = pytest.importorskip("torch")
    import oracle_lib
    from hadronic_afterburner_toolkit_gb300 import engine as E
    from hadronic_afterburner_toolkit_gb300 import synth

    p = dict(PARAMS, qnpts=41, KT_min=0.3, KT_max=0.6)
    L = E.load()
    hp = _params(E, qnpts=41, KT_min=0.3, KT_max=0.6)
    orc = oracle_lib.Oracle(**p)
    nb = orc.hist()["den"].size
    den = torch.zeros(nb, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    err = ctypes.create_string_buffer(256)

    edge = _edge_list(p)
    ev = synth.generate(2, 300.0, seed=5, sigma_xy=2.0, tau_mean=3.0)
    big = synth.generate(1, [MAX_POOL], seed=6, sigma_xy=2.0, tau_mean=3.0)
    assert big.n_particles == MAX_POOL
    cases = [(edge, edge, 0.0), (edge, edge, 1.1),
             ([np.ascontiguousarray(getattr(ev, k)) for k in COLS],
              [np.ascontiguousarray(getattr(big, k)) for k in COLS], 2.3)]
    _device_memory()  # loads the runtime library that reads the pool
    for k, (l1_np, pool_np, angle) in enumerate(cases):
        c, s = (1.0, 0.0) if angle == 0.0 else (math.cos(angle), math.sin(angle))
        l1 = [torch.from_numpy(x).cuda() for x in l1_np]
        pool = [torch.from_numpy(x).cuda() for x in pool_np]
        before = _device_memory()
        assert _call(L, E, hp, l1, pool, c, s, den, stream, err) == E.HBT_OK, err.value
        after = _device_memory()
        if k >= 1:
            # the first call may load the library's kernels; later ones
            # change nothing in device memory
            assert after == before, "device memory changed across a call: %s -> %s" % (
                before, after)
        rot = [pool_np[0] * c - pool_np[1] * s, pool_np[0] * s + pool_np[1] * c,
               pool_np[2], pool_np[3]]
        orc.bin_mixed(l1_np, rot)
        want = orc.hist()["den"]
        got = den.cpu().numpy().astype(np.float64)
        assert np.array_equal(got, want), "case %d: %d bins differ" % (
            k, int((got != want).sum()))
    assert want.sum() > 5000
