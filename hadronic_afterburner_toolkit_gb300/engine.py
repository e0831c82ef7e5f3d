"""Python binding of the GPU engine's C ABI (include/hbt_gpu.h) via ctypes.

This is a thin mirror for tests, benchmarks and Python callers; the C++
drop-in host (``HBT_correlation``) calls the same C ABI directly.  There is no
CPU fallback: if ``lib/libhbt_gpu.so`` is missing or cannot be loaded, every
entry point raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libhbt_gpu.so")

HBT_OK = 0
STATUS = {0: "HBT_OK", 1: "HBT_ERR_INVALID", 2: "HBT_ERR_CUDA", 3: "HBT_ERR_NOMEM",
          4: "HBT_ERR_TIMEOUT", 5: "HBT_ERR_DEVICE", 6: "HBT_ERR_STATE"}
PRECISION_FP64 = 0
PRECISION_FP32W = 1
PRECISION_DF64 = 2
KERNEL_SCREENED = 0
KERNEL_REFERENCE_CHAIN = 1
KERNEL_SCREENED_GRID = 2

_D = ctypes.c_double
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_PD = ctypes.POINTER(ctypes.c_double)
_PU64 = ctypes.POINTER(ctypes.c_uint64)


class HbtParams(ctypes.Structure):
    _fields_ = [
        ("qnpts", _I32), ("q_min", _D), ("q_max", _D),
        ("n_KT", _I32), ("KT_min", _D), ("KT_max", _D),
        ("n_Kphi", _I32), ("azimuthal_flag", _I32),
        ("invariant_radius_flag", _I32), ("long_comoving_boost", _I32),
        ("needed_number_of_pairs", _D), ("precision", _I32),
        ("kphi_defer_tol", _D), ("kernel", _I32),
    ]


class HbtSoa8(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("px", "py", "pz", "E", "x", "y", "z", "t")]


class HbtSoa4(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in ("px", "py", "pz", "E")]


class HbtJob(ctypes.Structure):
    _fields_ = [("kind", _I32), ("na", _I64), ("nb", _I64), ("a", HbtSoa8), ("b", HbtSoa8)]


class HbtTuning(ctypes.Structure):
    _fields_ = [("blocks_per_sm", _I32), ("cell_pt", _D), ("cell_y", _D),
                ("merge_chunk", _I32), ("use_graph", _I32), ("time_kernels", _I32),
                ("order_items", _I32)]


class HbtStats(ctypes.Structure):
    _fields_ = [(k, _U64) for k in ("pairs_same", "pairs_mixed", "launches",
                                    "ordered_passes", "deferred_kphi", "anomalies",
                                    "graph_captures", "graph_replays")] + \
        [("same_kernel_ms", _D), ("mixed_kernel_ms", _D)] + \
        [(k, _U64) for k in ("tiles_same", "tiles_mixed", "tiles_same_kept", "tiles_mixed_kept")]


# Every entry point of include/hbt_gpu.h: name -> (restype, argtypes)
_SIGNATURES = {
    "hbt_create": (_I32, [ctypes.POINTER(HbtParams), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "hbt_destroy": (None, [ctypes.c_void_p]),
    "hbt_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "hbt_set_stream": (_I32, [ctypes.c_void_p, ctypes.c_void_p]),
    "hbt_set_psi_ref": (_I32, [ctypes.c_void_p, _D]),
    "hbt_reset": (_I32, [ctypes.c_void_p]),
    "hbt_bin_same": (_I32, [ctypes.c_void_p, _I64, ctypes.POINTER(HbtSoa8)]),
    "hbt_bin_mixed": (_I32, [ctypes.c_void_p, _I64, ctypes.POINTER(HbtSoa4), _I64,
                             ctypes.POINTER(HbtSoa4)]),
    "hbt_bin_same_dev": (_I32, [ctypes.c_void_p, _I64, ctypes.POINTER(HbtSoa8)]),
    "hbt_bin_mixed_dev": (_I32, [ctypes.c_void_p, _I64, ctypes.POINTER(HbtSoa4), _I64,
                                 ctypes.POINTER(HbtSoa4)]),
    "hbt_bin_batch": (_I32, [ctypes.c_void_p, _I32, ctypes.POINTER(HbtJob)]),
    "hbt_bin_batch_dev": (_I32, [ctypes.c_void_p, _I32, ctypes.POINTER(HbtJob)]),
    "hbt_set_tuning": (_I32, [ctypes.c_void_p, ctypes.POINTER(HbtTuning)]),
    "hbt_get_tuning": (_I32, [ctypes.c_void_p, ctypes.POINTER(HbtTuning)]),
    "hbt_autotune_batch": (_I32, [ctypes.c_void_p, _I32, ctypes.POINTER(HbtJob), _D,
                                  ctypes.POINTER(HbtTuning), ctypes.POINTER(_D)]),
    "hbt_sync": (_I32, [ctypes.c_void_p, _U64]),
    "hbt_n_bins": (_I64, [ctypes.c_void_p]),
    "hbt_read_hist": (_I32, [ctypes.c_void_p] + [_PD] * 6),
    "hbt_read_hist_async": (_I32, [ctypes.c_void_p] + [_PD] * 6),
    "hbt_read_hist_wait": (_I32, [ctypes.c_void_p]),
    "hbt_read_qinv": (_I32, [ctypes.c_void_p] + [_PD] * 4),
    "hbt_read_counters": (_I32, [ctypes.c_void_p] + [_PU64] * 4),
    "hbt_get_stats": (_I32, [ctypes.c_void_p, ctypes.POINTER(HbtStats)]),
    "hbt_inject_alloc_failure": (_I32, [ctypes.c_void_p, _I32]),
    "hbt_bin_mixed_rotated_noalloc": (_I32, [ctypes.POINTER(HbtParams), _I64,
                                             ctypes.POINTER(HbtSoa4), _I64,
                                             ctypes.POINTER(HbtSoa4), _D, _D,
                                             ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_char_p, ctypes.c_size_t]),
}

_lib = None


class HbtError(RuntimeError):
    pass


def load(path: Optional[str] = None):
    """Load libhbt_gpu.so (raises if it is absent: no CPU fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise HbtError("native engine not built: %s (run __graft_entry__.build())" % p)
    L = ctypes.CDLL(p)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def exported_symbols():
    return list(_SIGNATURES)


def _arr(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a


def _ptr(a) -> int:
    """Host numpy array or an object exposing a device pointer (data_ptr())."""
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class Engine:
    """One HBT analysis on one GPU: device histograms + pair binning."""

    def __init__(self, *, qnpts=41, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0,
                 KT_max=1.0, n_Kphi=8, azimuthal_flag=0, invariant_radius_flag=0,
                 long_comoving_boost=1, needed_number_of_pairs=1e18,
                 precision=PRECISION_FP64, kphi_defer_tol=0.0, kernel=0, device=0):
        self.L = load()
        self.params = dict(qnpts=qnpts, q_min=q_min, q_max=q_max, n_KT=n_KT, KT_min=KT_min,
                           KT_max=KT_max, n_Kphi=n_Kphi, azimuthal_flag=azimuthal_flag,
                           invariant_radius_flag=invariant_radius_flag,
                           long_comoving_boost=long_comoving_boost,
                           needed_number_of_pairs=needed_number_of_pairs,
                           precision=precision, kphi_defer_tol=kphi_defer_tol,
                           kernel=kernel)
        p = HbtParams(**self.params)
        h = ctypes.c_void_p()
        self._check(self.L.hbt_create(ctypes.byref(p), device, ctypes.byref(h)), None)
        self._h = h

    # ------------------------------------------------------------- basics
    def _check(self, rc, h="self"):
        if rc != HBT_OK:
            msg = ""
            if h == "self" and getattr(self, "_h", None):
                msg = self.L.hbt_last_error(self._h).decode()
            raise HbtError("%s: %s" % (STATUS.get(rc, rc), msg))

    def close(self):
        if getattr(self, "_h", None):
            self.L.hbt_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_slots(self):
        p = self.params
        return p["n_KT"] * (p["n_Kphi"] if p["azimuthal_flag"] else 1)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int):
        self._check(self.L.hbt_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def set_psi_ref(self, psi: float):
        self._check(self.L.hbt_set_psi_ref(self._h, psi))

    def reset(self):
        self._check(self.L.hbt_reset(self._h))

    def sync(self, timeout_us: int = 0):
        self._check(self.L.hbt_sync(self._h, timeout_us))

    # ------------------------------------------------------------ binning
    def bin_same(self, cols8: Sequence, device: bool = False):
        """Same-event pairs of one gathered list (px, py, pz, E, x, y, z, t)."""
        if not device:
            cols8 = [_arr(c) for c in cols8]
        n = int(cols8[0].shape[0]) if hasattr(cols8[0], "shape") else len(cols8[0])
        soa = HbtSoa8(*[_ptr(c) for c in cols8])
        fn = self.L.hbt_bin_same_dev if device else self.L.hbt_bin_same
        self._check(fn(self._h, n, ctypes.byref(soa)))

    def bin_mixed(self, l1: Sequence, l2: Sequence, device: bool = False):
        """Mixed-event pairs list1 x list2 (px, py, pz, E each)."""
        if not device:
            l1 = [_arr(c) for c in l1]
            l2 = [_arr(c) for c in l2]
        n1 = int(l1[0].shape[0])
        n2 = int(l2[0].shape[0])
        a = HbtSoa4(*[_ptr(c) for c in l1[:4]])
        b = HbtSoa4(*[_ptr(c) for c in l2[:4]])
        fn = self.L.hbt_bin_mixed_dev if device else self.L.hbt_bin_mixed
        self._check(fn(self._h, n1, ctypes.byref(a), n2, ctypes.byref(b)))

    def bin_batch(self, jobs: Sequence, device: bool = False):
        """Many jobs in one persistent launch.  Each job is ("same", cols8)
        or ("mixed", cols4_list1, cols4_list2)."""
        arr, keep = self._job_array(jobs, device)
        fn = self.L.hbt_bin_batch_dev if device else self.L.hbt_bin_batch
        self._check(fn(self._h, len(jobs), arr))

    # ------------------------------------------------------------- tuning
    def set_tuning(self, **kw):
        t = HbtTuning()
        self._check(self.L.hbt_get_tuning(self._h, ctypes.byref(t)))
        for k, v in kw.items():
            setattr(t, k, v)
        self._check(self.L.hbt_set_tuning(self._h, ctypes.byref(t)))

    def tuning(self) -> dict:
        t = HbtTuning()
        self._check(self.L.hbt_get_tuning(self._h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in HbtTuning._fields_}

    def autotune(self, jobs: Sequence, max_pairs: float = 0.0):
        """Autotune the batched path on device-array jobs (bin_batch layout);
        returns (tuning dict, best time in ms)."""
        arr, keep = self._job_array(jobs, True)
        t = HbtTuning()
        ms = _D()
        self._check(self.L.hbt_autotune_batch(self._h, len(jobs), arr, max_pairs,
                                              ctypes.byref(t), ctypes.byref(ms)))
        return {k: getattr(t, k) for k, _ in HbtTuning._fields_}, ms.value

    @staticmethod
    def _job_array(jobs: Sequence, device: bool):
        arr = (HbtJob * max(len(jobs), 1))()
        keep = []
        for k, job in enumerate(jobs):
            if job[0] == "same":
                cols = job[1] if device else [_arr(c) for c in job[1]]
                keep.append(cols)
                arr[k].kind = 0
                arr[k].na = int(cols[0].shape[0])
                arr[k].nb = 0
                arr[k].a = HbtSoa8(*[_ptr(c) for c in cols])
            else:
                a = job[1] if device else [_arr(c) for c in job[1]]
                b = job[2] if device else [_arr(c) for c in job[2]]
                keep.append((a, b))
                arr[k].kind = 1
                arr[k].na = int(a[0].shape[0])
                arr[k].nb = int(b[0].shape[0])
                arr[k].a = HbtSoa8(*([_ptr(c) for c in a[:4]] + [0, 0, 0, 0]))
                arr[k].b = HbtSoa8(*([_ptr(c) for c in b[:4]] + [0, 0, 0, 0]))
        return arr, keep

    # ------------------------------------------------------------ results
    def hist(self) -> dict:
        n = int(self.L.hbt_n_bins(self._h))
        keys = ("count", "q_out", "q_side", "q_long", "num", "den")
        out = {k: np.zeros(n) for k in keys}
        self._check(self.L.hbt_read_hist(self._h, *[out[k].ctypes.data_as(_PD) for k in keys]))
        nq = self.params["n_KT"] * self.params["qnpts"]
        qk = ("qinv_sum", "qinv_num", "qinv_count", "qinv_den")
        qi = {k: np.zeros(nq) for k in qk}
        self._check(self.L.hbt_read_qinv(self._h, *[qi[k].ctypes.data_as(_PD) for k in qk]))
        out.update(qi)
        ns, nk = self.n_slots, self.params["n_KT"]
        ctr = [np.zeros(ns, np.uint64), np.zeros(ns, np.uint64),
               np.zeros(nk, np.uint64), np.zeros(nk, np.uint64)]
        self._check(self.L.hbt_read_counters(self._h, *[c.ctypes.data_as(_PU64) for c in ctr]))
        out.update(ctr_num=ctr[0], ctr_den=ctr[1], ctr_num_qinv=ctr[2], ctr_den_qinv=ctr[3])
        st = self.stats()
        out["anomalies"] = st["anomalies"]
        out["pairs_same"] = st["pairs_same"]
        out["pairs_mixed"] = st["pairs_mixed"]
        return out

    def counters(self) -> dict:
        """The pair counters alone (hbt_read_counters): binned numerator and
        denominator pairs per slot and per K_T bin of the q_inv histograms."""
        ns, nk = self.n_slots, self.params["n_KT"]
        ctr = [np.zeros(ns, np.uint64), np.zeros(ns, np.uint64),
               np.zeros(nk, np.uint64), np.zeros(nk, np.uint64)]
        self._check(self.L.hbt_read_counters(self._h, *[c.ctypes.data_as(_PU64) for c in ctr]))
        return dict(num=ctr[0], den=ctr[1], num_qinv=ctr[2], den_qinv=ctr[3])

    def stats(self) -> dict:
        s = HbtStats()
        self._check(self.L.hbt_get_stats(self._h, ctypes.byref(s)))
        return {k: (getattr(s, k) if t is _D else int(getattr(s, k)))
                for k, t in HbtStats._fields_}
