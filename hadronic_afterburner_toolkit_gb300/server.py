"""Python binding of the serving loop's C ABI (include/hbt_server.h).

A ``Server`` owns one GPU; ``submit`` queues one HBT analysis of one event
buffer (its own q grid, K_T / K_phi bins and precision) and returns a job id;
``wait`` / ``result`` give the histograms in the layout of ``Engine.hist``.
No CPU fallback: the calls raise when ``libhbt_gpu.so`` is missing.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import engine
from .engine import HbtError, HbtParams, HbtSoa8

_D = ctypes.c_double
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_PD = ctypes.POINTER(ctypes.c_double)
_PU64 = ctypes.POINTER(ctypes.c_uint64)
_PI32 = ctypes.POINTER(ctypes.c_int32)
_VP = ctypes.c_void_p

JOB_QUEUED, JOB_ACTIVE, JOB_DONE, JOB_FAILED = 0, 1, 2, 3


class HbtServerConfig(ctypes.Structure):
    _fields_ = [("device", _I32), ("memory_budget", _U64), ("max_active", _I32),
                ("round_tile_pairs", _I64), ("max_in_flight", _I32)]


class HbtRequest(ctypes.Structure):
    _fields_ = [("params", HbtParams), ("n_events", _I32),
                ("event_offsets", ctypes.POINTER(ctypes.c_int64)), ("particles", HbtSoa8),
                ("oversample", _I32), ("mixed_partners", _I32),
                ("Krap_min", _D), ("Krap_max", _D), ("seed", _I32)]


class HbtJobInfo(ctypes.Structure):
    _fields_ = [("state", _I32), ("status", _I32), ("solo", _I32), ("rounds", _I32),
                ("queue_ms", _D), ("latency_ms", _D), ("pairs_same", _U64),
                ("pairs_mixed", _U64), ("device_bytes", _U64), ("psi_ref", _D),
                ("n_bins", _I64), ("anomalies", _U64)]


class HbtServerStats(ctypes.Structure):
    _fields_ = [("submitted", _U64), ("completed", _U64), ("failed", _U64),
                ("rounds", _U64), ("pairs", _U64), ("bytes_in_use", _U64),
                ("peak_bytes", _U64), ("active", _I32), ("queued", _I32),
                ("peak_active", _I32), ("p50_ms", _D), ("p99_ms", _D), ("mean_ms", _D),
                ("max_ms", _D), ("gpu_busy_ms", _D)]


# Every entry point of include/hbt_server.h: name -> (restype, argtypes)
SIGNATURES = {
    "hbt_server_create": (_I32, [ctypes.POINTER(HbtServerConfig), ctypes.POINTER(_VP)]),
    "hbt_server_destroy": (None, [_VP]),
    "hbt_server_last_error": (ctypes.c_char_p, [_VP]),
    "hbt_server_submit": (_I32, [_VP, ctypes.POINTER(HbtRequest), ctypes.POINTER(_U64)]),
    "hbt_server_wait": (_I32, [_VP, _U64, _U64]),
    "hbt_server_job_info": (_I32, [_VP, _U64, ctypes.POINTER(HbtJobInfo)]),
    "hbt_server_mixing": (_I32, [_VP, _U64, _PI32, _PI32, _PD, _PD]),
    "hbt_server_read_hist": (_I32, [_VP, _U64] + [_PD] * 6),
    "hbt_server_read_qinv": (_I32, [_VP, _U64] + [_PD] * 4),
    "hbt_server_read_counters": (_I32, [_VP, _U64] + [_PU64] * 4),
    "hbt_server_release": (_I32, [_VP, _U64]),
    "hbt_server_get_stats": (_I32, [_VP, ctypes.POINTER(HbtServerStats)]),
    "hbt_server_reset_stats": (_I32, [_VP]),
}

_bound = None


def load():
    """The engine library with the server's signatures bound."""
    global _bound
    L = engine.load()
    if _bound is not L:
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _bound = L
    return L


def exported_symbols():
    return list(SIGNATURES)


def default_params(**kw) -> dict:
    p = dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=4, KT_min=0.0, KT_max=1.0, n_Kphi=8,
             azimuthal_flag=0, invariant_radius_flag=0, long_comoving_boost=1,
             needed_number_of_pairs=1e18, precision=engine.PRECISION_FP64,
             kphi_defer_tol=0.0, kernel=engine.KERNEL_SCREENED)
    p.update(kw)
    return p


class Server:
    """Continuous-batching HBT request loop on one GPU."""

    def __init__(self, device: int = 0, memory_budget: int = 0, max_active: int = 0,
                 round_tile_pairs: int = 0, max_in_flight: int = 0):
        self.L = load()
        cfg = HbtServerConfig(device=device, memory_budget=memory_budget,
                              max_active=max_active, round_tile_pairs=round_tile_pairs,
                              max_in_flight=max_in_flight)
        h = _VP()
        rc = self.L.hbt_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise HbtError("hbt_server_create: %s" % engine.STATUS.get(rc, rc))
        self._h = h
        self._meta = {}

    def _check(self, rc, what):
        if rc != 0:
            msg = self.L.hbt_server_last_error(self._h).decode()
            raise HbtError("%s: %s: %s" % (what, engine.STATUS.get(rc, rc), msg))

    def close(self):
        if getattr(self, "_h", None):
            self.L.hbt_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, cols8: Sequence, offsets, params: Optional[dict] = None, *,
               oversample: int = 0, mixed_partners: int = 0, Krap_min: float = -1.0,
               Krap_max: float = 1.0, seed: int = 1) -> int:
        """Queue one event buffer: cols8 = (px, py, pz, E, x, y, z, t) of all
        events one after another, offsets = n_events + 1 row offsets."""
        p = default_params(**(params or {}))
        cols = [np.ascontiguousarray(c, dtype=np.float64) for c in cols8]
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        req = HbtRequest(params=HbtParams(**p), n_events=len(off) - 1,
                         event_offsets=off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                         particles=HbtSoa8(*[c.ctypes.data for c in cols]),
                         oversample=oversample, mixed_partners=mixed_partners,
                         Krap_min=Krap_min, Krap_max=Krap_max, seed=seed)
        jid = _U64()
        self._check(self.L.hbt_server_submit(self._h, ctypes.byref(req), ctypes.byref(jid)),
                    "hbt_server_submit")
        self._meta[jid.value] = p
        return int(jid.value)

    def wait(self, job: int, timeout_us: int = 0):
        self._check(self.L.hbt_server_wait(self._h, job, timeout_us), "hbt_server_wait")

    def info(self, job: int) -> dict:
        i = HbtJobInfo()
        self._check(self.L.hbt_server_job_info(self._h, job, ctypes.byref(i)),
                    "hbt_server_job_info")
        return {k: getattr(i, k) for k, _ in HbtJobInfo._fields_}

    def mixing(self, job: int, n_events: int):
        P = ctypes.c_int32()
        self._check(self.L.hbt_server_mixing(self._h, job, ctypes.byref(P), None, None, None),
                    "hbt_server_mixing")
        n = n_events * P.value
        partners = np.zeros(max(n, 1), np.int32)
        c = np.zeros(max(n, 1))
        s = np.zeros(max(n, 1))
        self._check(self.L.hbt_server_mixing(self._h, job, ctypes.byref(P),
                                             partners.ctypes.data_as(_PI32),
                                             c.ctypes.data_as(_PD), s.ctypes.data_as(_PD)),
                    "hbt_server_mixing")
        return P.value, partners[:n].reshape(n_events, P.value), c[:n].reshape(
            n_events, P.value), s[:n].reshape(n_events, P.value)

    def result(self, job: int) -> dict:
        """Histograms of a done job (Engine.hist layout)."""
        p = self._meta[job]
        n_slots = p["n_KT"] * (p["n_Kphi"] if p["azimuthal_flag"] == 1 else 1)
        nb = n_slots * p["qnpts"] ** 3
        keys = ("count", "q_out", "q_side", "q_long", "num", "den")
        out = {k: np.zeros(nb) for k in keys}
        self._check(self.L.hbt_server_read_hist(self._h, job,
                                                *[out[k].ctypes.data_as(_PD) for k in keys]),
                    "hbt_server_read_hist")
        nq = p["n_KT"] * p["qnpts"]
        qk = ("qinv_sum", "qinv_num", "qinv_count", "qinv_den")
        qi = {k: np.zeros(nq) for k in qk}
        self._check(self.L.hbt_server_read_qinv(self._h, job,
                                                *[qi[k].ctypes.data_as(_PD) for k in qk]),
                    "hbt_server_read_qinv")
        out.update(qi)
        nk = p["n_KT"]
        ctr = [np.zeros(n_slots, np.uint64), np.zeros(n_slots, np.uint64),
               np.zeros(nk, np.uint64), np.zeros(nk, np.uint64)]
        self._check(self.L.hbt_server_read_counters(self._h, job,
                                                    *[c.ctypes.data_as(_PU64) for c in ctr]),
                    "hbt_server_read_counters")
        out.update(ctr_num=ctr[0], ctr_den=ctr[1], ctr_num_qinv=ctr[2], ctr_den_qinv=ctr[3])
        info = self.info(job)
        for k in ("pairs_same", "pairs_mixed", "anomalies"):
            out[k] = int(info[k])
        return out

    def release(self, job: int):
        self._check(self.L.hbt_server_release(self._h, job), "hbt_server_release")
        self._meta.pop(job, None)

    def stats(self) -> dict:
        s = HbtServerStats()
        self._check(self.L.hbt_server_get_stats(self._h, ctypes.byref(s)),
                    "hbt_server_get_stats")
        return {k: getattr(s, k) for k, _ in HbtServerStats._fields_}

    def reset_stats(self):
        self._check(self.L.hbt_server_reset_stats(self._h), "hbt_server_reset_stats")
