"""Python binding of the balance-function pair binning (include/hbt_bf.h).

``BfEngine`` holds the eight (Delta y, Delta phi) histograms of one analysis
on the GPU; ``bin`` runs a set of event-pair jobs over species lists in one
launch.  No CPU fallback: the calls raise when ``libhbt_gpu.so`` is missing.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np

from . import engine
from .engine import HbtError

_D = ctypes.c_double
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_VP = ctypes.c_void_p
_PD = ctypes.POINTER(ctypes.c_double)
NPHI = 20


class HbtBfParams(ctypes.Structure):
    _fields_ = [("Bnpts", _I32), ("Brap_max", _D)]


class HbtBfList(ctypes.Structure):
    _fields_ = [("n_events", _I32), ("offsets", ctypes.POINTER(ctypes.c_int64)),
                ("phi", _PD), ("y", _PD)]


class HbtBfJob(ctypes.Structure):
    _fields_ = [("hist", _I32), ("la", _I32), ("ea", _I32), ("lb", _I32), ("eb", _I32),
                ("mixed", _I32), ("rotation", _D)]


JOB_DTYPE = np.dtype([("hist", "<i4"), ("la", "<i4"), ("ea", "<i4"), ("lb", "<i4"),
                      ("eb", "<i4"), ("mixed", "<i4"), ("rotation", "<f8")], align=True)


def job_array(jobs) -> np.ndarray:
    """(hist, la, ea, lb, eb, mixed, rotation) tuples as an array laid out
    like ``hbt_bf_job``, which ``BfEngine.bin`` passes without conversion."""
    return np.array([tuple(j) for j in jobs], dtype=JOB_DTYPE)


class HbtBfStats(ctypes.Structure):
    _fields_ = [("pairs", _I64), ("bytes_uploaded", _I64), ("fp64_pairs", _I64),
                ("upload_ms", _D), ("kernel_ms", _D)]


SIGNATURES = {
    "hbt_bf_create": (_I32, [ctypes.POINTER(HbtBfParams), ctypes.c_int, ctypes.POINTER(_VP)]),
    "hbt_bf_destroy": (None, [_VP]),
    "hbt_bf_last_error": (ctypes.c_char_p, [_VP]),
    "hbt_bf_reset": (_I32, [_VP]),
    "hbt_bf_bin": (_I32, [_VP, _I32, ctypes.POINTER(HbtBfList), _I32, ctypes.POINTER(HbtBfJob)]),
    "hbt_bf_read": (_I32, [_VP, _I32, _PD]),
    "hbt_bf_get_stats": (_I32, [_VP, ctypes.POINTER(HbtBfStats)]),
}

_bound = None


def load():
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


class BfEngine:
    """The eight balance-function histograms of one analysis on one GPU."""

    def __init__(self, Bnpts: int, Brap_max: float, device: int = 0):
        self.L = load()
        self.Bnpts = int(Bnpts)
        p = HbtBfParams(Bnpts=self.Bnpts, Brap_max=Brap_max)
        h = _VP()
        rc = self.L.hbt_bf_create(ctypes.byref(p), device, ctypes.byref(h))
        if rc != 0:
            raise HbtError("hbt_bf_create: %s" % engine.STATUS.get(rc, rc))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.L.hbt_bf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise HbtError("%s: %s: %s" % (what, engine.STATUS.get(rc, rc),
                                           self.L.hbt_bf_last_error(self._h).decode()))

    def bin(self, lists: Sequence, jobs: Sequence):
        """lists: (offsets, phi, y) per species list; jobs: (hist, la, ea, lb,
        eb, mixed, rotation) tuples, or an array made by ``job_array``."""
        keep = []
        arr = (HbtBfList * max(len(lists), 1))()
        for k, (off, phi, y) in enumerate(lists):
            off = np.ascontiguousarray(off, dtype=np.int64)
            phi = np.ascontiguousarray(phi, dtype=np.float64)
            y = np.ascontiguousarray(y, dtype=np.float64)
            keep += [off, phi, y]
            arr[k] = HbtBfList(len(off) - 1, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                               phi.ctypes.data_as(_PD), y.ctypes.data_as(_PD))
        if isinstance(jobs, np.ndarray) and jobs.dtype == JOB_DTYPE:
            ja = np.ascontiguousarray(jobs)
            jarr = ctypes.cast(ja.ctypes.data, ctypes.POINTER(HbtBfJob))
        else:
            jarr = (HbtBfJob * max(len(jobs), 1))(*[HbtBfJob(*j) for j in jobs])
        self._check(self.L.hbt_bf_bin(self._h, len(lists), arr, len(jobs), jarr), "hbt_bf_bin")

    def hist(self, which: int) -> np.ndarray:
        out = np.zeros(self.Bnpts * NPHI)
        self._check(self.L.hbt_bf_read(self._h, which, out.ctypes.data_as(_PD)), "hbt_bf_read")
        return out.reshape(self.Bnpts, NPHI)

    def reset(self):
        self._check(self.L.hbt_bf_reset(self._h), "hbt_bf_reset")

    def stats(self) -> dict:
        """Pairs, uploaded bytes, FP64-fallback pairs and device times of the
        last ``bin`` call."""
        st = HbtBfStats()
        self._check(self.L.hbt_bf_get_stats(self._h, ctypes.byref(st)), "hbt_bf_get_stats")
        return {k: getattr(st, k) for k, _ in HbtBfStats._fields_}
