"""HBT radii fits on the GPU (include/hbt_fit.h) and the drop-in for the
reference's ebe_scripts/fit_HBT_radii.py.

``fit_tables`` fits every (table, q_cut) of a list of eight-column
correlation tables in one call and returns the script's rows
[q_cut, lambda, lambda_err, R_out, R_out_err, ..., R_ol_err].

``fit_database`` / ``main`` replace the script. The script reads an HDF5
database (one group per event, one dataset per K_T table) and stores
``HBT_radii_KT_<cut>.dat`` datasets back into it. Here the database is a
folder with one sub-folder per event holding the tables as text files of the
same name (the eight-column layout, read with numpy.loadtxt); the radii are
written beside them as text (the script's header line, then one row per
q_cut in ``%.10e``). When h5py is importable, an ``.h5`` database is read and
written like the script does. Events are processed in sorted name order
(HDF5's link order), K_T bins in the script's order.

No CPU fallback: the calls raise when ``libhbt_gpu.so`` is missing.
"""
from __future__ import annotations

import ctypes
import os
import sys
from typing import Sequence

import numpy as np

from . import engine
from .engine import HbtError

_D = ctypes.c_double
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_VP = ctypes.c_void_p
_PD = ctypes.POINTER(ctypes.c_double)

Q_CUT_MAX_LIST = (0.05, 0.075, 0.1, 0.125, 0.15)   # fit_HBT_radii.py:37
KT_CUT_LIST = ("0_0.2", "0.2_0.4", "0.4_0.6", "0.6_0.8")  # :38
P0 = (1.0, 5.0, 5.0, 5.0, 0.1, 0.1)  # :75
HEADER = ("# q_cut[GeV]  lambda  lambda_err  R_out[fm]  R_out_err[fm]  "
          "R_side[fm]  R_side_err[fm]  R_long [fm]  R_long_err[fm]  "
          "R_os[fm]  R_os_err[fm]  R_ol[fm]  R_ol_err[fm]")  # :42-44
STATUS = {0: "converged", 1: "iteration limit", 2: "singular covariance", 3: "too few rows"}


class HbtFitTable(ctypes.Structure):
    _fields_ = [("n_rows", _I64), ("stride", _I64), ("q_out", _PD), ("q_side", _PD),
                ("q_long", _PD), ("C", _PD), ("C_err", _PD)]


class HbtFitOptions(ctypes.Structure):
    _fields_ = [("n_cuts", _I32), ("q_cut_max", _PD), ("q_cut_min", _D), ("p0", _D * 6),
                ("max_iterations", _I32)]


class HbtFitResult(ctypes.Structure):
    _fields_ = [("q_cut", _D), ("p", _D * 6), ("err", _D * 6), ("chi2", _D),
                ("n_points", _I32), ("iterations", _I32), ("status", _I32), ("reserved", _I32)]


RESULT_DTYPE = np.dtype([("q_cut", "<f8"), ("p", "<f8", (6,)), ("err", "<f8", (6,)),
                         ("chi2", "<f8"), ("n_points", "<i4"), ("iterations", "<i4"),
                         ("status", "<i4"), ("reserved", "<i4")])


class HbtFitStats(ctypes.Structure):
    _fields_ = [("fits", _I64), ("rows", _I64), ("points", _I64), ("passes", _I64),
                ("upload_ms", _D), ("kernel_ms", _D)]


SIGNATURES = {
    "hbt_fit_create": (_I32, [ctypes.c_int, ctypes.POINTER(_VP)]),
    "hbt_fit_destroy": (None, [_VP]),
    "hbt_fit_last_error": (ctypes.c_char_p, [_VP]),
    "hbt_fit_radii": (_I32, [_VP, _I32, ctypes.POINTER(HbtFitTable),
                             ctypes.POINTER(HbtFitOptions), ctypes.POINTER(HbtFitResult)]),
    "hbt_fit_get_stats": (_I32, [_VP, ctypes.POINTER(HbtFitStats)]),
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


class Fitter:
    """A fit context on one GPU (device buffers reused across calls)."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = _VP()
        rc = self.L.hbt_fit_create(device, ctypes.byref(h))
        if rc != 0:
            raise HbtError("hbt_fit_create: %s" % engine.STATUS.get(rc, rc))
        self._h = h
        self.last = None

    def close(self):
        if getattr(self, "_h", None):
            self.L.hbt_fit_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fit(self, tables: Sequence[np.ndarray], q_cut_max_list=Q_CUT_MAX_LIST,
            q_cut_min: float = 0.0, p0=P0, max_iterations: int = 0) -> np.ndarray:
        """Rows [n_tables, n_cuts, 13] of the script's layout; the per-fit
        status, chi^2, rows and iterations are in ``self.last``. A table is
        an array of at least eight columns (the script's layout) or a tuple
        (q_out, q_side, q_long, C, C_err) of separate arrays."""
        keep = []
        arr = (HbtFitTable * max(len(tables), 1))()
        for k, t in enumerate(tables):
            if isinstance(t, tuple):
                cols = [np.ascontiguousarray(c, dtype=np.float64) for c in t]
                if len(cols) != 5 or len({c.size for c in cols}) != 1:
                    raise ValueError("table %d: five columns of one length" % k)
                keep += cols
                arr[k] = HbtFitTable(cols[0].size, 1, *[c.ctypes.data_as(_PD) for c in cols])
                continue
            t = np.ascontiguousarray(t, dtype=np.float64)
            if t.ndim != 2 or t.shape[1] < 8:
                raise ValueError("table %d: need at least eight columns" % k)
            keep.append(t)
            base = t.ctypes.data
            col = lambda j: ctypes.cast(base + 8 * j, _PD)  # noqa: E731
            arr[k] = HbtFitTable(t.shape[0], t.shape[1], col(0), col(1), col(2), col(6), col(7))
        cuts = np.ascontiguousarray(q_cut_max_list, dtype=np.float64)
        opt = HbtFitOptions(len(cuts), cuts.ctypes.data_as(_PD), q_cut_min, (_D * 6)(*p0),
                            max_iterations)
        nc = len(cuts)
        out = (HbtFitResult * max(len(tables) * nc, 1))()
        rc = self.L.hbt_fit_radii(self._h, len(tables), arr, ctypes.byref(opt), out)
        if rc != 0:
            raise HbtError("hbt_fit_radii: %s: %s" % (engine.STATUS.get(rc, rc),
                                                      self.L.hbt_fit_last_error(self._h).decode()))
        res = np.frombuffer(out, dtype=RESULT_DTYPE, count=len(tables) * nc).reshape(
            len(tables), nc)
        rows = np.empty((len(tables), nc, 13))
        rows[..., 0] = res["q_cut"]
        rows[..., 1::2] = res["p"]
        rows[..., 2::2] = res["err"]
        info = np.empty((len(tables), nc), dtype=[("status", "i4"), ("chi2", "f8"),
                                                   ("n_points", "i4"), ("iterations", "i4")])
        for k in ("status", "chi2", "n_points", "iterations"):
            info[k] = res[k]
        self.last = info
        return rows

    def stats(self) -> dict:
        st = HbtFitStats()
        rc = self.L.hbt_fit_get_stats(self._h, ctypes.byref(st))
        if rc != 0:
            raise HbtError("hbt_fit_get_stats: %s" % engine.STATUS.get(rc, rc))
        return {k: getattr(st, k) for k, _ in HbtFitStats._fields_}


def fit_tables(tables, q_cut_max_list=Q_CUT_MAX_LIST, q_cut_min=0.0, p0=P0, device=0):
    return Fitter(device).fit(tables, q_cut_max_list, q_cut_min, p0)


def _text_database(folder):
    events = sorted(e for e in os.listdir(folder) if os.path.isdir(os.path.join(folder, e)))
    jobs = []
    for ev in events:
        for kt in KT_CUT_LIST:
            f = os.path.join(folder, ev, "HBT_correlation_function_KT_%s.dat" % kt)
            if os.path.exists(f):
                jobs.append((ev, kt, np.loadtxt(f, ndmin=2)))
    return jobs


def fit_database(database: str, device: int = 0, verbose: bool = True) -> int:
    """Fits every event's K_T tables of a text-folder (or, with h5py, HDF5)
    database and stores the radii beside them. Returns the tables fitted."""
    if os.path.isdir(database):
        jobs = _text_database(database)
        h5 = None
    else:
        import h5py  # only for an HDF5 database
        h5 = h5py.File(database, "r+")
        jobs = []
        for ev in list(h5.keys()):
            for kt in KT_CUT_LIST:
                name = "HBT_correlation_function_KT_%s.dat" % kt
                if name in h5[ev].keys():
                    jobs.append((ev, kt, np.array(h5[ev].get(name))))
    rows = Fitter(device).fit([j[2] for j in jobs]) if jobs else np.empty((0, 5, 13))
    for (ev, kt, _), r in zip(jobs, rows):
        name = "HBT_radii_KT_%s.dat" % kt
        if verbose:
            k = list(Q_CUT_MAX_LIST).index(0.1)
            print("%s %s: R_out = %g fm, R_side = %g fm, R_long = %g fm"
                  % (ev, kt, r[k, 3], r[k, 5], r[k, 7]))
        if h5 is None:
            np.savetxt(os.path.join(database, ev, name), r, fmt="%.10e",
                       header=HEADER[2:], comments="# ")
        else:
            grp = h5[ev]
            if name in grp.keys():
                del grp[name]
            ds = grp.create_dataset(name, data=r, compression="gzip", compression_opts=9)
            ds.attrs.create("header", np.bytes_(HEADER))
    if h5 is not None:
        h5.close()
    return len(jobs)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        print("Usage: python -m hadronic_afterburner_toolkit_gb300.radii database_folder_or.h5")
        return 0
    fit_database(argv[0])
    return 0


if __name__ == "__main__":
    sys.exit(main())
