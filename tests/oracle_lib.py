"""ctypes access to the CPU oracle (oracle/liboracle.so) for the tests.

Test infrastructure: the oracle is what results are compared against, never the thing measured.
Also parses the golden inputs (mode-10 gzip text and OSCAR text) into CSR
event tables, applies the species filter and splits buffers with the
reader's rule, and replays whole golden cases through the oracle.
"""
from __future__ import annotations

import ctypes
import gzip
import os
import subprocess

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "liboracle.so")
GOLDEN = os.path.join(REPO, "tests", "golden")

_D = ctypes.c_double
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_PD = ctypes.POINTER(ctypes.c_double)
_PPD = ctypes.POINTER(_PD)


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("qnpts", _I32), ("q_min", _D), ("q_max", _D),
        ("n_KT", _I32), ("KT_min", _D), ("KT_max", _D),
        ("n_Kphi", _I32), ("azimuthal_flag", _I32),
        ("invariant_radius_flag", _I32), ("long_comoving_boost", _I32),
        ("needed_number_of_pairs", _D), ("HBTrap_min", _D), ("HBTrap_max", _D),
        ("number_of_mixed_events", _I32), ("seed", _I32),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_process_buffer.argtypes = [ctypes.c_void_p, _I32, ctypes.POINTER(_I64), _PPD,
                                         _I32, ctypes.POINTER(_I64), _PPD]
        L.orc_bin_same.argtypes = [ctypes.c_void_p, _I64, _PPD]
        L.orc_bin_mixed.argtypes = [ctypes.c_void_p, _I64, _PPD, _I64, _PPD]
        L.orc_bin_same_mt.argtypes = [ctypes.c_void_p, _I64, _PPD, _I32]
        L.orc_bin_mixed_mt.argtypes = [ctypes.c_void_p, _I64, _PPD, _I64, _PPD, _I32]
        L.orc_rapidity_shift.argtypes = [_I64, _PD, _PD, _D]
        L.orc_set_psi_ref.argtypes = [ctypes.c_void_p, _D]
        L.orc_get_psi_ref.restype = _D
        L.orc_get_psi_ref.argtypes = [ctypes.c_void_p]
        L.orc_event_plane_angle.restype = _D
        L.orc_event_plane_angle.argtypes = [_I64, _PD, _PD, _I32]
        L.orc_n_bins.restype = _I64
        L.orc_n_bins.argtypes = [ctypes.c_void_p]
        L.orc_get_hist.argtypes = [ctypes.c_void_p] + [_PD] * 6
        L.orc_get_qinv.argtypes = [ctypes.c_void_p] + [_PD] * 4
        L.orc_get_counters.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_uint64)] * 4
        for f in ("orc_anomalies", "orc_pairs_same", "orc_pairs_mixed"):
            getattr(L, f).restype = ctypes.c_uint64
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.orc_write.restype = ctypes.c_int
        L.orc_write.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _I32]
        _lib = L
    return _lib


def _pd(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_PD)


def _cols(arrs):
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in arrs]
    ptrs = (_PD * len(arrs))(*[_pd(a) for a in arrs])
    return ptrs, arrs  # keep arrays alive


class Oracle:
    """One oracle context: histograms, pair counters and the RNG."""

    def __init__(self, **kw):
        self.params = dict(kw)
        p = OrcParams()
        defaults = dict(qnpts=41, q_min=-0.15, q_max=0.15, n_KT=5, KT_min=0.0,
                        KT_max=1.0, n_Kphi=8, azimuthal_flag=0,
                        invariant_radius_flag=0, long_comoving_boost=1,
                        needed_number_of_pairs=1e18, HBTrap_min=-1.0,
                        HBTrap_max=1.0, number_of_mixed_events=0, seed=1)
        defaults.update(kw)
        for k, v in defaults.items():
            setattr(p, k, v)
        self.p = defaults
        self._h = lib().orc_create(ctypes.byref(p))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    @property
    def n_slots(self):
        return self.p["n_KT"] * (self.p["n_Kphi"] if self.p["azimuthal_flag"] else 1)

    def bin_same(self, cols8, nthreads: int = 1):
        ptrs, keep = _cols(cols8)
        n = keep[0].size
        if nthreads > 1:
            lib().orc_bin_same_mt(self._h, n, ptrs, nthreads)
        else:
            lib().orc_bin_same(self._h, n, ptrs)

    def bin_mixed(self, l1, l2, nthreads: int = 1):
        p1, k1 = _cols(l1)
        p2, k2 = _cols(l2)
        if nthreads > 1:
            lib().orc_bin_mixed_mt(self._h, k1[0].size, p1, k2[0].size, p2, nthreads)
        else:
            lib().orc_bin_mixed(self._h, k1[0].size, p1, k2[0].size, p2)

    def set_psi_ref(self, psi: float):
        lib().orc_set_psi_ref(self._h, psi)

    def process_buffer(self, ev, mixed=None):
        mixed = ev if mixed is None else mixed
        cols = [ev.px, ev.py, ev.pz, ev.E, ev.x, ev.y, ev.z, ev.t]
        mcols = [mixed.px, mixed.py, mixed.pz, mixed.E, mixed.x, mixed.y, mixed.z, mixed.t]
        p, k = _cols(cols)
        mp, mk = _cols(mcols)
        off = np.ascontiguousarray(ev.offsets, dtype=np.int64)
        moff = np.ascontiguousarray(mixed.offsets, dtype=np.int64)
        lib().orc_process_buffer(self._h, ev.n_events, off.ctypes.data_as(ctypes.POINTER(_I64)), p,
                                 mixed.n_events, moff.ctypes.data_as(ctypes.POINTER(_I64)), mp)

    def hist(self) -> dict:
        n = lib().orc_n_bins(self._h)
        out = {k: np.zeros(n) for k in ("count", "q_out", "q_side", "q_long", "num", "den")}
        lib().orc_get_hist(self._h, *[_pd(out[k]) for k in
                                      ("count", "q_out", "q_side", "q_long", "num", "den")])
        nq = self.p["n_KT"] * self.p["qnpts"]
        qi = {k: np.zeros(nq) for k in ("qinv_sum", "qinv_num", "qinv_count", "qinv_den")}
        lib().orc_get_qinv(self._h, *[_pd(qi[k]) for k in
                                      ("qinv_sum", "qinv_num", "qinv_count", "qinv_den")])
        out.update(qi)
        ns, nk = self.n_slots, self.p["n_KT"]
        ctr = [np.zeros(ns, np.uint64), np.zeros(ns, np.uint64),
               np.zeros(nk, np.uint64), np.zeros(nk, np.uint64)]
        lib().orc_get_counters(self._h, *[c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
                                          for c in ctr])
        out.update(ctr_num=ctr[0], ctr_den=ctr[1], ctr_num_qinv=ctr[2], ctr_den_qinv=ctr[3])
        out["anomalies"] = int(lib().orc_anomalies(self._h))
        out["pairs_same"] = int(lib().orc_pairs_same(self._h))
        out["pairs_mixed"] = int(lib().orc_pairs_mixed(self._h))
        return out

    def write(self, path: str, eco_output: int = 0):
        rc = lib().orc_write(self._h, path.encode(), eco_output)
        assert rc == 0


def rapidity_shift(ev, shift: float):
    E = np.ascontiguousarray(ev.E, dtype=np.float64).copy()
    pz = np.ascontiguousarray(ev.pz, dtype=np.float64).copy()
    lib().orc_rapidity_shift(E.size, _pd(E), _pd(pz), shift)
    ev.E, ev.pz = E, pz


def event_plane_angle(px, py, n_order: int = 2) -> float:
    px = np.ascontiguousarray(px, dtype=np.float64)
    py = np.ascontiguousarray(py, dtype=np.float64)
    return lib().orc_event_plane_angle(px.size, _pd(px), _pd(py), n_order)


# ---------------------------------------------------------------- inputs

def read_params(path: str) -> dict:
    """key = value # comment, names lower-cased (ParameterReader semantics)."""
    out = {}
    for line in open(path):
        line = line.split("#", 1)[0]
        if not line.strip():
            continue
        k, v = line.split("=", 1)
        out[k.strip().lower()] = float(v.strip())
    return out


def _events_from_rows(evs):
    from hadronic_afterburner_toolkit_gb300 import synth
    mult = np.array([len(e) for e in evs], dtype=np.int64)
    off = np.zeros(mult.size + 1, dtype=np.int64)
    np.cumsum(mult, out=off[1:])
    rows = [r for e in evs for r in e]
    if rows:
        a = np.array(rows, dtype=np.float64).reshape(-1, 10)
    else:
        a = np.zeros((0, 10))
    # row layout: monval mass t x y z E px py pz
    return synth.Events(off, a[:, 0].astype(np.int32), a[:, 1], a[:, 2], a[:, 3],
                        a[:, 4], a[:, 5], a[:, 6], a[:, 7], a[:, 8], a[:, 9])


def read_mode10(path: str):
    """Every event of an iSS gzip sample file, in file order."""
    evs = []
    with gzip.open(path, "rt") as f:
        lines = f.read().split("\n")
    k = 0
    while k < len(lines) and lines[k].strip():
        n = int(lines[k].split()[0])
        k += 1
        ev = []
        for _ in range(n):
            ev.append([float(v) for v in lines[k].split()[:10]])
            k += 1
        evs.append(ev)
    return _events_from_rows(evs)


def read_oscar(path: str):
    evs = []
    with open(path) as f:
        lines = f.read().split("\n")[3:]
    k = 0
    while k < len(lines) and lines[k].strip():
        n = int(lines[k].split()[1])
        k += 1
        ev = []
        for _ in range(n):
            v = lines[k].split()
            # idx monval px py pz E mass x y z t -> monval mass t x y z E px py pz
            px, py, pz, E, m, x, y, z, t = (float(s) for s in v[2:11])
            ev.append([float(v[1]), m, t, x, y, z, E, px, py, pz])
            k += 1
        evs.append(ev)
    return _events_from_rows(evs)


def filter_species(ev, monval: int):
    """Keep particles whose Monte-Carlo number equals ``monval`` (every event
    is kept, possibly empty)."""
    from hadronic_afterburner_toolkit_gb300 import synth
    keep = ev.monval == monval
    evid = np.repeat(np.arange(ev.n_events), ev.multiplicities())
    mult = np.bincount(evid[keep], minlength=ev.n_events).astype(np.int64)
    off = np.zeros(ev.n_events + 1, dtype=np.int64)
    np.cumsum(mult, out=off[1:])
    fields = ("monval", "mass", "t", "x", "y", "z", "E", "px", "py", "pz")
    return synth.Events(off, *[getattr(ev, f)[keep] for f in fields])


def reference_checkout() -> str:
    """The reference checkout on this machine, if any: HBT_REFERENCE_ROOT,
    else the one the oracle's build recipe (oracle/Makefile) finds; "" when
    there is none."""
    env = os.environ.get("HBT_REFERENCE_ROOT", "")
    if env:
        return env
    try:
        out = subprocess.run(["make", "-s", "-C", ORACLE_DIR, "print-ref"],
                             capture_output=True, text=True, timeout=60)
    except (OSError, subprocess.SubprocessError):
        return ""
    return out.stdout.strip() if out.returncode == 0 else ""


def golden_case(name: str, root: str = GOLDEN):
    """(params, events, mixed_events_or_None) of one golden case (a folder
    of root holding parameters.dat and the input files)."""
    d = os.path.join(root, name)
    prm = read_params(os.path.join(d, "parameters.dat"))
    if int(prm["read_in_mode"]) == 10:
        ev = read_mode10(os.path.join(d, "particle_samples.gz"))
        mp = os.path.join(d, "particle_samples_mixed_event.gz")
        mixed = read_mode10(mp) if os.path.exists(mp) else None
    else:
        ev = read_oscar(os.path.join(d, "OSCAR.DAT"))
        mp = os.path.join(d, "OSCAR_mixed_event.DAT")
        mixed = read_oscar(mp) if os.path.exists(mp) else None
    return prm, ev, mixed


def oracle_params_from(prm: dict) -> dict:
    return dict(qnpts=int(prm["qnpts"]), q_min=prm["q_min"], q_max=prm["q_max"],
                n_KT=int(prm["n_kt"]), KT_min=prm["kt_min"], KT_max=prm["kt_max"],
                n_Kphi=int(prm["n_kphi"]), azimuthal_flag=int(prm["azimuthal_flag"]),
                invariant_radius_flag=int(prm["invariant_radius_flag"]),
                long_comoving_boost=int(prm["long_comoving_boost"]),
                needed_number_of_pairs=prm["needed_number_of_pairs"],
                HBTrap_min=prm["hbtrap_min"], HBTrap_max=prm["hbtrap_max"],
                number_of_mixed_events=int(prm.get("number_of_mixed_events", 0)),
                seed=int(prm["randomseed"]))


def buffer_ranges(mult, event_buffer_size):
    """Reader buffering: whole events until the count reaches the size."""
    out, e, n = [], 0, len(mult)
    while e < n:
        s, cnt = e, 0
        while cnt < event_buffer_size and e < n:
            cnt += int(mult[e])
            e += 1
        out.append((s, e))
    return out


def run_golden_case_through_oracle(name: str, out_dir: str, root: str = GOLDEN) -> Oracle:
    from hadronic_afterburner_toolkit_gb300 import synth
    prm, ev, mixed = golden_case(name, root)
    shift = prm.get("rapidity_shift", 0.0)
    if shift != 0.0:
        rapidity_shift(ev, shift)
        if mixed is not None:
            rapidity_shift(mixed, shift)
    mon = int(prm["particle_monval"])
    size = int(prm["event_buffer_size"])
    orc = Oracle(**oracle_params_from(prm))
    # buffers are formed on the unfiltered stream (the reader counts every
    # particle it reads), then filtered by species
    rng_same = buffer_ranges(ev.multiplicities(), size)
    rng_mixed = buffer_ranges(mixed.multiplicities(), size) if mixed is not None else None
    for b, (s, e) in enumerate(rng_same):
        buf = filter_species(synth.subset(ev, s, e), mon)
        if mixed is not None:
            ms, me = rng_mixed[b]
            mbuf = filter_species(synth.subset(mixed, ms, me), mon)
        else:
            mbuf = None
        orc.process_buffer(buf, mbuf)
    orc.write(out_dir, int(prm.get("ecooutput", 0)))
    return orc


# ------------------------------------------------------- balance function

GOLDEN_BF = os.path.join(REPO, "tests", "golden_bf")


class OrcBfParams(ctypes.Structure):
    _fields_ = [("particle_alpha", _I32), ("particle_beta", _I32), ("BpT_min", _D),
                ("BpT_max", _D), ("Bnpts", _I32), ("Brap_max", _D), ("rap_type", _I32),
                ("seed", _I32)]


def _bf_lib():
    L = lib()
    if getattr(L, "_bf_bound", False):
        return L
    _PI32 = ctypes.POINTER(_I32)
    L.orc_bf_create.restype = ctypes.c_void_p
    L.orc_bf_create.argtypes = [ctypes.POINTER(OrcBfParams)]
    L.orc_bf_destroy.argtypes = [ctypes.c_void_p]
    L.orc_bf_boost.argtypes = [_I64] + [_PD] * 5 + [_D] + [_PD] * 4
    L.orc_bf_process_buffer.argtypes = [ctypes.c_void_p, _I32, ctypes.POINTER(_I64), _PI32] + \
        [_PD] * 4 + [_I32, ctypes.POINTER(_I64), _PI32] + [_PD] * 4
    L.orc_bf_bin.argtypes = [ctypes.c_void_p, _I32, _I64, _PD, _PD, _PD, _I64, _PD, _PD, _PD,
                             _I32, _D]
    L.orc_bf_get_hist.argtypes = [ctypes.c_void_p, _I32, _PD]
    L.orc_bf_get_norm.argtypes = [ctypes.c_void_p, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]
    L.orc_bf_write.restype = ctypes.c_int
    L.orc_bf_write.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    L._bf_bound = True
    return L


def bf_boost(ev, shift: float = 0.0) -> dict:
    """pT, phi_p, rap_y, rap_eta of every particle (the reader's boost)."""
    n = ev.px.size
    out = {k: np.zeros(n) for k in ("pT", "phi", "y", "eta")}
    cols = [np.ascontiguousarray(getattr(ev, k), dtype=np.float64)
            for k in ("mass", "px", "py", "pz", "E")]
    _bf_lib().orc_bf_boost(n, *[_pd(c) for c in cols], shift,
                           *[_pd(out[k]) for k in ("pT", "phi", "y", "eta")])
    return out


class BfOracle:
    def __init__(self, **kw):
        p = OrcBfParams(**kw)
        self.p = dict(kw)
        self._h = _bf_lib().orc_bf_create(ctypes.byref(p))

    def __del__(self):
        if getattr(self, "_h", None):
            _bf_lib().orc_bf_destroy(self._h)
            self._h = None

    def process_buffer(self, ev, kin, mev=None, mkin=None):
        """ev: events of one buffer; kin: bf_boost of it (likewise the pool)."""
        if mev is None:
            mev, mkin = ev, kin
        keep = []

        def args(e, k):
            off = np.ascontiguousarray(e.offsets, dtype=np.int64)
            mon = np.ascontiguousarray(e.monval, dtype=np.int32)
            cols = [np.ascontiguousarray(k[x]) for x in ("pT", "phi", "y", "eta")]
            keep.append((off, mon, cols))
            return ([e.n_events, off.ctypes.data_as(ctypes.POINTER(_I64)),
                     mon.ctypes.data_as(ctypes.POINTER(_I32))] + [_pd(c) for c in cols])
        _bf_lib().orc_bf_process_buffer(self._h, *args(ev, kin), *args(mev, mkin))

    def hist(self, which: int) -> np.ndarray:
        out = np.zeros(self.p["Bnpts"] * 20)
        _bf_lib().orc_bf_get_hist(self._h, which, _pd(out))
        return out.reshape(self.p["Bnpts"], 20)

    def write(self, path: str):
        assert _bf_lib().orc_bf_write(self._h, path.encode()) == 0


def bf_golden_case(name: str, root: str = GOLDEN_BF):
    d = os.path.join(root, name)
    prm = read_params(os.path.join(d, "parameters.dat"))
    if int(prm["read_in_mode"]) == 10:
        ev = read_mode10(os.path.join(d, "particle_samples.gz"))
        mp = os.path.join(d, "particle_samples_mixed_event.gz")
        mixed = read_mode10(mp) if os.path.exists(mp) else None
    else:
        ev = read_oscar(os.path.join(d, "OSCAR.DAT"))
        mp = os.path.join(d, "OSCAR_mixed_event.DAT")
        mixed = read_oscar(mp) if os.path.exists(mp) else None
    return prm, ev, mixed


def bf_params_from(prm: dict) -> dict:
    return dict(particle_alpha=int(prm["particle_alpha"]), particle_beta=int(prm["particle_beta"]),
                BpT_min=prm["bpt_min"], BpT_max=prm["bpt_max"], Bnpts=int(prm["bnpts"]),
                Brap_max=prm["brap_max"], rap_type=int(prm["rap_type"]),
                seed=int(prm["randomseed"]))


def run_bf_golden_case_through_oracle(name: str, out_dir: str,
                                      root: str = GOLDEN_BF) -> BfOracle:
    from hadronic_afterburner_toolkit_gb300 import synth
    prm, ev, mixed = bf_golden_case(name, root)
    shift = prm.get("rapidity_shift", 0.0)
    size = int(prm["event_buffer_size"])
    orc = BfOracle(**bf_params_from(prm))
    rng_same = buffer_ranges(ev.multiplicities(), size)
    rng_mixed = buffer_ranges(mixed.multiplicities(), size) if mixed is not None else None
    for b, (s, e) in enumerate(rng_same):
        buf = synth.subset(ev, s, e)
        if mixed is not None:
            ms, me = rng_mixed[b]
            mbuf = synth.subset(mixed, ms, me)
            orc.process_buffer(buf, bf_boost(buf, shift), mbuf, bf_boost(mbuf, shift))
        else:
            orc.process_buffer(buf, bf_boost(buf, shift))
    orc.write(out_dir)
    return orc
