"""Regenerate the radii-fit fixture by running the reference's own script.

    python tests/golden_fit/make_golden_fit.py [REFERENCE_ROOT]

ebe_scripts/fit_HBT_radii.py reads an HDF5 database (one group per event,
one eight-column table per K_T bin) through h5py, which is not installed
here, and calls numpy's removed ``string_`` for its header attribute. The
unmodified script is run with runpy against a small in-memory stand-in for
the part of h5py it uses (File, keys, get, create_dataset, attrs.create)
holding the tables of ``tables.database()``, and with ``string_`` bound to
``numpy.bytes_``. The fit rows it stores (q_cut, lambda, lambda_err, R_out,
R_out_err, ..., R_ol_err per q_cut) are written to expected.json.
"""
from __future__ import annotations

import builtins
import json
import os
import runpy
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import tables  # noqa: E402


def _stub_h5py(db):
    mod = types.ModuleType("h5py")

    class Attrs(dict):
        def create(self, name, value):
            self[name] = value

    class Dataset:
        def __init__(self, data):
            self.data = np.asarray(data)
            self.attrs = Attrs()

    class Group:
        def __init__(self, items):
            self.items = dict(items)

        def keys(self):
            return self.items.keys()

        def get(self, name):
            return self.items.get(name)

        def __delitem__(self, name):
            del self.items[name]

        def create_dataset(self, name, data=None, compression=None, compression_opts=None):
            ds = Dataset(data)
            self.items[name] = ds
            return ds

    class File:
        def __init__(self, name, mode=None):
            self.groups = {ev: Group(t) for ev, t in db.items()}
            mod.last_file = self

        def keys(self):
            return self.groups.keys()

        def __getitem__(self, key):
            return self.groups[key]

        def close(self):
            pass

    mod.File = File
    return mod


def reference_fits(ref: str, db: dict):
    """Runs the unmodified reference script on database `db` (through the
    h5py stand-in) and returns (header, {event: {K_T cut: rows}}).  The
    interpreter state it touches (sys.modules["h5py"], sys.argv,
    builtins.string_) is restored afterwards."""
    script = os.path.join(ref, "ebe_scripts", "fit_HBT_radii.py")
    h5 = _stub_h5py(db)
    saved = (sys.modules.get("h5py"), list(sys.argv), getattr(builtins, "string_", None))
    sys.modules["h5py"] = h5
    builtins.string_ = np.bytes_
    sys.argv = [script, "database.h5"]
    try:
        runpy.run_path(script, run_name="__main__")
    finally:
        if saved[0] is None:
            sys.modules.pop("h5py", None)
        else:
            sys.modules["h5py"] = saved[0]
        sys.argv = saved[1]
        if saved[2] is None:
            del builtins.string_
        else:
            builtins.string_ = saved[2]
    out = {}
    for ev, grp in h5.last_file.groups.items():
        out[ev] = {}
        for cut in tables.KT_CUTS:
            ds = grp.items["HBT_radii_KT_%s.dat" % cut]
            out[ev][cut] = [[float(x) for x in row] for row in ds.data]
        header = grp.items["HBT_radii_KT_%s.dat" % tables.KT_CUTS[0]].attrs["header"]
    return header, out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HBT_REFERENCE_ROOT")
    if not ref:
        raise SystemExit("usage: %s <reference checkout> (or set HBT_REFERENCE_ROOT)" % sys.argv[0])
    header, out = reference_fits(ref, tables.database())
    with open(os.path.join(HERE, "expected.json"), "w") as f:
        json.dump({"header": header.decode(), "fits": out}, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
