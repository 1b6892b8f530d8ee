"""Output store with the reference's HDF5 layout.

The reference writes every product into ``output_file_name`` with h5py,
deleting and recreating a dataset that already exists
(``write_data.py:1-56``).  This store keeps the same group paths and dataset
names.  When h5py is importable each write also goes to the HDF5 file; when
it is not (as on hosts without libhdf5), the datasets are kept in memory and
mirrored to ``<output_file_name>.npz`` after every measurement.  Paths are
normalised the way HDF5 resolves them ('Snapshot_99//w/xi_gg/' ==
'Snapshot_99/w/xi_gg').
"""

from __future__ import annotations

import os

import numpy as np

try:  # pragma: no cover - depends on the host
    import h5py  # noqa: F401
    HAVE_H5PY = True
except Exception:
    HAVE_H5PY = False

_STORES: dict[str, "OutputFile"] = {}


def norm_path(*parts):
    return "/".join(p for part in parts for p in str(part).split("/") if p)


class OutputFile:
    def __init__(self, name):
        self.name = name
        self.data: dict[str, np.ndarray] = {}

    def write(self, group, dataset, value):
        self.data[norm_path(group, dataset)] = np.asarray(value)

    def read(self, path):
        return self.data[norm_path(path)]

    def keys(self):
        return sorted(self.data)

    def flush(self):
        """Mirror the datasets to disk (HDF5 with h5py, else npz)."""
        if self.name is None:
            return
        if HAVE_H5PY:
            import h5py
            with h5py.File(self.name, "a") as f:
                for path, v in self.data.items():
                    if path in f:
                        del f[path]
                    f.create_dataset(path, data=v)
        else:
            d = os.path.dirname(os.path.abspath(self.name))
            if os.path.isdir(d):
                np.savez(self.name + ".npz", **{k.replace("/", "|"): v for k, v in self.data.items()})


def open_output(name) -> OutputFile:
    """The store behind ``output_file_name`` (created on first use)."""
    key = os.path.abspath(name) if name is not None else None
    if key not in _STORES:
        _STORES[key] = OutputFile(name)
    return _STORES[key]


def read_npz_mirror(path):
    """{hdf5 path: array} from a ``.npz`` mirror written by ``OutputFile.flush``."""
    z = np.load(path)
    return {k.replace("|", "/"): z[k] for k in z.files}
