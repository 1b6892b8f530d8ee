"""Output store with the reference's HDF5 layout.

The reference writes every product into ``output_file_name`` with h5py,
deleting and recreating a dataset that already exists
(``write_data.py:1-56``).  This store keeps the same group paths and dataset
names and writes a real HDF5 file either way: through h5py when it is
importable, else through the built-in writer (``hdf5.write_file``), which
rewrites the whole file after each measurement.  In that case datasets
already in the file (earlier runs, other processes) are read first and kept,
as h5py's append mode keeps them; a file the built-in reader cannot parse is
left untouched and the write raises.  Paths are normalised the way HDF5
resolves them ('Snapshot_99//w/xi_gg/' == 'Snapshot_99/w/xi_gg').
"""

from __future__ import annotations

import os

import numpy as np

from . import hdf5

try:  # pragma: no cover - depends on the host
    import h5py  # noqa: F401
    HAVE_H5PY = True
except Exception:
    HAVE_H5PY = False

_STORES: dict[str, "OutputFile"] = {}


def norm_path(*parts):
    return "/".join(p for part in parts for p in str(part).split("/") if p)


class OutputFile:
    def __init__(self, name, use_h5py=None):
        self.name = name
        self.use_h5py = HAVE_H5PY if use_h5py is None else use_h5py
        self.data: dict[str, np.ndarray] = {}
        self._loaded = False

    def _load(self):
        """Datasets already in the file, under the ones written since."""
        if self._loaded:
            return
        self._loaded = True
        if self.name is None or self.use_h5py or not os.path.exists(self.name):
            return
        try:
            old = hdf5.read_file(self.name)
        except (ValueError, NotImplementedError) as exc:
            raise RuntimeError(f"{self.name} exists but cannot be read without h5py ({exc}); "
                               "remove it or install h5py") from exc
        self.data = {**old, **self.data}

    def write(self, group, dataset, value):
        self._load()
        self.data[norm_path(group, dataset)] = np.asarray(value)

    def read(self, path):
        self._load()
        return self.data[norm_path(path)]

    def keys(self):
        self._load()
        return sorted(self.data)

    def flush(self):
        """Write the datasets to ``output_file_name``."""
        if self.name is None:
            return
        if self.use_h5py:
            import h5py
            with h5py.File(self.name, "a") as f:
                for path, v in self.data.items():
                    if path in f:
                        del f[path]
                    f.create_dataset(path, data=v)
            return
        d = os.path.dirname(os.path.abspath(self.name))
        if os.path.isdir(d):
            self._load()
            hdf5.write_file(self.name, self.data)


def open_output(name) -> OutputFile:
    """The store behind ``output_file_name`` (created on first use)."""
    key = os.path.abspath(name) if name is not None else None
    if key not in _STORES:
        _STORES[key] = OutputFile(name)
    return _STORES[key]


def read_output(name) -> dict:
    """``{hdf5 path: array}`` of an output file (h5py not needed)."""
    return hdf5.read_file(name)
