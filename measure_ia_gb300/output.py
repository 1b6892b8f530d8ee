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

A store of a named file lives only while it holds datasets not yet written:
``flush`` writes the file and releases the store, and the next
``open_output`` of that name reads the file again.  Without a file name
(``output_file_name=None``) the products stay in an in-memory store owned by
the measuring object (``store_for``), never shared between objects.
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

# stores of named files with datasets not yet flushed, by absolute path
_OPEN: dict[str, "OutputFile"] = {}

# the datasets of the last file this process wrote with the built-in writer:
# (absolute path, (size, mtime_ns) of the file just after the write, copies of
# the datasets).  A store opened on that file while it is still unchanged
# takes them instead of parsing the file again (measuring into one file over
# and over re-reads nothing); any other write to the file changes its size or
# time and the file is read
_LAST_WRITTEN: list = []


def _stamp(name):
    st = os.stat(name)
    return (st.st_size, st.st_mtime_ns)


def norm_path(*parts):
    s = "/".join(map(str, parts))
    if "//" in s or s[:1] == "/" or s[-1:] == "/":   # empty components: drop them
        s = "/".join(p for p in s.split("/") if p)
    return s


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
        if self.name is None or not os.path.exists(self.name):
            return
        if self.use_h5py:
            import h5py
            old = {}
            with h5py.File(self.name, "r") as f:
                f.visititems(lambda path, obj: old.__setitem__(path, obj[()]) if isinstance(obj, h5py.Dataset)
                             else None)
        else:
            key = os.path.abspath(self.name)
            if _LAST_WRITTEN and _LAST_WRITTEN[0] == key and _LAST_WRITTEN[1] == _stamp(self.name):
                self.data = {**_LAST_WRITTEN[2], **self.data}
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
        """Write the datasets to ``output_file_name`` and release the store
        (a later ``open_output`` of the name reads the file)."""
        if self.name is None:
            return
        if self.use_h5py:
            import h5py
            with h5py.File(self.name, "a") as f:
                for path, v in self.data.items():
                    if path in f:
                        del f[path]
                    f.create_dataset(path, data=v)
        else:
            d = os.path.dirname(os.path.abspath(self.name))
            if not os.path.isdir(d):  # nowhere to write: the datasets stay in this store
                return
            self._load()
            hdf5.write_file(self.name, self.data)
            _LAST_WRITTEN[:] = [os.path.abspath(self.name), _stamp(self.name),
                                {k: np.array(v, copy=True) for k, v in self.data.items()}]
        key = os.path.abspath(self.name)
        if _OPEN.get(key) is self:
            del _OPEN[key]


def open_output(name) -> OutputFile:
    """The store behind ``output_file_name``: the open one with unflushed
    datasets, else a new one that reads the file on first use.  ``None`` gives
    a new in-memory store (use ``store_for`` to keep one per object)."""
    if name is None:
        return OutputFile(None)
    key = os.path.abspath(name)
    if key not in _OPEN:
        _OPEN[key] = OutputFile(name)
    return _OPEN[key]


def store_for(obj) -> OutputFile:
    """The output store of a measuring object: its file's store, or, without a
    file name, an in-memory store kept on the object itself."""
    if obj.output_file_name is not None:
        return open_output(obj.output_file_name)
    st = getattr(obj, "_memory_store", None)
    if st is None:
        st = OutputFile(None)
        obj._memory_store = st
    return st


def read_output(name) -> dict:
    """``{hdf5 path: array}`` of an output file (h5py not needed)."""
    return hdf5.read_file(name)
