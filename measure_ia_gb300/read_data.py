"""Catalogue and result ingestion: ReadData (``read_data.py`` of the reference).

Same constructor and methods as the reference:

* ``read_cat`` -- one dataset of ``<data_path>/<catalogue>.hdf5`` under
  ``<snap_group><sub_group>`` (``read_data.py:86-118``);
* ``read_subhalo`` -- a dataset of the simulation's group catalogue,
  concatenated over its files ``<fof_folder>.<n>.hdf5`` (``:120-164``);
* ``read_snapshot`` / ``read_snapshot_multiple`` -- the same over the
  snapshot files, optionally written into ``output_file_name``
  (``:166-302``);
* ``read_MeasureIA_output`` -- w / multipoles, their jackknife errors and
  covariances from a measurement file (``:304-376``).

Files are read with h5py when it is installed, else with the package's own
HDF5 reader (``hdf5.File``: contiguous, compact and chunked datasets with the
deflate, shuffle and fletcher32 filters).  ``read_cat`` and ``read_subhalo``
take an optional ``device``: the data then goes to that CUDA device through
pinned host memory, a contiguous dataset being read from the file straight
into the pinned buffer.  Missing datasets in the first file of a
multi-file read raise KeyError; the reference prints the available names and
then fails on an unbound variable.
"""

from __future__ import annotations

import os

import numpy as np

from . import hdf5
from .output import HAVE_H5PY, norm_path, open_output
from .sim_info import SimInfo


class _Reader:
    """Dataset reads from one file, by h5py or by hdf5.File."""

    def __init__(self, path):
        self.path = path
        if HAVE_H5PY:
            import h5py
            self.f = h5py.File(path, "r")
        else:
            self.f = hdf5.File(path)

    def close(self):
        self.f.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def read(self, path, cut=None):
        if HAVE_H5PY:
            ds = self.f[norm_path(path)]
            return ds[:] if cut is None else ds[cut[0]:cut[1]]
        a = self.f.read(norm_path(path))
        return a if cut is None else a[cut[0]:cut[1]]

    def keys(self, group):
        if HAVE_H5PY:
            return list(self.f[norm_path(group)].keys())
        return self.f.keys(norm_path(group))

    def to_device(self, path, device, cut=None):
        """The dataset (rows cut[0]:cut[1]) as a tensor on ``device``, staged in
        pinned memory; a contiguous little-endian dataset is read from the file
        straight into the pinned buffer."""
        import torch
        ext = None if HAVE_H5PY else self.f.contiguous_extent(norm_path(path))
        if ext is not None and ext[2].byteorder in ("<", "=", "|") and np.little_endian and len(ext[3]) > 0:
            off, nbytes, dt, shape = ext
            rows = shape[0]
            r0, r1 = (0, rows) if cut is None else slice(cut[0], cut[1]).indices(rows)[:2]
            r1 = max(r0, r1)
            row_bytes = nbytes // rows if rows else 0
            host = torch.empty((r1 - r0) * row_bytes, dtype=torch.uint8, pin_memory=True)
            _pread_into(self.path, off + r0 * row_bytes, memoryview(host.numpy()))
            arr = host.numpy().view(dt.newbyteorder("=")).reshape((r1 - r0,) + tuple(shape[1:]))
            return torch.from_numpy(arr).to(device, non_blocking=True)
        a = np.ascontiguousarray(self.read(path, cut))
        return torch.from_numpy(a).pin_memory().to(device, non_blocking=True)


_PREAD_PART = 8 << 20


def _pread_into(path, offset, mv):
    """Fill ``mv`` from ``path`` at ``offset``; large ranges are read in
    parallel slices of 8 MB (the reads release the GIL)."""
    n = len(mv)
    fd = os.open(path, os.O_RDONLY)
    try:
        def part(a, b):
            while a < b:
                got = os.preadv(fd, [mv[a:b]], offset + a)
                if got <= 0:
                    raise OSError(f"short read of {path} at {offset + a}")
                a += got

        if n <= 2 * _PREAD_PART:
            part(0, n)
            return
        import concurrent.futures as cf
        cuts = list(range(0, n, _PREAD_PART)) + [n]
        with cf.ThreadPoolExecutor(max_workers=min(8, len(cuts) - 1)) as ex:
            list(ex.map(lambda ab: part(*ab), zip(cuts[:-1], cuts[1:])))
    finally:
        os.close(fd)


def _concat(parts, stack):
    out = parts[0]
    for p in parts[1:]:
        out = np.vstack((out, p)) if stack else np.append(out, p)
    return out


class ReadData(SimInfo):
    """Reads simulation catalogues and MeasureIA output files (the
    reference's ``ReadData``)."""

    def __init__(self, simulation, catalogue, snapshot, sub_group="", output_file_name=None, data_path="./data/raw/"):
        SimInfo.__init__(self, simulation, snapshot, boxsize=None, file_info=True)
        self.catalogue = catalogue
        self.sub_group = sub_group + "/"
        self.data_path = data_path + "/"
        self.output_file_name = output_file_name
        self.r = self.rp = None
        self.w_gg = self.w_gp = None
        self.multipoles_gg = self.multipoles_gp = None
        self.cov_multipoles_gg = self.errors_multipoles_gg = None
        self.cov_multipoles_gp = self.errors_multipoles_gp = None
        self.cov_w_gg = self.errors_w_gg = None
        self.cov_w_gp = self.errors_w_gp = None

    # ---- one catalogue file -------------------------------------------------
    def read_cat(self, dataset_name, cut=None, device=None):
        """``<snap_group><sub_group><dataset_name>`` of ``<catalogue>.hdf5``
        (rows ``cut[0]:cut[1]`` if given); on ``device`` when given."""
        if self.catalogue == "Subhalo":
            raise KeyError("Use read_subhalo method")
        elif self.catalogue == "Snapshot":
            raise KeyError("Use read_snapshot method")
        path = self.snap_group + self.sub_group + dataset_name
        with _Reader(f"{self.data_path}{self.catalogue}.hdf5") as f:
            if device is not None:
                return f.to_device(path, device, cut)
            return f.read(path, cut)

    # ---- multi-file group catalogues and snapshots --------------------------
    def _first(self, f, group, name, what):
        try:
            return f.read(f"{group}/{name}")
        except KeyError:
            raise KeyError(f"Variable not found in {what} files: {name}. Choose from {f.keys(group)}")

    def read_subhalo(self, dataset_name, Nfiles=0, device=None):
        """A group-catalogue dataset over the files ``<fof_folder>.<n>.hdf5``;
        files where it is missing are skipped (with a message)."""
        with _Reader(f"{self.data_path}{self.fof_folder}.0.hdf5") as f:
            data = self._first(f, self.catalogue, dataset_name, "Subhalo")
        stack = data.ndim > 1
        parts = [data]
        if Nfiles == 0:
            Nfiles = self.N_files
        for n in range(1, int(Nfiles)):
            try:
                with _Reader(f"{self.data_path}{self.fof_folder}.{n}.hdf5") as f:
                    parts.append(f.read(f"{self.catalogue}/{dataset_name}"))
            except KeyError:
                print("problem at file ", n)
        data = _concat(parts, stack)
        if device is not None:
            import torch
            return torch.from_numpy(np.ascontiguousarray(data)).pin_memory().to(device, non_blocking=True)
        return data

    def read_snapshot(self, dataset_name):
        """A snapshot dataset over the files ``<snap_folder>.<n>.hdf5``,
        returned, or written to ``output_file_name`` under the snapshot
        group when one is set."""
        print(dataset_name)
        with _Reader(f"{self.data_path}{self.snap_folder}.0.hdf5") as f:
            data = self._first(f, self.catalogue, dataset_name, "Snapshot")
        stack = data.ndim > 1
        parts = [data]
        for n in range(1, int(self.N_files)):
            try:
                with _Reader(f"{self.data_path}{self.snap_folder}.{n}.hdf5") as f:
                    parts.append(f.read(f"{self.catalogue}/{dataset_name}"))
            except KeyError:
                print("problem at file ", n)
        data = _concat(parts, stack)
        if self.output_file_name is not None:
            store = open_output(self.output_file_name)
            store.write(self.snap_group, dataset_name, data)
            store.flush()
            return None
        return data

    def read_snapshot_multiple(self, dataset_name):
        """Several snapshot datasets in one pass over the files.  With
        ``output_file_name`` each is written under the snapshot group; without
        it the reference's return value is kept: the last variable of the
        first file with every later file's variables appended in turn."""
        with _Reader(f"{self.data_path}{self.snap_folder}.0.hdf5") as f:
            first = [self._first(f, self.catalogue, v, "Snapshot") for v in dataset_name]
        stacks = [d.ndim > 1 for d in first]
        columns = [[d] for d in first]
        data = first[-1]
        for n in range(1, int(self.N_files)):
            try:
                with _Reader(f"{self.data_path}{self.snap_folder}.{n}.hdf5") as f:
                    for i, v in enumerate(dataset_name):
                        d = f.read(f"{self.catalogue}/{v}")
                        columns[i].append(d)
                        if self.output_file_name is None:
                            data = np.vstack((data, d)) if stacks[i] else np.append(data, d)
            except KeyError:
                print("problem at file ", n)
        if self.output_file_name is not None:
            store = open_output(self.output_file_name)
            for v, parts, st in zip(dataset_name, columns, stacks):
                store.write(self.snap_group, v, _concat(parts, st))
            store.flush()
            return None
        return data

    # ---- measurement results ------------------------------------------------
    def read_MeasureIA_output(self, dataset_name, num_jk):
        """w_gg, w_g+, multipoles and (with num_jk) their jackknife errors and
        covariances from ``<catalogue>.hdf5``, into the attributes the
        reference sets; products missing from the file stay None."""
        for a in ("r", "rp", "w_gg", "w_gp", "multipoles_gg", "multipoles_gp", "cov_multipoles_gg",
                  "errors_multipoles_gg", "cov_multipoles_gp", "errors_multipoles_gp", "cov_w_gg", "errors_w_gg",
                  "cov_w_gp", "errors_w_gp"):
            setattr(self, a, None)
        path = f"{self.data_path}{self.catalogue}.hdf5"
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        with _Reader(path) as f:
            g = self.snap_group
            if g and norm_path(g) not in f.keys(""):
                raise KeyError(f"Unable to open object '{norm_path(g)}' in {path}")
            for grp, val, sep_attr, sep, cov, err in (
                    ("multipoles_gg", "multipoles_gg", "r", "_r", "cov_multipoles_gg", "errors_multipoles_gg"),
                    ("multipoles_g_plus", "multipoles_gp", "r", "_r", "cov_multipoles_gp", "errors_multipoles_gp"),
                    ("w_gg", "w_gg", "rp", "_rp", "cov_w_gg", "errors_w_gg"),
                    ("w_g_plus", "w_gp", "rp", "_rp", "cov_w_gp", "errors_w_gp")):
                # attributes are set as they are read: a missing covariance keeps the values before it
                try:
                    setattr(self, val, f.read(f"{g}{grp}/{dataset_name}"))
                    setattr(self, sep_attr, f.read(f"{g}{grp}/{dataset_name}{sep}"))
                    if num_jk is not None:
                        setattr(self, cov, f.read(f"{g}{grp}/{dataset_name}_jackknife_cov_{num_jk}"))
                        setattr(self, err, f.read(f"{g}{grp}/{dataset_name}_jackknife_{num_jk}"))
                except KeyError:
                    pass
