"""The built-in HDF5 writer and reader (hosts without h5py).

No HDF5 library exists on these hosts, so the writer is checked three ways:
its files read back through the package's reader and through the
independent reader in ``tests/golden/h5read.py`` (written against h5py's
files); a dataset's object-header messages are byte-for-byte those h5py
wrote for the same array in the reference's golden output file (values
below, read from ``mock_IA_TNG300.hdf5``: Snapshot_99/w_gg/low_rp and
low_jackknife_cov_8); and the structures sit where h5py puts them.
"""

import os
import struct
import sys

import numpy as np
import pytest

from measure_ia_gb300 import hdf5
from measure_ia_gb300.output import OutputFile
from golden_io import reference_file

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import h5read  # noqa: E402

# h5py's messages for a (10,) and a (10, 10) float64 dataset, without the
# storage address: (type, flags, body)
H5PY_1D = [(0x1, 0, "01010100000000000a000000000000000a00000000000000"),
           (0x3, 1, "11203f000800000000004000340b0034ff03000000000000"),
           (0x5, 1, "0202020100000000")]
H5PY_2D_SPACE = "01020100000000000a000000000000000a000000000000000a000000000000000a00000000000000"
GOLDEN_H5 = reference_file("tests/data/processed/TNG300/mock_IA_TNG300.hdf5")


def _sample(rng):
    d = {"Snapshot_99/w/xi_gg/a": rng.normal(size=(10, 8)),
         "Snapshot_99/w/xi_gg/a_DD": rng.normal(size=(10, 8)),
         "top": np.arange(5, dtype=np.int64), "f32": rng.normal(size=3).astype(np.float32),
         "u8": np.arange(4, dtype=np.uint8), "i32": -np.arange(6, dtype=np.int32).reshape(2, 3),
         "scalar": np.float64(3.5), "empty": np.zeros((0, 3)), "big_endian": np.arange(3, dtype=">f8")}
    for i in range(300):            # 38 symbol-table nodes: a two-level B-tree
        d[f"w_g_plus/s_jk125/s_{i}_SplusD"] = rng.normal(size=(4,))
    return d


def _messages(b, addr):
    n, = struct.unpack_from("<H", b, addr + 2)
    out, p = [], addr + 16
    for _ in range(n):
        t, s, f = struct.unpack_from("<HHB", b, p)
        out.append((t, f, b[p + 8:p + 8 + s]))
        p += 8 + s
    return out


def test_round_trip_through_both_readers(tmp_path):
    d = _sample(np.random.default_rng(0))
    path = str(tmp_path / "rt.hdf5")
    hdf5.write_file(path, d)
    a, b = hdf5.read_file(path), h5read.read_all(path)
    assert set(a) == set(b) == set(d)
    for k, v in d.items():
        v = np.asarray(v)
        assert a[k].shape == v.shape and a[k].dtype == v.dtype.newbyteorder("="), k
        np.testing.assert_array_equal(a[k], v)
        np.testing.assert_array_equal(b[k], v)


def test_repeated_layout_reuses_image(tmp_path):
    """A second write of the same paths, shapes and types reuses the first
    file's image with the new data placed in it: the bytes equal a fresh
    write of the new values; a changed shape or type writes afresh."""
    rng = np.random.default_rng(5)
    d1 = _sample(rng)
    d2 = {k: (np.asarray(v) + 1).astype(np.asarray(v).dtype) for k, v in d1.items()}
    p1, p2 = str(tmp_path / "one.hdf5"), str(tmp_path / "two.hdf5")
    hdf5._IMAGES.clear()
    hdf5.write_file(p1, d1)
    assert len(hdf5._IMAGES) == 1
    hdf5.write_file(p2, d2)                                   # layout hit
    assert len(hdf5._IMAGES) == 1
    hdf5._IMAGES.clear()
    fresh = str(tmp_path / "fresh.hdf5")
    hdf5.write_file(fresh, d2)
    assert open(p2, "rb").read() == open(fresh, "rb").read()
    got = hdf5.read_file(p2)
    for k, v in d2.items():
        np.testing.assert_array_equal(got[k], v)
    d3 = dict(d2, top=np.arange(6, dtype=np.int64))           # another shape
    d4 = dict(d2, top=np.arange(5, dtype=np.int32))           # another type
    for d in (d3, d4):
        hdf5.write_file(p2, d)
        got = hdf5.read_file(p2)
        assert got["top"].shape == d["top"].shape and got["top"].dtype == d["top"].dtype
        np.testing.assert_array_equal(got["top"], d["top"])
    assert len(hdf5._IMAGES) == 3


def test_layout_matches_h5py(tmp_path):
    rng = np.random.default_rng(1)
    path = str(tmp_path / "h.hdf5")
    hdf5.write_file(path, {"Snapshot_99/w_gg/low_rp": rng.normal(size=10),
                           "Snapshot_99/w_gg/low_jackknife_cov_8": rng.normal(size=(10, 10))})
    b = open(path, "rb").read()
    # superblock: version 0, 8-byte offsets and lengths, K = 4 / 16, EOF = file size
    assert b[:8] == hdf5.SIGNATURE and b[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])
    assert struct.unpack_from("<HHI", b, 16) == (4, 16, 0)
    base, free, eof, drv = struct.unpack_from("<QQQQ", b, 24)
    assert (base, free, eof, drv) == (0, hdf5.UNDEF, len(b), hdf5.UNDEF)
    _, root, cache, _, bt, hp = struct.unpack_from("<QQIIQQ", b, 56)
    assert cache == 1
    assert b[bt:bt + 4] == b"TREE" and b[hp:hp + 4] == b"HEAP"
    # local heap: "" at offset 0 and a free list ending in 1
    size, free_at, seg = struct.unpack_from("<QQQ", b, hp + 8)
    assert b[seg:seg + 8] == b"\0" * 8 and free_at < size
    assert struct.unpack_from("<Q", b, seg + free_at)[0] == hdf5.FREE_NULL
    r = hdf5._Reader(b)
    grp = r.members(bt, hp)["Snapshot_99"]
    (t, _, body), = _messages(b, grp)
    gbt, ghp = struct.unpack_from("<QQ", body)
    sub = r.members(gbt, ghp)["w_gg"]
    (_, _, body), = _messages(b, sub)
    members = r.members(*struct.unpack_from("<QQ", body))
    m1 = _messages(b, members["low_rp"])
    assert [(t, f, body.hex()) for t, f, body in m1[:3]] == H5PY_1D
    t, f, lay = m1[3]
    assert (t, f, lay[:2].hex(), struct.unpack_from("<Q", lay, 10)[0]) == (0x8, 0, "0301", 80)
    m2 = _messages(b, members["low_jackknife_cov_8"])
    assert m2[0][2].hex() == H5PY_2D_SPACE and struct.unpack_from("<Q", m2[3][2], 10)[0] == 800


def test_store_appends_and_replaces(tmp_path):
    path = str(tmp_path / "out.hdf5")
    a = OutputFile(path, use_h5py=False)
    a.write("Snapshot_99/w/xi_gg", "d_DD", np.ones((2, 3)))
    a.write("Snapshot_99/w/xi_gg", "d_rp", np.arange(2.0))
    a.flush()
    b = OutputFile(path, use_h5py=False)          # another process, same file
    b.write("Snapshot_99/w/xi_gg/", "d_DD", np.zeros((2, 3)))
    b.write("Snapshot_99/w_gg", "d", np.arange(3.0))
    b.flush()
    got = hdf5.read_file(path)
    assert set(got) == {"Snapshot_99/w/xi_gg/d_DD", "Snapshot_99/w/xi_gg/d_rp", "Snapshot_99/w_gg/d"}
    np.testing.assert_array_equal(got["Snapshot_99/w/xi_gg/d_DD"], np.zeros((2, 3)))
    np.testing.assert_array_equal(got["Snapshot_99/w/xi_gg/d_rp"], np.arange(2.0))


@pytest.mark.parametrize("parts,want", [
    (("Snapshot_99//w/xi_gg/",), "Snapshot_99/w/xi_gg"),
    (("Snapshot_99", "w/xi_gg"), "Snapshot_99/w/xi_gg"),
    (("", "w", "x"), "w/x"),
    (("/a/", "/b/"), "a/b"),
    (("a", ""), "a"),
    (("", ""), ""),
    (("a/b", "c_0_rp"), "a/b/c_0_rp"),
    ((99, "w"), "99/w")])
def test_paths_normalise_as_hdf5_resolves_them(parts, want):
    """Empty components drop out, as HDF5 resolves 'a//b/' to 'a/b'."""
    from measure_ia_gb300.output import norm_path
    assert norm_path(*parts) == want


def test_store_refuses_an_unreadable_file(tmp_path):
    path = str(tmp_path / "notes.hdf5")
    with open(path, "wb") as f:
        f.write(b"not an hdf5 file")
    s = OutputFile(path, use_h5py=False)
    with pytest.raises(RuntimeError):
        s.write("w", "d", np.ones(2))
    assert open(path, "rb").read() == b"not an hdf5 file"


def test_writer_rejects_what_it_cannot_store(tmp_path):
    with pytest.raises(TypeError):
        hdf5.write_file(str(tmp_path / "b.hdf5"), {"m": np.ones(3, dtype=bool)})
    with pytest.raises(ValueError):
        hdf5.write_file(str(tmp_path / "c.hdf5"), {"a": np.ones(2), "a/b": np.ones(2)})
    assert not os.path.exists(str(tmp_path / "b.hdf5"))


@pytest.mark.skipif(GOLDEN_H5 is None, reason="MIA_REFERENCE_ROOT unset or without the golden file")
def test_reader_on_h5py_files():
    x, y = hdf5.read_file(GOLDEN_H5), h5read.read_all(GOLDEN_H5)
    assert set(x) == set(y) and len(x) > 700
    for k in x:
        np.testing.assert_array_equal(x[k], y[k])
