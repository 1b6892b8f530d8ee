"""ReadData (catalogue and result ingestion) on files laid out as the
reference expects them: multi-file group catalogues and snapshots (some
files chunked and compressed), catalogue files with snapshot and sub groups,
and MeasureIA output files (the reference's golden outputs, rewritten from
their fixture, and the golden HDF5 file itself where it exists)."""

import os

import numpy as np
import pytest

from measure_ia_gb300 import hdf5
from measure_ia_gb300.read_data import ReadData
from golden_io import reference_file

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN_H5 = reference_file("tests/data/processed/TNG300/mock_IA_TNG300.hdf5")


def _multi(tmp_path, stem, group, per_file, chunked=(1,), missing=()):
    """Files <stem>.<n>.hdf5 with group/<name> datasets; file n of `missing`
    lacks them."""
    os.makedirs(os.path.dirname(str(tmp_path) + stem), exist_ok=True)
    for n, arrays in enumerate(per_file):
        d = {"Header/n": np.array([n])}
        if n not in missing:
            d.update({f"{group}/{k}": v for k, v in arrays.items()})
        hdf5.write_file(f"{tmp_path}{stem}.{n}.hdf5", d, chunks=16 if n in chunked else None)


def test_read_subhalo_concatenates_files(tmp_path, capsys):
    rng = np.random.default_rng(0)
    files = [{"SubhaloPos": rng.normal(size=(m, 3)), "SubhaloMass": rng.normal(size=m)} for m in (40, 25, 33, 50)]
    rd = ReadData("TNG300", "Subhalo", 99, data_path=str(tmp_path))
    _multi(tmp_path, rd.fof_folder, "Subhalo", files, chunked=(1, 3), missing=(2,))
    pos = rd.read_subhalo("SubhaloPos", Nfiles=4)
    np.testing.assert_array_equal(pos, np.vstack([files[0]["SubhaloPos"], files[1]["SubhaloPos"],
                                                  files[3]["SubhaloPos"]]))
    assert "problem at file  2" in capsys.readouterr().out
    mass = rd.read_subhalo("SubhaloMass", Nfiles=2)
    np.testing.assert_array_equal(mass, np.append(files[0]["SubhaloMass"], files[1]["SubhaloMass"]))
    with pytest.raises(KeyError, match="Choose from"):
        rd.read_subhalo("Nothing", Nfiles=2)
    with pytest.raises(OSError):           # a file that is not there fails, as in the reference
        rd.read_subhalo("SubhaloMass", Nfiles=6)


def test_read_snapshot_and_output(tmp_path):
    rng = np.random.default_rng(1)
    files = [{"Coordinates": rng.uniform(0, 205, (m, 3)), "Masses": rng.uniform(1, 2, m)} for m in (30, 20, 10)]
    rd = ReadData("TNG300", "PartType4", 99, data_path=str(tmp_path))
    rd.N_files = 3
    _multi(tmp_path, rd.snap_folder, "PartType4", files, chunked=(0,))
    want = np.vstack([f["Coordinates"] for f in files])
    np.testing.assert_array_equal(rd.read_snapshot("Coordinates"), want)
    out = str(tmp_path / "snap_out.hdf5")
    rd2 = ReadData("TNG300", "PartType4", 99, data_path=str(tmp_path), output_file_name=out)
    rd2.N_files = 3
    assert rd2.read_snapshot("Coordinates") is None
    assert rd2.read_snapshot_multiple(["Coordinates", "Masses"]) is None
    got = hdf5.read_file(out)
    np.testing.assert_array_equal(got["Snapshot_99/Coordinates"], want)
    np.testing.assert_array_equal(got["Snapshot_99/Masses"], np.concatenate([f["Masses"] for f in files]))
    # without an output file the reference returns its running array: the last variable of
    # file 0, then every later file's variables appended in order
    rd.N_files = 3
    for f in files:
        f["Ages"] = rng.uniform(size=len(f["Masses"]))
    _multi(tmp_path, rd.snap_folder, "PartType4", files, chunked=(0,))
    got = rd.read_snapshot_multiple(["Masses", "Ages"])
    want = files[0]["Ages"]
    for f in files[1:]:
        want = np.append(np.append(want, f["Masses"]), f["Ages"])
    np.testing.assert_array_equal(got, want)
    with pytest.raises(ValueError):      # 1-D then 2-D variables: the reference's vstack fails too
        rd.read_snapshot_multiple(["Masses", "Coordinates"])


def test_read_cat(tmp_path):
    rng = np.random.default_rng(2)
    a = rng.normal(size=(100, 3))
    hdf5.write_file(str(tmp_path / "galaxies.hdf5"), {"Snapshot_99/Centrals/Position": a})
    rd = ReadData("TNG300", "galaxies", 99, sub_group="Centrals", data_path=str(tmp_path))
    np.testing.assert_array_equal(rd.read_cat("Position"), a)
    np.testing.assert_array_equal(rd.read_cat("Position", cut=[10, 20]), a[10:20])
    for cat in ("Subhalo", "Snapshot"):
        with pytest.raises(KeyError):
            ReadData("TNG300", cat, 99, data_path=str(tmp_path)).read_cat("Position")


def _golden_outputs():
    z = np.load(os.path.join(HERE, "golden", "tng300_mock_outputs.npz"))
    return {k[len("small/"):]: z[k] for k in z.files if k.startswith("small/")}


def test_read_measureia_output(tmp_path):
    out = _golden_outputs()
    hdf5.write_file(str(tmp_path / "mock.hdf5"), out)
    rd = ReadData("TNG300", "mock", 99, data_path=str(tmp_path))
    rd.read_MeasureIA_output("All", 8)
    g = "Snapshot_99"
    np.testing.assert_array_equal(rd.w_gg, out[f"{g}/w_gg/All"])
    np.testing.assert_array_equal(rd.rp, out[f"{g}/w_g_plus/All_rp"])
    np.testing.assert_array_equal(rd.cov_w_gp, out[f"{g}/w_g_plus/All_jackknife_cov_8"])
    np.testing.assert_array_equal(rd.errors_multipoles_gg, out[f"{g}/multipoles_gg/All_jackknife_8"])
    np.testing.assert_array_equal(rd.multipoles_gp, out[f"{g}/multipoles_g_plus/All"])
    rd.read_MeasureIA_output("All", None)          # no jackknife: values only
    assert rd.cov_w_gg is None and rd.w_gg is not None
    rd.read_MeasureIA_output("Nothing", 8)          # absent products stay None
    assert rd.w_gg is None and rd.multipoles_gp is None
    with pytest.raises(KeyError):
        ReadData("TNG300", "mock", 50, data_path=str(tmp_path)).read_MeasureIA_output("All", 8)


@pytest.mark.skipif(GOLDEN_H5 is None, reason="MIA_REFERENCE_ROOT unset or without the golden file")
def test_read_measureia_output_h5py_file():
    out = _golden_outputs()
    rd = ReadData("TNG300", "mock_IA_TNG300", 99, data_path=os.path.dirname(GOLDEN_H5))
    rd.read_MeasureIA_output("high", 8)
    np.testing.assert_array_equal(rd.w_gp, out["Snapshot_99/w_g_plus/high"])
    np.testing.assert_array_equal(rd.cov_multipoles_gp, out["Snapshot_99/multipoles_g_plus/high_jackknife_cov_8"])


@pytest.mark.gpu
def test_read_to_device(tmp_path):
    import torch
    rng = np.random.default_rng(3)
    a = rng.normal(size=(1000, 3))
    hdf5.write_file(str(tmp_path / "cat.hdf5"), {"Position": a, "Weight": rng.uniform(size=1000)})
    rd = ReadData("TNG300", "cat", None, data_path=str(tmp_path))
    t = rd.read_cat("Position", device="cuda")
    torch.cuda.synchronize()
    assert t.is_cuda and t.dtype == torch.float64
    np.testing.assert_array_equal(t.cpu().numpy(), a)
    np.testing.assert_array_equal(rd.read_cat("Position", cut=[100, 250], device="cuda").cpu().numpy(), a[100:250])
