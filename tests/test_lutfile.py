"""Optics look-up-table files (dointegration.createNCDF layout, the
hydrophobic conversion, the band file) written without the netCDF library.

Files are read back with scipy.io.netcdf_file, an independent reader of the
classic format, and compared with the reference's own outputs: the variables
dointegration.fun wrote (tests/golden/table_*.npz) and hydrophobic.
doConversion's results on those tables (tests/golden/hydrophobic.npz).
"""
import json
import os

import numpy as np
import pytest
import scipy.io

from conftest import load_golden
from geosmie_gb300 import lutfile, ncfile

NAMES = ["rh", "wavelength", "bin", "p", "ang"] + [k for k, _ in lutfile.VAR_TYPES]


def _golden_table(name):
    g = load_golden("table_%s.npz" % name)
    return {k[4:]: g[k] for k in g.files if k.startswith("out_")}


def test_optics_file_matches_reference_layout_cpu(tmp_path):
    t = _golden_table("lognorm")
    path = str(tmp_path / "optics_lognorm.nomom.nc4")
    lutfile.write_optics(path, t, t["rh"], t["wavelength"], t["ang"])
    f = scipy.io.netcdf_file(path, "r", mmap=False)
    assert list(f.dimensions) == ["rh", "wavelength", "bin", "p", "ang"]
    assert list(f.variables) == NAMES
    for k in NAMES:
        v = f.variables[k]
        np.testing.assert_array_equal(v.data, t[k], err_msg=k)
        ln, un = lutfile.VARDICT[k]
        assert v.long_name.decode() == ln and v.units.decode() == un, k
    assert f.variables["p11"].dimensions == ("bin", "wavelength", "rh", "ang")
    assert f.variables["pback"].dimensions == ("bin", "wavelength", "rh", "p")
    assert f.variables["rEff"].dimensions == ("bin", "rh")
    f.close()


def test_optics_file_legacy_and_cdf5_cpu(tmp_path):
    t = _golden_table("trivial")
    path = str(tmp_path / "legacy.nc4")
    lutfile.write_optics(path, t, t["rh"], t["wavelength"], t["ang"], oppclassic=True)
    f = scipy.io.netcdf_file(path, "r", mmap=False)
    assert list(f.dimensions) == ["rh", "lambda", "radius", "nPol", "ang"]
    assert f.variables["p11"].dimensions == ("radius", "rh", "lambda", "ang")
    np.testing.assert_array_equal(f.variables["p11"].data, t["p11"].transpose(0, 2, 1, 3))
    np.testing.assert_array_equal(f.variables["qext"].data, t["qext"].transpose(0, 2, 1))
    assert f.variables["pback"].dimensions == ("nPol", "radius", "rh", "lambda")
    np.testing.assert_array_equal(f.variables["pback"].data, t["pback"].transpose(3, 0, 2, 1))
    f.close()
    path5 = str(tmp_path / "cdf5.nc4")
    lutfile.write_optics(path5, t, t["rh"], t["wavelength"], t["ang"], version=5)
    data, dims, _ = lutfile.read(path5)
    assert data["bin"].dtype == np.int64 and list(data["p"]) == [11, 12, 33, 34, 22, 44]
    for k in NAMES[5:]:
        np.testing.assert_array_equal(data[k], t[k])


@pytest.mark.parametrize("legacy", [False, True])
def test_hydrophobic_matches_reference_cpu(tmp_path, legacy):
    h = load_golden("hydrophobic.npz")
    for name in ("trivial", "seasalt"):
        t = _golden_table(name)
        tag = "%s_%s" % (name, "legacy" if legacy else "new")
        src = str(tmp_path / ("in_%s.nc4" % tag))
        lutfile.write_optics(src, t, t["rh"], t["wavelength"], t["ang"], oppclassic=legacy)
        lutfile.doConversion(os.path.basename(src), "out_%s.nc4" % tag, str(tmp_path), legacy)
        f = scipy.io.netcdf_file(str(tmp_path / ("out_%s.nc4" % tag)), "r", mmap=False)
        rad = "radius" if legacy else "bin"
        assert f.dimensions[rad] == 2
        for k in NAMES:
            kk = {"wavelength": "lambda", "bin": "radius", "p": "nPol"}.get(k, k) if legacy else k
            np.testing.assert_array_equal(f.variables[kk].data, h["%s__%s" % (tag, kk)], err_msg=(tag, kk))
        f.close()
    # a two-bin file is copied unchanged, as in the reference
    t = _golden_table("lognorm")
    dims, variables = lutfile.optics_file(t, t["rh"], t["wavelength"], t["ang"], legacy)
    d2, v2 = lutfile.hydrophobic(dims, variables, legacy)
    assert d2 == dims and all(a[3] is b[3] for a, b in zip(variables, v2))


def test_band_file_cpu(tmp_path):
    from oracle import bands as obands
    d = load_golden("bands.npz")
    data = {k[3:]: d[k] for k in d.files if k.startswith("in_")}
    out = obands.fun(data, "su", "RRTMG")
    path = str(tmp_path / "bands.nc4")
    lutfile.write_bands(path, out)
    f = scipy.io.netcdf_file(path, "r", mmap=False)
    for k in obands.VARS + ["wavelength", "rh", "bandLow", "bandUp", "rEff", "rMass"]:
        np.testing.assert_array_equal(f.variables[k].data, np.asarray(out[k]), err_msg=k)
    q = [b"".join(r).decode().rstrip("\0") for r in f.variables["qname"].data]
    assert q == out["qname"]
    assert f.variables["bandLow"].units.decode() == "micrometers"
    f.close()


def test_ncfile_rejects_int64_in_classic_cpu(tmp_path):
    with pytest.raises(ValueError):
        ncfile.write(str(tmp_path / "x.nc"), [("n", 2)], [("u", "u8", ("n",), np.arange(2), {})], version=2)
    with pytest.raises(ValueError):
        ncfile.read(__file__)


@pytest.mark.gpu
def test_optics_file_from_gpu_table_gpu(tmp_path):
    """dointegration.fun end to end: the GPU table of a reference particle
    definition written as its optics file, against the reference's file."""
    from geosmie_gb300 import table
    g = load_golden("table_lognorm.npz")
    params = json.loads(str(g["params_json"]))
    got = table.run_table(params, list(g["mlist"]), g["waterm"])
    path = str(tmp_path / lutfile.optics_filename("lognorm.json"))
    lutfile.write_optics(path, got, g["out_rh"], g["out_wavelength"], g["out_ang"])
    f = scipy.io.netcdf_file(path, "r", mmap=False)
    p11 = np.abs(g["out_p11"])
    for k in ["p11", "p12", "p22", "p33", "p34", "p44"]:
        assert np.max(np.abs(f.variables[k].data - g["out_" + k]) / p11) < 1e-9, k
    for k in ["qext", "qsca", "g"]:
        r = g["out_" + k]
        assert np.max(np.abs(f.variables[k].data - r) / np.abs(r)) < 1e-10, k
    np.testing.assert_array_equal(f.variables["bin"].data, g["out_bin"])
    f.close()
