"""Optics look-up-table files: the NetCDF side of dointegration and its
post-processors, written with ``ncfile`` (no netCDF library).

  optics_file / write_optics   dointegration.createNCDF (:205-422) and the
                               per-entry writes of fun (:1003-1036): the
                               dimensions rh, wavelength|lambda, bin|radius,
                               p|nPol (6), ang; the coordinate variables; the
                               30 table variables with their long_name and
                               units, in the reference's order, non-legacy
                               (bin, wavelength, rh, ...) or legacy (radius,
                               rh, lambda, ...; pback (nPol, radius, rh,
                               lambda)) layout
  hydrophobic / doConversion   hydrophobic.doConversion (:18-124): a second
                               radius index whose first entry holds the RH = 0
                               values of the (one-bin) hydrophilic table at
                               every RH
  write_bands                  the band file of bandaverage.fun (:223-290)

Integer index variables ('bin', 'p') are int64 in the reference's NETCDF4
files; the default classic version 2 here stores them as 32-bit integers
(version=5 keeps int64).  The reference's zlib compression is a NETCDF4
storage option with no classic equivalent.
"""
import os

import numpy as np

from . import ncfile

# (long_name, units) of every variable (createNCDF :223-335)
VARDICT = {
    "bin": ("radius bin index (1-indexed)", "dimensionless"),
    "p": ("Scattering matrix element index, ordered as P11, P12, P33, P34, P22, P44", "dimensionless"),
    "rh": ("relative humidity", "fraction"),
    "wavelength": ("wavelength", "m"),
    "ang": ("scattering angle", "degrees"),
    "p11": ("P11 element of the normalized scattering matrix", "dimensionless"),
    "p12": ("P12 element of the normalized scattering matrix", "dimensionless"),
    "p22": ("P22 element of the normalized scattering matrix", "dimensionless"),
    "p33": ("P33 element of the normalized scattering matrix", "dimensionless"),
    "p34": ("P34 element of the normalized scattering matrix", "dimensionless"),
    "p44": ("P44 element of the normalized scattering matrix", "dimensionless"),
    "qsca": ("scattering efficiency", "dimensionless"),
    "qabs": ("absorption efficiency", "dimensionless"),
    "qext": ("extinction efficiency", "dimensionless"),
    "g": ("asymmetry factor", "dimensionless"),
    "ssa": ("single-scattering albedo", "dimensionless"),
    "bsca": ("mass scattering efficiency", "m2 (kg dry mass)-1"),
    "bext": ("mass extinction efficiency", "m2 (kg dry mass)-1"),
    "csca": ("mass scattering cross-section", "m2"),
    "cext": ("mass extinction cross-section", "m2"),
    "bbck": ("mass backscatter efficiency", "m2 (kg dry mass)-1 sr-1"),
    "lidar_ratio": ("lidar ratio", ""),
    "mass": ("particle mass", "kg"),
    "volume": ("particle volume per kg dry mass", "m3 kg-1"),
    "area": ("particle cross sectional area per kg dry mass", "m2 kg-1"),
    "rEff": ("effective radius of bin", "m"),
    "rMass": ("effective mass of wet particle", "kg"),
    "rUp": ("upper edge of radius bin", "m"),
    "rLow": ("lower edge of radius bin", "m"),
    "pback": ("phase function in backscatter direction, ordered as P11, P12, P33, P34, P22, P44", "dimensionless"),
    "qb": ("backscattering efficiency", "dimensionless"),
    "rhop": ("wet particle density", "kg m-3"),
    "growth_factor": ("growth factor = ratio of wet to dry particle radius", "fraction"),
    "refreal": ("real refractive index of wet particle", "dimensionless"),
    "refimag": ("imaginary refractive index of wet particle", "dimensionless"),
}

# variable -> dimension type, in the order the reference creates them (:372-405)
VAR_TYPES = [("p11", "fun"), ("p12", "fun"), ("p22", "fun"), ("p33", "fun"), ("p34", "fun"), ("p44", "fun"),
             ("qsca", "scalar"), ("qabs", "scalar"), ("qext", "scalar"), ("g", "scalar"), ("ssa", "scalar"),
             ("qb", "scalar"), ("bsca", "scalar"), ("bext", "scalar"), ("csca", "scalar"), ("cext", "scalar"),
             ("bbck", "scalar"), ("lidar_ratio", "scalar"), ("mass", "nolambda"), ("volume", "nolambda"),
             ("area", "nolambda"), ("rEff", "nolambda"), ("rMass", "nolambda"), ("rUp", "nolambda"),
             ("rLow", "nolambda"), ("pback", "element"), ("rhop", "nolambda"), ("growth_factor", "nolambda"),
             ("refreal", "scalar"), ("refimag", "scalar")]
NPOL = [11, 12, 33, 34, 22, 44]


def _names(oppclassic):
    return ("radius", "lambda", "nPol") if oppclassic else ("bin", "wavelength", "p")


def optics_file(table, rh, lambdas, ang, oppclassic=False):
    """(dims, variables) of the optics file of a table dict in the
    non-legacy layout (as table.run_table returns it)."""
    rad, lam, npol = _names(oppclassic)
    nbin = np.asarray(table["qext"]).shape[0]
    dims = [("rh", len(rh)), (lam, len(lambdas)), (rad, nbin), (npol, 6), ("ang", len(ang))]
    if oppclassic:
        dtypes = {"scalar": (rad, "rh", lam), "nolambda": (rad, "rh"), "fun": (rad, "rh", lam, "ang"),
                  "element": (npol, rad, "rh", lam)}
    else:
        dtypes = {"scalar": (rad, lam, "rh"), "nolambda": (rad, "rh"), "fun": (rad, lam, "rh", "ang"),
                  "element": (rad, lam, "rh", "p")}

    def attrs(key):
        ln, un = VARDICT[key]
        return {"long_name": ln, "units": un}
    variables = [("rh", "f8", ("rh",), np.asarray(rh, np.float64), attrs("rh")),
                 (lam, "f8", (lam,), np.asarray(lambdas, np.float64), attrs("wavelength")),
                 (rad, "i8", (rad,), np.arange(1, nbin + 1), attrs("bin")),
                 (npol, "i8", (npol,), np.array(NPOL), attrs("p")),
                 ("ang", "f8", ("ang",), np.asarray(ang, np.float64), attrs("ang"))]
    for key, dt in VAR_TYPES:
        a = np.asarray(table[key], np.float64)
        if oppclassic:   # legacy writes (:1007-1015)
            if dt == "fun":
                a = a.transpose(0, 2, 1, 3)
            elif dt == "scalar":
                a = a.transpose(0, 2, 1)
            elif dt == "element":
                a = a.transpose(3, 0, 2, 1)
        variables.append((key, "f8", dtypes[dt], a, attrs(key)))
    return dims, variables


def optics_filename(partID0, oppclassic=False):
    """optics_<id>.nomom.nc4 (legacy: .nomom.legacy.nc4), fun :674-679."""
    part = partID0.split("/")[-1].replace(".json", "")
    return "optics_%s.nomom.legacy.nc4" % part if oppclassic else "optics_%s.nomom.nc4" % part


def write_optics(path, table, rh, lambdas, ang, oppclassic=False, version=2):
    dims, variables = optics_file(table, rh, lambdas, ang, oppclassic)
    ncfile.write(path, dims, variables, version=version)
    return path


def read(path):
    """{name: array} and {name: dims} of a file (text variables as bytes)."""
    dims, variables, _ = ncfile.read(path)
    return {k: v[2] for k, v in variables.items()}, {k: v[0] for k, v in variables.items()}, dims


def hydrophobic(dims, variables, oppclassic=False):
    """doConversion (:18-124) on (dims, variables) of a file: the radius
    dimension becomes 2; index 0 holds the first bin's RH = 0 values at every
    RH (hydrophobic), index 1 the first bin's values (hydrophilic)."""
    rad = "radius" if oppclassic else "bin"
    if dict(dims).get(rad) == 2:   # shapes unchanged: the reference copies every variable
        return list(dims), list(variables)
    new_dims = [(n, 2 if n == rad else s) for n, s in dims]
    out = []
    for name, code, vdims, data, attrs in variables:
        a = np.asarray(data)
        if rad not in vdims:
            out.append((name, code, vdims, a, attrs))
            continue
        shape = tuple(2 if d == rad else a.shape[i] for i, d in enumerate(vdims))
        b = np.zeros(shape, dtype=a.dtype)
        if a.ndim == 1:
            if name == rad:
                b[:] = [1, 2]
            else:
                b[:] = a[0]
        elif a.ndim == 2:   # (radius, rh)
            b[0, :] = a[0, 0]
            b[1, :] = a[0, :]
        elif a.ndim == 3:
            if oppclassic:   # (radius, rh, lambda)
                b[0] = a[0, 0][None, :]
                b[1] = a[0]
            else:            # (bin, wavelength, rh)
                b[0] = a[0, :, 0][:, None]
                b[1] = a[0]
        elif a.ndim == 4:
            if a.shape[0] == 6 and vdims[0] != rad:   # legacy pback (nPol, radius, rh, lambda)
                b[:, 0] = a[:, 0, 0][:, None, :]
                b[:, 1] = a[:, 0]
            elif oppclassic:   # (radius, rh, lambda, ang)
                b[0] = a[0, 0][None]
                b[1] = a[0]
            else:              # (bin, wavelength, rh, ang|p)
                b[0] = a[0, :, 0][:, None, :]
                b[1] = a[0]
        else:
            raise ValueError("unhandled number of dimensions for %s" % name)
        out.append((name, code, vdims, b, attrs))
    return new_dims, out


def doConversion(infn, outfn, pfx, oppclassic, version=2):
    """hydrophobic.doConversion: read pfx/infn, write pfx/outfn."""
    dims, variables, gattrs = ncfile.read(os.path.join(pfx, infn))
    codes = {"f": "f8", "i": "i8", "S": "c"}
    vlist = [(k, codes[v[2].dtype.kind] if v[2].dtype.kind != "f" or v[2].dtype.itemsize == 8 else "f4",
              v[0], v[2], v[1]) for k, v in variables.items()]
    new_dims, new_vars = hydrophobic(list(dims.items()), vlist, oppclassic)
    ncfile.write(os.path.join(pfx, outfn), new_dims, new_vars, gattrs=gattrs, version=version)


def write_bands(path, out, oppclassic=False, version=2):
    """The band file of bandaverage.fun (:223-290) from bands.fun's dict:
    dimensions rh, wavelength|lambda, bin|radius, nchar (80)."""
    rad, lam = ("radius", "lambda") if oppclassic else ("bin", "wavelength")
    nbin, nband, nrh = np.asarray(out["qext"]).shape
    dims = [("rh", nrh), (lam, nband), (rad, nbin), ("nchar", 80)]
    variables = []
    for k in ["qsca", "qext", "bsca", "bext", "g", "bbck", "refreal", "refimag"]:
        a = np.asarray(out[k], np.float64)
        if oppclassic:
            variables.append((k, "f8", (rad, "rh", lam), a.transpose(0, 2, 1), {}))
        else:
            variables.append((k, "f8", (rad, lam, "rh"), a, {}))
    variables += [(lam, "f8", (lam,), out["wavelength"], {}), ("rh", "f8", ("rh",), out["rh"], {}),
                  ("qname", "c", (rad, "nchar"), out["qname"], {}),
                  ("bandLow", "f8", (lam,), out["bandLow"],
                   {"long_name": "Lower edges of the bands", "units": "micrometers"}),
                  ("bandUp", "f8", (lam,), out["bandUp"],
                   {"long_name": "Upper edges of the bands", "units": "micrometers"}),
                  (rad, "f8", (rad,), out["bin"], {}), ("rLow", "f8", (rad,), out["rLow"], {}),
                  ("rUp", "f8", (rad,), out["rUp"], {}), ("rEff", "f8", (rad, "rh"), out["rEff"], {}),
                  ("rMass", "f8", (rad, "rh"), out["rMass"], {})]
    ncfile.write(path, dims, variables, version=version)
    return path
