"""Band averaging: the bandaverage.py / runbands.py drop-in.

``fun(data, part, mode, useSolar, noIR)`` mirrors geosmie/bandaverage.py
``fun`` (:126-294) on a table dict (the variables of the optics file, as
``table.run_table`` returns them, non-legacy layout [bin][wavelength][rh])
and returns the band file's variables instead of writing them; the eight
averaged quantities are computed by one GPU call (``gbmie_band_average``)
for all variables, bins, bands and RH values.  ``get_bands`` holds the band
sets of getBands (:73-124).

Kept from the reference: the band edges and centres, the 100-point
wavenumber average of doAverage (:18-50), the noIR settings (:181-193), the
GEOS5 merge of bands 0 and 2 weighted by their widths in wavelength
(:201-221), RRTMG's edges converted to micrometres and reversed (:248-257),
`qname` = part + 3-digit bin number, rLow/rUp of the first RH.  useSolar is
accepted and, as in the reference, has no effect on the averages.
Not kept (reference defects that make its run fail or write wrong
metadata): the GEOS5 merge drops the first band centre once per variable
(the band-centre write then fails) and writes 19 edges for 18 bands -- here
band 0's centre and edges are dropped once; RRTMGP's edges stay Python
lists, so `lBandLow * 1e6` raises -- here they are arrays; `bandUp` is
written with the lower edges -- here the upper edges.
"""
import ctypes

import numpy as np
import torch

from . import _native

VARS = ["qsca", "qext", "bsca", "bext", "g", "bbck", "refreal", "refimag"]


def get_bands(mode):
    """(low edges, up edges, band centres in m, edges-in-wavenumber flag,
    output band count) of a band set (getBands :73-124): GEOS5 and PURDUE
    edges are wavelengths in m, RRTMG and RRTMGP wavenumbers in cm^-1."""
    use_wavenum = True
    nmod = 0
    if mode == "GEOS5":
        use_wavenum = False
        low = np.array([.175, .225, .285, .300, .325, .400, .690, 1.220, 2.270, 29.412, 18.519, 12.5, 10.204,
                        9.091, 8.230, 7.246, 5.263, 3.333, 16.129]) * 1.e-6
        up = np.array([.225, .285, .300, .325, .400, .690, 1.220, 2.270, 3.850, 40., 29.412, 18.519, 12.5,
                       10.204, 9.091, 8.230, 7.246, 5.263, 18.519]) * 1.e-6
        nmod = -1   # bands 0 and 2 are merged
    elif mode == "RRTMG":
        sw_l = [2600., 3250., 4000., 4650., 5150., 6150., 7700., 8050., 12850., 16000., 22650., 29000., 38000.,
                820.]
        sw_r = [3250., 4000., 4650., 5150., 6150., 7700., 8050., 12850., 16000., 22650., 29000., 38000., 50000.,
                2600.]
        lw_l = [10., 350., 500., 630., 700., 820., 980., 1080., 1180., 1390., 1480., 1800., 2080., 2250., 2380.,
                2600.]
        lw_r = [350., 500., 630., 700., 820., 980., 1080., 1180., 1390., 1480., 1800., 2080., 2250., 2380., 2600.,
                3250.]
        low, up = np.array(sw_l + lw_l), np.array(sw_r + lw_r)
    elif mode == "RRTMGP":
        sw_l = [820., 2680., 3250., 4000., 4650., 5150., 6150., 7700., 8050., 12850., 16000., 22650., 29000.,
                38000.]
        sw_r = [2680., 3250., 4000., 4650., 5150., 6150., 7700., 8050., 12850., 16000., 22650., 29000., 38000.,
                50000.]
        lw_l = [10., 250., 500., 630., 700., 820., 980., 1080., 1180., 1390., 1480., 1800., 2080., 2250., 2390.,
                2680.]
        lw_r = [250., 500., 630., 700., 820., 980., 1080., 1180., 1390., 1480., 1800., 2080., 2250., 2390., 2680.,
                3250.]
        low, up = np.array(sw_l + lw_l), np.array(sw_r + lw_r)
    elif mode == "PURDUE":
        use_wavenum = False
        low = np.array([.175, .225, .245, .280, .295, .310, .325, .400, .700, 1.220, 2.270, 3.33, 5.26, 7.25, 8.23,
                        9.09, 10.2, 12.5, 16.13, 18.52, 29.41]) * 1.e-6
        up = np.array([.225, .280, .260, .295, .310, .320, .400, .700, 1.220, 2.270, 10.00, 5.26, 7.25, 8.23, 9.09,
                       10.2, 12.5, 18.52, 18.52, 29.41, 40.0]) * 1.e-6
    else:
        raise ValueError("unknown band set: %s" % mode)
    mean = (low + up) / 2.
    if use_wavenum:
        mean = (mean * 100.) ** (-1)
    return low, up, mean, use_wavenum, len(low) + nmod


def band_average(lam, values, low, up, use_wavenum, device=0):
    """Band means of values [nvar, nbin, nlam, nrh] (wavelength lam [nlam] in
    m) over bands with edges low/up (wavelengths in m, or wavenumbers in
    cm^-1 when use_wavenum): [nvar, nbin, nband, nrh]."""
    ctx = _native.context(device)
    dv = ctx.device
    vals = np.ascontiguousarray(values, np.float64)
    nvar, nbin, nlam, nrh = vals.shape
    low = np.asarray(low, np.float64)
    up = np.asarray(up, np.float64)
    if not use_wavenum:   # doAverage :26-29, per band on numpy scalars as there
        low = np.array([(100. * e) ** (-1) for e in low])
        up = np.array([(100. * e) ** (-1) for e in up])
    wnum = (100. * np.asarray(lam, np.float64)) ** (-1)
    t_w = torch.as_tensor(np.ascontiguousarray(wnum)).to(dv)
    t_v = torch.as_tensor(vals).to(dv)
    t_a = torch.as_tensor(np.ascontiguousarray(low)).to(dv)
    t_b = torch.as_tensor(np.ascontiguousarray(up)).to(dv)
    out = torch.empty((nvar, nbin, low.size, nrh), dtype=torch.float64, device=dv)
    ctx.call("gbmie_band_average", ctypes.c_int32(nvar), ctypes.c_int32(nbin), ctypes.c_int32(nlam),
             ctypes.c_int32(nrh), _native.ptr(t_w), _native.ptr(t_v), ctypes.c_int32(low.size), _native.ptr(t_a),
             _native.ptr(t_b), _native.ptr(out))
    ctx.sync()
    return out.cpu().numpy()


def fun(data, part, mode, useSolar=False, noIR=False, device=0, opfn=None):
    """bandaverage.fun (:126-294): {name: array} of the band file's variables
    (non-legacy layout [bin][band][rh]), written to opfn as a NetCDF classic
    file (lutfile.write_bands) when opfn is given.  data holds 'wavelength'
    (m), 'rh', 'bin', 'rEff', 'rMass', 'rLow', 'rUp' and the eight averaged
    quantities [bin][wavelength][rh]."""
    lam = np.asarray(data["wavelength"], np.float64)
    rh = np.asarray(data["rh"], np.float64)
    reff = np.asarray(data["rEff"], np.float64)
    low, up, mean, use_wavenum, nbands = get_bands(mode)
    nbin = reff.shape[0]
    vals = np.stack([np.asarray(data[k], np.float64) for k in VARS])
    avg = band_average(lam, vals, low, up, use_wavenum, device=device)
    out = {k: avg[i] for i, k in enumerate(VARS)}
    if noIR and mode == "GEOS5":
        ind = np.where(low > 3e-6)[0]
        out["qsca"][:, ind, :] = 0
        out["bsca"][:, ind, :] = 0
        out["qext"][:, ind, :] = 1e-32
        out["bext"][:, ind, :] = 1e-32
    if mode == "GEOS5":   # width-weighted merge of bands 0 and 2 into 2, band 0 dropped
        bw1 = up[0] - low[0]
        bw2 = up[2] - low[2]
        for k in VARS:
            v = out[k]
            v[:, 2, :] = (bw1 * v[:, 0, :] + bw2 * v[:, 2, :]) / (bw1 + bw2)
            out[k] = np.ascontiguousarray(v[:, 1:, :])
        mean = mean[1:]
        low, up = low[1:], up[1:]
    out["wavelength"] = np.asarray(mean, np.float64)
    out["rh"] = rh
    if mode == "RRTMG":   # wavenumbers -> wavelength [m], reversed (:248-257)
        low, up = np.asarray(up)[::-1] ** (-1) * 0.01, np.asarray(low)[::-1] ** (-1) * 0.01
    out["bandLow"] = np.asarray(low, np.float64) * 1e6
    out["bandUp"] = np.asarray(up, np.float64) * 1e6
    out["qname"] = ["%s%03d" % (part, i) for i in range(1, nbin + 1)]
    out["bin"] = np.asarray(data["bin"], np.float64)
    out["rLow"] = np.asarray(data["rLow"], np.float64)[:, 0]
    out["rUp"] = np.asarray(data["rUp"], np.float64)[:, 0]
    out["rEff"] = reff
    out["rMass"] = np.asarray(data["rMass"], np.float64)
    out["_dims"] = {"qsca": ("bin", "wavelength", "rh"), "wavelength": ("wavelength",), "rh": ("rh",),
                    "bandLow": ("wavelength",), "bandUp": ("wavelength",), "qname": ("bin", "nchar"),
                    "bin": ("bin",), "rLow": ("bin",), "rUp": ("bin",), "rEff": ("bin", "rh"),
                    "rMass": ("bin", "rh")}
    if opfn is not None:
        from . import lutfile
        lutfile.write_bands(opfn, out)
    return out
