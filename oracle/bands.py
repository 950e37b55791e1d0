"""CPU restatement of GEOSmie's band averaging (test infrastructure only:
imported by tests/ and bench.py's CPU legs, never by the product path).

Follows geosmie/bandaverage.py:
  get_bands   getBands :73-124 (band edges of GEOS5, RRTMG, RRTMGP, PURDUE)
  do_average  doAverage :18-50: 100 points evenly spaced in wavenumber
              between the band's edges (wavelength edges converted with
              1/(100 lambda)), clipped to the table's wavenumber range, the
              variable linearly interpolated there (scipy interp1d, which
              delegates to numpy.interp for 1-D float64 data), their mean
  fun         fun :126-294 without the NetCDF write: the averages of the
              eight variables, noIR (:181-193), the GEOS5 merge of bands 0
              and 2 (:201-221) and the band-centre / edge variables.
Reference defects not copied: the GEOS5 merge drops the first band centre
once per variable (8 times instead of once, so the file write fails) and
writes 19 edges into the 18-band dimension (here the merged set drops band
0's edges); RRTMGP's edges stay Python lists, so `lBandLow * 1e6` (:260)
raises; `bandUp` is written with the lower edges (:269).
Pinned against the reference's own bandaverage run on a synthetic table
(tests/golden/bands.npz, tests/golden/make_golden.py).
"""
import numpy as np

VARS = ["qsca", "qext", "bsca", "bext", "g", "bbck", "refreal", "refimag"]
NSUB = 100


def get_bands(mode):
    """(low edges, up edges, band centres in m, edges-in-wavenumber flag,
    output band count), getBands :73-124."""
    use_wavenum = True
    mod = 0
    if mode == "GEOS5":
        use_wavenum = False
        low = np.array([.175, .225, .285, .300, .325, .400, .690, 1.220, 2.270,
                        29.412, 18.519, 12.5, 10.204, 9.091, 8.230, 7.246, 5.263, 3.333, 16.129]) * 1e-6
        up = np.array([.225, .285, .300, .325, .400, .690, 1.220, 2.270, 3.850,
                       40., 29.412, 18.519, 12.5, 10.204, 9.091, 8.230, 7.246, 5.263, 18.519]) * 1e-6
        mod = -1
    elif mode == "RRTMG":
        low = np.array([2600., 3250., 4000., 4650., 5150., 6150., 7700., 8050., 12850., 16000., 22650., 29000.,
                        38000., 820., 10., 350., 500., 630., 700., 820., 980., 1080., 1180., 1390., 1480., 1800.,
                        2080., 2250., 2380., 2600.])
        up = np.array([3250., 4000., 4650., 5150., 6150., 7700., 8050., 12850., 16000., 22650., 29000., 38000.,
                       50000., 2600., 350., 500., 630., 700., 820., 980., 1080., 1180., 1390., 1480., 1800.,
                       2080., 2250., 2380., 2600., 3250.])
    elif mode == "RRTMGP":
        low = np.array([820., 2680., 3250., 4000., 4650., 5150., 6150., 7700., 8050., 12850., 16000., 22650.,
                        29000., 38000., 10., 250., 500., 630., 700., 820., 980., 1080., 1180., 1390., 1480.,
                        1800., 2080., 2250., 2390., 2680.])
        up = np.array([2680., 3250., 4000., 4650., 5150., 6150., 7700., 8050., 12850., 16000., 22650., 29000.,
                       38000., 50000., 250., 500., 630., 700., 820., 980., 1080., 1180., 1390., 1480., 1800.,
                       2080., 2250., 2390., 2680., 3250.])
    elif mode == "PURDUE":
        use_wavenum = False
        low = np.array([.175, .225, .245, .280, .295, .310, .325, .400, .700, 1.220, 2.270, 3.33, 5.26, 7.25,
                        8.23, 9.09, 10.2, 12.5, 16.13, 18.52, 29.41]) * 1e-6
        up = np.array([.225, .280, .260, .295, .310, .320, .400, .700, 1.220, 2.270, 10.00, 5.26, 7.25, 8.23,
                       9.09, 10.2, 12.5, 18.52, 18.52, 29.41, 40.0]) * 1e-6
    else:
        raise ValueError("unknown band set %s" % mode)
    mean = (low + up) / 2.0
    if use_wavenum:
        mean = (mean * 100.0) ** (-1)
    return low, up, mean, use_wavenum, len(low) + mod


def wavenumber_edges(low, up, use_wavenum):
    """Band edges in cm^-1 (doAverage :26-29)."""
    low = np.asarray(low, np.float64)
    up = np.asarray(up, np.float64)
    if not use_wavenum:
        low = (100.0 * low) ** (-1)
        up = (100.0 * up) ** (-1)
    return low, up


def do_average(lam, var, bandl, bandr, use_wavenum):
    """doAverage :18-50 for one band and one 1-D variable of wavelength."""
    if not use_wavenum:
        bandl = (100.0 * bandl) ** (-1)
        bandr = (100.0 * bandr) ** (-1)
    wnum = (100.0 * np.asarray(lam, np.float64)) ** (-1)
    beg, end = (bandl, bandr) if bandl < bandr else (bandr, bandl)
    x = np.clip(np.linspace(beg, end, NSUB), np.min(wnum), np.max(wnum))
    order = np.argsort(wnum, kind="mergesort")
    y = np.interp(x, wnum[order], np.asarray(var, np.float64)[order])
    return np.sum(y) / len(y)


def fun(data, part, mode, noIR=False):
    """bandaverage.fun :126-294 on the non-legacy layout (variables
    [bin][wavelength][rh]): {name: array} of the output file's variables."""
    lam = np.asarray(data["wavelength"], np.float64)
    rh = np.asarray(data["rh"], np.float64)
    reff = np.asarray(data["rEff"], np.float64)
    low, up, mean, use_wavenum, nbands = get_bands(mode)
    nbin = reff.shape[0]
    out = {}
    for name in VARS:
        v = np.asarray(data[name], np.float64)
        o = np.zeros((nbin, len(low), len(rh)))
        for irh in range(len(rh)):
            for k in range(len(low)):
                for b in range(nbin):
                    o[b, k, irh] = do_average(lam, v[b, :, irh], low[k], up[k], use_wavenum)
        out[name] = o
    if noIR and mode == "GEOS5":
        ind = np.where(low > 3e-6)[0]
        out["qsca"][:, ind, :] = 0.0
        out["bsca"][:, ind, :] = 0.0
        out["qext"][:, ind, :] = 1e-32
        out["bext"][:, ind, :] = 1e-32
    if mode == "GEOS5":
        bw1 = up[0] - low[0]
        bw2 = up[2] - low[2]
        for name in VARS:
            v = out[name]
            v[:, 2, :] = (bw1 * v[:, 0, :] + bw2 * v[:, 2, :]) / (bw1 + bw2)
            out[name] = v[:, 1:, :]
        mean = mean[1:]
        low, up = low[1:], up[1:]
    out["wavelength"] = np.asarray(mean, np.float64)
    out["rh"] = rh
    if mode == "RRTMG":
        lo_w = up[::-1] ** (-1) * 0.01
        up_w = low[::-1] ** (-1) * 0.01
        low, up = lo_w, up_w
    out["bandLow"] = np.asarray(low, np.float64) * 1e6
    out["bandUp"] = np.asarray(up, np.float64) * 1e6
    out["qname"] = ["%s%03d" % (part, i) for i in range(1, nbin + 1)]
    out["bin"] = np.asarray(data["bin"], np.float64)
    out["rLow"] = np.asarray(data["rLow"], np.float64)[:, 0]
    out["rUp"] = np.asarray(data["rUp"], np.float64)[:, 0]
    out["rEff"] = reff
    out["rMass"] = np.asarray(data["rMass"], np.float64)
    return out
