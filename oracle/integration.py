"""CPU restatement of the runoptics table builder -- oracle only.

TEST INFRASTRUCTURE: imported by tests/, __graft_entry__.smoke() and bench.py
(CPU baseline / reference arm).  Never imported by the product package.

Follows geosmie/dointegration.py and geosmie/particleparams.py of the GEOSmie
source tree: size-parameter grids, humidity growth, volume-mixed refractive
index, PSD weights, the integratePSD weighting (including its aliasing of the
area weight, which makes every key after 'g' qsca-weighted), the phase-function
normalisation and the per-(bin, wavelength, RH) post-processing.  The NetCDF
writer is not restated: :func:`run_table` returns the variables as arrays with
the non-legacy dimension order of createNCDF (dointegration.py:205-422).
"""
import numpy as np

from . import pymie

SCATKEYS = ["p11", "p12", "p22", "p33", "p34", "p44"]          # dointegration.py:17
SCALARKEYS = ["qext", "qsca", "qabs", "qb", "g", "csca", "cext"]  # :19
EXTRAKEYS = ["ssa", "bsca", "bext", "bbck", "refreal", "refimag", "lidar_ratio"]  # :20
ELEKEYS = ["pback"]                                              # :21
NLSCALARKEYS = ["mass", "volume", "area", "rEff", "rMass", "rhop",
                "growth_factor", "rLow", "rUp"]                  # :22
PBACK_ORDER = ["p11", "p12", "p33", "p34", "p22", "p44"]        # :990


def angmie():
    """The 371-angle output grid, dointegration.py:739-742."""
    a1 = np.linspace(0.0, 1.0, 100, endpoint=False)
    a2 = np.linspace(1.0, 10.0, 100, endpoint=False)
    a3 = np.linspace(10.0, 180.0, 171, endpoint=True)
    return np.concatenate([a1, a2, a3])


def get_dr(arr):
    """Centred differences, dointegration.py:93-101."""
    arr = np.asarray(arr, dtype=np.float64)
    d = np.empty_like(arr)
    d[0] = arr[1] - arr[0]
    d[1:-1] = ((arr[1:-1] - arr[:-2]) + (arr[2:] - arr[1:-1])) / 2.0
    d[-1] = arr[-1] - arr[-2]
    return d


def get_x_arr_carma(minx, maxx, nbinperdecade):
    """CARMA volume-ratio grid and its widths, dointegration.py:103-153."""
    rat = maxx / minx
    numdec = np.log10(maxx / minx)
    nbin = numdec * nbinperdecade
    rm_rat = (rat ** 3) ** (1.0 / nbin)
    rmin = minx * ((1.0 + rm_rat) / 2.0) ** (1.0 / 3.0)
    cpi = 4.0 / 3.0 * np.pi
    rvolmin = cpi * rmin ** 3.0
    vrfact = ((3.0 / 2.0 / np.pi / (rm_rat + 1)) ** (1.0 / 3.0)) * (rm_rat ** (1.0 / 3.0) - 1.0)
    ret, dr = [], []
    for i in range(int(nbin)):
        rvol = rvolmin * rm_rat ** i
        ret.append((rvol / cpi) ** (1.0 / 3.0))
        dr.append(vrfact * rvol ** (1.0 / 3.0))
    return np.array(ret), np.array(dr)


def initialize_xarr(params, radind, minlam, maxlam):
    """Per-bin size-parameter grid, dointegration.py:425-463."""
    pparam = params["psd"]["params"]
    psdtype = params["psd"]["type"]
    if psdtype == "lognorm":
        minx = pparam["rmin0"][radind][0] * 2 * np.pi / maxlam
        maxx = pparam["rmax0"][radind][-1] * 2 * np.pi / minlam * 3.0
        return get_x_arr_carma(minx, maxx, pparam["numperdec"][radind])
    if psdtype == "ss":
        minx = pparam["rMinMaj"][radind] * 2 * np.pi / maxlam
        maxx = pparam["rMaxMaj"][radind] * 2 * np.pi / minlam * 10
        return get_x_arr_carma(minx, maxx, pparam["numperdec"][radind])
    if psdtype == "du":
        minx = pparam["rMinMaj"][radind][0] * 2 * np.pi / maxlam
        maxx = pparam["rMaxMaj"][radind][-1] * 2 * np.pi / minlam
        return (np.linspace(np.log10(minx), np.log10(maxx), 1000)) ** 10.0, None
    raise ValueError("unknown psd type %s" % psdtype)


def humidity_growth(rhdep, siz0, rh, allrh):
    """Humidified size, particleparams.py:85-108 ('simple'/'trivial', 'ss',
    'su').  For 'su' the CARMA sulfate law (carma_utils.py:245-314) is taken
    from geosmie_gb300.growth, which tests/test_growth.py pins bit for bit
    to the reference's own wtpct, dens and grow_v75."""
    rhi = list(allrh).index(rh)
    rhtype = rhdep["type"]
    rhp = rhdep["params"]
    if rhtype in ("simple", "trivial"):
        return siz0 * rhp["gf"][rhi]
    if rhtype == "ss":
        siz = siz0 * 100
        if rh == 0.0:
            return siz0
        c1, c2, c3, c4 = rhp["c1"], rhp["c2"], rhp["c3"], rhp["c4"]
        return (c1 * siz ** c2 / (c3 * siz ** c4 - np.log10(rh)) + siz ** 3.0) ** (1.0 / 3.0) / 100.0
    if rhtype == "su":
        if rh == 0.0:
            return siz0
        from geosmie_gb300 import growth
        return siz0 * float(growth.grow_v75(rh, siz0, temp=rhp["temp"]))
    raise NotImplementedError("growth type %s is outside the restated path" % rhtype)


def lognorm_psd(rmode, sigma, xx, lambd, rmax, rmin):
    """dN/dx of a lognormal in size-parameter space, particleparams.py:113-127."""
    xconv = 2 * np.pi / lambd
    xmode, xmax, xmin = rmode * xconv, rmax * xconv, rmin * xconv
    dndx = 1.0 / (xx * (2 * np.pi) ** 0.5 * np.log(sigma)) \
        * np.exp(-(np.log(xx / xmode) ** 2) / (2.0 * np.log(sigma) ** 2))
    dndx[xx >= xmax] = 0.0
    dndx[xx <= xmin] = 0.0
    return dndx


def humid_refractive_index(params, radind, rhi, rh, nref0, nrefwater):
    """Growth factor and volume-mixed index, dointegration.py:493-536 (:505);
    'simple', 'trivial', 'ss' and 'su'."""
    rtype = params["rhDep"]["type"]
    if rtype == "simple" or (rtype == "trivial" and rhi == 0):
        gf = params["rhDep"]["params"]["gf"][rhi]
        rrat = 1.0 / gf
    elif rtype == "ss":
        pparam = params["psd"]["params"]
        try:
            rminmaj = pparam["rMinMaj"][radind]
        except KeyError:
            rminmaj = pparam["rmin0"][radind][0]
        rminuse = humidity_growth(params["rhDep"], rminmaj, rh[rhi], rh)
        rrat = rminmaj / rminuse
        gf = 1.0 / rrat
    elif rtype == "su":   # the first mode's lower radius (dointegration.py:522-528)
        rminmaj = params["psd"]["params"]["rmin0"][radind][0]
        rminuse = humidity_growth(params["rhDep"], rminmaj, rh[rhi], rh)
        rrat = rminmaj / rminuse
        gf = 1.0 / rrat
    else:
        raise NotImplementedError("growth type %s is outside the restated path" % rtype)
    nuse = [nrefwater + (n0 - nrefwater) * rrat ** 3.0 for n0 in nref0]
    return [v.real for v in nuse], [v.imag for v in nuse], gf, rrat


def calculate_psd(params, radind, onerh, rh, xxarr, drarr, rrat, lam):
    """PSD weights per component, dointegration.py:539-664 (lognorm, ss, du)."""
    pparam = params["psd"]["params"]
    psdtype = params["psd"]["type"]
    rparams = params["rhDep"]
    rarr = xxarr / (2 * np.pi / lam)
    psd, ref = [], []
    if psdtype == "lognorm":
        rmodes = [humidity_growth(rparams, r0, onerh, rh) for r0 in pparam["r0"][radind]]
        rmaxs0 = list(pparam["rmax0"][radind])
        rmaxs = [humidity_growth(rparams, v, onerh, rh) for v in rmaxs0]
        rmins = list(pparam["rmin0"][radind])
        rlow, rup = rmins[0], rmaxs0[0]
        sigmas = pparam["sigma"][radind]
        for k in range(len(rmodes)):
            this = lognorm_psd(rmodes[k], sigmas[k], xxarr, lam, rmaxs[k], rmins[k])
            this = this * drarr
            this = this / np.sum(this)
            psd.append(this)
            rr = xxarr * lam / 2.0 / np.pi
            ref.append(np.sum(rr ** 4.0 * this) / np.sum(rr ** 3.0 * this))
    elif psdtype == "ss":
        rminmaj = pparam["rMinMaj"][radind]
        rmaxmaj = pparam["rMaxMaj"][radind]
        rlow, rup = rminmaj, rmaxmaj
        rminuse = humidity_growth(rparams, rminmaj, onerh, rh)
        rmaxuse = humidity_growth(rparams, rmaxmaj, onerh, rh)
        rrat = rminmaj / rminuse
        dr = get_dr(rarr)
        r80rat = 1.65 * rrat
        r80 = rarr * r80rat * 1e6
        afac = 4.7 * (1.0 + 30.0 * r80) ** (-0.017 * r80 ** (-1.44))
        bfac = (0.433 - np.log10(r80)) / 0.433
        dndr80 = 1.373 * r80 ** (-afac) * (1.0 + 0.057 * r80 ** 3.45) * 10.0 ** (1.607 * np.exp(-bfac ** 2.0))
        dndr = dndr80 * r80rat
        dndr[rarr < rminuse] = 0.0
        dndr[rarr > rmaxuse] = 0.0
        dndr = dndr / np.sum(dndr)
        this = dndr * dr
        this = this / np.sum(this)
        psd = [this]
        rr = xxarr * lam / 2.0 / np.pi
        ref = [np.sum(rr ** 4 * this) / np.sum(rr ** 3 * this)]
    elif psdtype == "du":
        for k in range(len(pparam["rMinMaj"][radind])):
            rminmaj = pparam["rMinMaj"][radind][k]
            rmaxmaj = pparam["rMaxMaj"][radind][k]
            rlow, rup = rminmaj, rmaxmaj
            dndr = rarr ** (-4.0)
            dr = get_dr(xxarr)
            dndr[rarr < rminmaj] = 0.0
            dndr[rarr > rmaxmaj] = 0.0
            if np.max(dndr) == 0.0:
                raise ValueError("empty du size bin")
            this = dndr * dr
            this = this / np.sum(this)
            psd.append(this)
            rr = xxarr * lam / 2.0 / np.pi
            ref.append(np.sum(rr ** 4.0 * this) / np.sum(rr ** 3.0 * this))
    else:
        raise ValueError("unknown psd type %s" % psdtype)
    return psd, ref, rlow, rup


def raw_mie(x_arr, costarr, lam, mr, mi, batch=True, m_core=None, core_ratio=None):
    """Per-size Mie results of one (lambda, component), dointegration.py:1211-1254.

    Returns the dict rawMie builds: the six Mueller arrays [nx, nang] and the
    per-size qext, qsca, qabs, qb, g, csca, cext.  With m_core: coated
    spheres of outer size x_arr, shell index mr + i mi, core index m_core and
    core size core_ratio * x (pymiecoated Mie(m=m_core, m2=shell, x, y)).
    """
    x_arr = np.asarray(x_arr, dtype=np.float64)
    rr = x_arr * lam / (2.0 * np.pi)
    if m_core is not None:
        eps_s = complex(mr, mi) ** 2
        eps_c = complex(m_core) ** 2
        ans, bns, nmax = [], [], []
        for xx in x_arr:
            a, b, nm = pymie.mie_coeffs(eps_c, float(core_ratio) * xx, y=xx, eps2=eps_s)
            ans.append(a)
            bns.append(b)
            nmax.append(nm)
        nmax = np.array(nmax)
        pr = pymie.batch_props(ans, bns, nmax, x_arr)
        s1, s2 = pymie.batch_s12(ans, bns, nmax, costarr)
        vals = {"qext": pr[:, 0], "qsca": pr[:, 1], "qabs": pr[:, 2], "qb": pr[:, 3], "asy": pr[:, 4]}
    elif batch:
        eps = complex(mr, mi) ** 2
        ans, bns, nmax = pymie.batch_coeffs_homog(x_arr, eps)
        pr = pymie.batch_props(ans, bns, nmax, x_arr)
        s1, s2 = pymie.batch_s12(ans, bns, nmax, costarr)
        vals = {"qext": pr[:, 0], "qsca": pr[:, 1], "qabs": pr[:, 2], "qb": pr[:, 3],
                "asy": pr[:, 4]}
    else:
        v = pymie.size_range(x_arr, costarr, mr, mi)
        s1 = np.array([[a for a, _ in row] for row in v["s12"]])
        s2 = np.array([[b for _, b in row] for row in v["s12"]])
        vals = {k: np.array(v[k]) for k in ["qext", "qsca", "qabs", "qb", "asy"]}
    ret = {}
    mue = pymie.mueller(s1, s2)
    for k, key in enumerate(SCATKEYS):
        ret[key] = mue[k]
    ret["qext"] = vals["qext"]
    ret["qsca"] = vals["qsca"]
    ret["qabs"] = vals["qabs"]
    ret["qb"] = vals["qb"]
    ret["g"] = vals["asy"]
    ret["csca"] = vals["qsca"] * np.pi * rr ** 2
    ret["cext"] = vals["qext"] * np.pi * rr ** 2
    return ret


def integrate_psd(xxarr, rawret, psd, fracs, lam, reff0, rhop0, rhop):
    """Size-distribution integration, dointegration.py:1064-1209 ('dumix').

    Key order is SCATKEYS + SCALARKEYS (the order of rawMie's dict).  The area
    weight is multiplied in place by qsca when 'g' is reached (:1156-1157);
    because the weight aliases the area array, 'csca' and 'cext' are weighted
    by area*qsca as well.  qb is integrated as a back-scattering phase value,
    p11back * qsca_bar / (4 pi) (:1133-1169).
    """
    rr = xxarr * lam / (2.0 * np.pi)
    keys = list(rawret[0].keys())
    ret = {k: 0.0 for k in ["num", "area", "volume", "mass", "rEff", "rMass", "bsca",
                             "bext", "bbck", "lidar_ratio"]}
    for key in keys:
        ret[key] = np.zeros(rawret[0][key].shape[1]) if key in SCATKEYS else 0.0
    for fi, frac in enumerate(fracs):
        this = {k: np.zeros_like(v) for k, v in ret.items()}
        w_psd = psd[fi]
        num = np.sum(w_psd)
        rarr2 = rr ** 2.0 * w_psd
        rarr3 = rr ** 3.0 * w_psd
        rarr4 = rr ** 4.0 * w_psd
        area = np.pi * np.sum(rarr2) / num
        volume = 4.0 / 3.0 * np.pi * np.sum(rarr3) / num
        weight = np.pi * rr ** 2.0          # aliased: 'g' rescales it in place
        this["num"] = num
        this["area"] = area
        this["mass"] = volume * rhop
        this["volume"] = volume
        this["rEff"] = np.sum(rarr3) / np.sum(rarr2)
        reff_mass = np.sum(rarr4) / np.sum(rarr3)
        this["rMass"] = 4.0 / 3.0 * np.pi * rhop * reff_mass ** 3.0
        rmass0 = 4.0 / 3.0 * np.pi * rhop0 * reff0[fi] ** 3
        for key in keys:
            if key == "qb":
                q = np.asarray(rawret[fi]["qsca"])
                beta = np.sum(q * rarr2) * np.pi
                p11 = np.asarray(rawret[fi]["qb"]) * (np.pi * rr ** 2.0) * (4.0 * np.pi)
                p11back = np.dot(p11, w_psd) / beta
            if key == "g":
                weight = weight * np.asarray(rawret[fi]["qsca"])
            sumarea = np.sum(w_psd * weight)
            if key in SCATKEYS:
                this[key] = np.dot(np.asarray(rawret[fi][key]).T, w_psd)
            elif key == "qb":
                this[key] = p11back * this["qsca"] / (4.0 * np.pi)
            else:
                this[key] = np.dot(np.asarray(rawret[fi][key]), w_psd * weight) / sumarea
        conv = 1.0 / rhop / this["rEff"] * this["rMass"] / rmass0
        this["bsca"] = 3.0 / 4.0 * this["qsca"] * conv
        this["bext"] = 3.0 / 4.0 * this["qext"] * conv
        this["bbck"] = 3.0 / 4.0 * this["qb"] * conv / (4 * np.pi)
        for k in this:
            ret[k] = ret[k] + frac * this[k]
    return ret


def finalize_unit(ret, ang, gf, rhop, mr, mi, rlow, rup):
    """Post-integration values of one (bin, lambda, RH), dointegration.py:950-1001.

    lidar ratio, ssa, the phase normalisation p11n = 2 p11 / trapz(p11 sin t, t)
    over the (non-uniform) angle grid, the rescaling of the other elements,
    pback, and the refractive-index record.  area/volume are divided by the
    dry mass by the caller (they need the RH=0 value).
    """
    out = dict(ret)
    out["lidar_ratio"] = ret["qext"] / ret["qb"] * 4 * np.pi
    out["ssa"] = ret["qsca"] / ret["qext"]
    out["rLow"] = rlow
    out["rUp"] = rup
    theta = np.radians(ang)
    p11n = 2.0 * ret["p11"] / np.trapezoid(ret["p11"] * np.sin(theta), theta)
    for k in ["p12", "p22", "p33", "p34", "p44"]:
        out[k] = ret[k] * p11n / ret["p11"]
    out["p11"] = p11n
    out["pback"] = np.array([out[k][-1] for k in PBACK_ORDER])
    out["growth_factor"] = gf
    out["rhop"] = rhop
    out["refreal"] = mr[0]
    out["refimag"] = -np.abs(mi[0])
    return out


def run_table(params, mlist, waterm, ang=None, batch=True, lambdas=None):
    """The body of dointegration.fun (:672-1036) without the NetCDF file.

    params: the JSON dict (particleparams.getPPJSON); mlist: list of
    [lambda, mr, mi] tables per component; waterm: [lambda, mr, mi] of water.
    Refractive indices are linearly interpolated like scipy interp1d.
    Returns {key: array} with the non-legacy dimensions (bin, lambda, rh[, ang|p])
    and (bin, rh) for the lambda-independent keys (the last lambda is kept,
    as in the reference file).
    """
    if ang is None:
        ang = angmie()
    costarr = np.cos(np.radians(ang))
    lambarr = np.asarray(mlist[0][0]) if lambdas is None else np.asarray(lambdas)
    rh = list(params["rh"])
    psdtype = params["psd"]["type"]
    pparam = params["psd"]["params"]
    nbin = len(pparam["r0"]) if psdtype == "lognorm" else len(pparam["rMinMaj"])
    nl, nr, na = len(lambarr), len(rh), len(ang)
    out = {}
    for k in SCATKEYS:
        out[k] = np.zeros((nbin, nl, nr, na))
    for k in SCALARKEYS + EXTRAKEYS:
        out[k] = np.zeros((nbin, nl, nr))
    out["pback"] = np.zeros((nbin, nl, nr, 6))
    for k in NLSCALARKEYS:
        out[k] = np.zeros((nbin, nr))
    if "maxrh" in params:
        rh = list(np.minimum(np.array(rh), params["maxrh"]))
    minlam, maxlam = lambarr[0], lambarr[-1]
    for b in range(nbin):
        xxarr, drarr = initialize_xarr(params, b, minlam, maxlam)
        for li, lam in enumerate(lambarr):
            nref0 = [complex(np.interp(lam, t[0], t[1]), -np.interp(lam, t[0], t[2])) for t in mlist]
            if params["rhDep"]["type"] == "trivial":
                nw = complex(1, 0)
            else:
                nw = complex(np.interp(lam, waterm[0], waterm[1]), np.interp(lam, waterm[0], waterm[2]))
            _, _, _, rrat0 = humid_refractive_index(params, b, 0, rh, nref0, nw)
            _, reff0, _, _ = calculate_psd(params, b, 0.0, rh, xxarr, drarr, rrat0, lam)
            mass0 = None
            for rhi, onerh in enumerate(rh):
                if params["rhDep"]["type"] == "trivial" and rhi > 0:
                    for k in SCATKEYS + ["pback"]:
                        out[k][b, li, rhi] = out[k][b, li, 0]
                    for k in SCALARKEYS + EXTRAKEYS:
                        out[k][b, li, rhi] = out[k][b, li, 0]
                    for k in NLSCALARKEYS:
                        out[k][b, rhi] = out[k][b, 0]
                    continue
                mr, mi, gf, rrat = humid_refractive_index(params, b, rhi, rh, nref0, nw)
                psd, _, rlow, rup = calculate_psd(params, b, onerh, rh, xxarr, drarr, rrat, lam)
                rhop0 = params["rhop0"][b] if isinstance(params["rhop0"], list) else params["rhop0"]
                rhop = rrat ** 3.0 * rhop0 + (1.0 - rrat ** 3.0) * 1000.0
                allret = [raw_mie(xxarr, costarr, lam, mr[k], mi[k], batch=batch) for k in range(len(mr))]
                if len(allret) == 1:
                    allret = [allret[0] for _ in range(len(psd))]
                ret = integrate_psd(xxarr, allret, psd, pparam["fracs"][b], lam, reff0, rhop0, rhop)
                fin = finalize_unit(ret, ang, gf, rhop, mr, mi, rlow, rup)
                if rhi == 0:
                    mass0 = fin["volume"] * rhop0
                fin["area"] = fin["area"] / mass0
                fin["volume"] = fin["volume"] / mass0
                for k in SCATKEYS:
                    out[k][b, li, rhi] = fin[k]
                out["pback"][b, li, rhi] = fin["pback"]
                for k in SCALARKEYS + EXTRAKEYS:
                    out[k][b, li, rhi] = fin[k]
                for k in NLSCALARKEYS:
                    out[k][b, rhi] = fin[k]
    return out


def psd_volume(xxarr, lam, psd, fracs):
    """The 'volume' that integrate_psd accumulates over the PSD components
    (4/3 pi sum r^3 psd / sum psd, weighted by frac), in its order of
    operations; it needs no Mie results."""
    rr = xxarr * lam / (2.0 * np.pi)
    vol = 0.0
    for fi, frac in enumerate(fracs):
        w_psd = psd[fi]
        vol = vol + frac * (4.0 / 3.0 * np.pi * np.sum(rr ** 3.0 * w_psd) / np.sum(w_psd))
    return vol


def run_spec(spec, n_gsf=0, n_gsf_nodes=0, units=None, batch=True):
    """CPU evaluation of a table spec (the arrays of geosmie_gb300's
    TablePlan / gbmie_table_desc) with the restated reference formulas:
    raw_mie, lognormal / r^-4 / given PSD weights, integrate_psd,
    finalize_unit, the RH=0 mass normalisation, and (n_gsf > 0) the GSF
    expansion of oracle/spher_expan.c on the normalised phase matrix
    (n_gsf_nodes > n_gsf: an expansion on that many nodes, its first n_gsf
    coefficients kept).

    Returns arrays shaped like the GPU results: scatkeys [nbin, nl, nrh,
    nang], scalar keys [nbin, nl, nrh], pback [nbin, nl, nrh, 6], 'nl_<key>'
    [nbin, nl, nrh], pmom [nbin, nl, nrh, 6, n_gsf] in the pygeos p order.
    units: None for every (wavelength, RH) unit, or a list of (wavelength
    index, RH index) pairs to evaluate (the others stay zero).  batch=False
    evaluates homogeneous spheres size by size as pymiecoated's MultipleMie
    does (raw_mie's per-size path) instead of vectorised over sizes.
    """
    from . import gsf as ogsf
    lam = np.asarray(spec["lambda"], np.float64)
    grid = np.asarray(spec["grid"], np.float64)
    dgrid = np.asarray(spec["dgrid"], np.float64)
    m = np.asarray(spec["m"], np.complex128)
    frac = np.asarray(spec["frac"], np.float64)
    ang = np.asarray(spec["ang"], np.float64)
    cost = np.cos(np.radians(ang))
    nl, nrh, ncomp = m.shape
    nbin = frac.shape[0]
    kind = int(spec["psd_kind"])
    radius_grid = int(spec["grid_kind"]) == 1
    rh0 = int(spec.get("rh0_index", 0))
    out = {k: np.zeros((nbin, nl, nrh, ang.size)) for k in SCATKEYS}
    for k in SCALARKEYS + EXTRAKEYS:
        out[k] = np.zeros((nbin, nl, nrh))
    for k in NLSCALARKEYS:
        out["nl_" + k] = np.zeros((nbin, nl, nrh))
    out["pback"] = np.zeros((nbin, nl, nrh, 6))

    def weights(li, ri, b, c, x):
        if kind == 2:
            return np.asarray(spec["weights"])[li, ri, b, c]
        pp = np.asarray(spec["psd_param"])[b, c]
        if kind == 0:
            gfp = np.asarray(spec["gf_psd"])[ri]
            w = lognorm_psd(pp[0] * gfp, pp[3], x, lam[li], pp[2] * gfp, pp[1]) * dgrid
        else:
            r = x * lam[li] / (2 * np.pi)
            w = r ** (-4.0) * dgrid
            w[r < pp[0]] = 0.0
            w[r > pp[1]] = 0.0
        return w / np.sum(w)

    todo = {}
    for li, ri in (units if units is not None else [(li, ri) for li in range(nl) for ri in range(nrh)]):
        todo.setdefault(int(li), []).append(int(ri))
    for li in sorted(todo):
        x = 2 * np.pi * grid / lam[li] if radius_grid else grid
        rr = x * lam[li] / (2 * np.pi)
        reff0 = [[np.sum(rr ** 4 * weights(li, rh0, b, c, x)) / np.sum(rr ** 3 * weights(li, rh0, b, c, x))
                  for c in range(ncomp)] for b in range(nbin)]
        # dry mass from RH index 0 (dointegration.py:992-993): the PSD alone
        mass0 = [psd_volume(x, lam[li], [weights(li, 0, b, c, x) for c in range(ncomp)], frac[b]) *
                 float(np.asarray(spec["rhop0"])[b]) for b in range(nbin)]
        for ri in sorted(set(todo[li])):
            if spec.get("m_core") is not None:
                mcore = np.asarray(spec["m_core"], np.complex128)
                cr = float(np.asarray(spec["core_ratio"])[ri])
                raws = [raw_mie(x, cost, lam[li], m[li, ri, c].real, m[li, ri, c].imag, m_core=mcore[li, ri, c],
                                core_ratio=cr) for c in range(ncomp)]
            else:
                raws = [raw_mie(x, cost, lam[li], m[li, ri, c].real, m[li, ri, c].imag, batch=batch)
                        for c in range(ncomp)]
            for b in range(nbin):
                psd = [weights(li, ri, b, c, x) for c in range(ncomp)]
                rhop = float(np.asarray(spec["rhop"])[b, ri])
                rhop0 = float(np.asarray(spec["rhop0"])[b])
                ret = integrate_psd(x, raws, psd, frac[b], lam[li], reff0[b], rhop0, rhop)
                fin = finalize_unit(ret, ang, float(np.asarray(spec["gf"])[ri]), rhop, [m[li, ri, 0].real],
                                    [m[li, ri, 0].imag], float(np.asarray(spec["rlow"])[b]),
                                    float(np.asarray(spec["rup"])[b]))
                fin["area"] = fin["area"] / mass0[b]
                fin["volume"] = fin["volume"] / mass0[b]
                for k in SCATKEYS:
                    out[k][b, li, ri] = fin[k]
                out["pback"][b, li, ri] = fin["pback"]
                for k in SCALARKEYS + EXTRAKEYS:
                    out[k][b, li, ri] = fin[k]
                for k in NLSCALARKEYS:
                    out["nl_" + k][b, li, ri] = fin[k]
    if n_gsf:
        F = np.stack([out[k] for k in ["p11", "p22", "p33", "p44", "p12", "p34"]], axis=3)
        ng = max(n_gsf, n_gsf_nodes)
        done = np.zeros((nl, nrh), bool)
        for li in todo:
            done[li, todo[li]] = True
        sel = np.broadcast_to(done[None], (nbin, nl, nrh))
        coef, _ = ogsf.expand(ang, F[sel].reshape(-1, 6, ang.size), ng)
        pm = np.zeros((nbin, nl, nrh, 6, n_gsf))
        pm[sel] = coef[..., :n_gsf][:, [0, 4, 2, 5, 1, 3], :]
        out["pmom"] = pm
    return out
