"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in a container where the GEOSmie sources are present:

    python tests/golden/make_golden.py --ref /root/reference

(or with the reference tree named by the GEOSMIE_REF environment variable).

It imports the reference's own Python code -- pymiecoated (mie_coated.Mie,
MultipleMie, mie_coeffs, mie_props) and geosmie/dointegration.fun -- with
three shims for modules this image lacks: a no-op ``numba`` (the reference
then runs as plain Python), an in-memory ``netCDF4.Dataset`` that records the
variables dointegration.fun writes, and an empty ``matplotlib`` (imported by
carma_utils but not used on this path).  numpy 2 removed ``np.trapz``, which
dointegration.py:979 calls; it is aliased to ``np.trapezoid``.

Outputs (small .npz files, committed):
  mie_single.npz   homogeneous Mie(m=..., x=...) and Mie(eps=, mu=, x=):
                   a_n/b_n, the six efficiencies, S1/S2 at five cosines
  mie_coated.npz   coated Mie(m=, m2=, x=, y=): efficiencies, S1/S2, a_n/b_n
  size_range.npz   MultipleMie(...).calculateS12SizeRange(mr, mi)
  table_*.npz      dointegration.fun on small particle definitions, with the
                   inputs (JSON text, refractive-index tables, water table)
                   needed to rerun them without the reference tree.
  bands.npz        bandaverage.fun (GEOS5, RRTMG, RRTMGP, PURDUE; GEOS5 also
                   with noIR) on a seeded synthetic table of 60 wavelengths,
                   with its inputs, and doAverage on edge cases.
  hydrophobic.npz  hydrophobic.doConversion on the one-bin tables above
                   (table_trivial, table_seasalt), non-legacy and legacy
                   layout, from files laid out by geosmie_gb300.lutfile.
  gsf_reconstruct.npz  utils/eval_gsfun.py's reconstruction of the phase
                   matrix (OPTICS.calcP11/P12/P22_P33/P34, d_mn) from the
                   oracle's pmom of a smooth Gauss-node table; eval_gsfun
                   imports xarray, replaced by a small named-array stand-in.
  rungsf_pygeos.npz  gsf/convertncdf.processFileRaw (pygeos mode) on
                   table_lognorm's reference phase matrix, with a stand-in
                   ./spher_expan.x (the oracle's C restatement writing the
                   Fortran program's text layout).
"""
import argparse
import contextlib
import io
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# --------------------------------------------------------------------------
# shims
# --------------------------------------------------------------------------
def _install_shims():
    numba = types.ModuleType("numba")

    def jit(*a, **k):
        if a and callable(a[0]) and len(a) == 1 and not k:
            return a[0]
        return lambda f: f
    numba.jit = jit
    numba.njit = jit
    sys.modules["numba"] = numba

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    mpl.use = lambda *a, **k: None
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt

    nc = types.ModuleType("netCDF4")

    class Var:
        def __init__(self, shape, dtype="f8"):
            self.data = np.full(shape, "", dtype="<U1") if dtype == "c" else np.zeros(shape)

        def __setitem__(self, k, v):
            try:
                self.data[k] = v
            except ValueError:
                # bandaverage.fun (GEOS5) writes 11 band centres into its
                # 18-band dimension, which netCDF4 rejects too: keep what it wrote
                self.data = np.asarray(v)
                self.mismatch = True

        def __getitem__(self, k):
            return self.data[k]

    class Dataset:
        opened = []

        def __init__(self, path, mode="r"):
            self.path = path
            self.dims = {}
            self.variables = {}
            Dataset.opened.append(self)

        def createDimension(self, name, size):
            self.dims[name] = size

        def createVariable(self, name, dtype, dims, **kw):
            if isinstance(dims, str):
                dims = (dims,)
            v = Var(tuple(self.dims[d] for d in dims), dtype)
            v.dims = dims
            self.variables[name] = v
            return v

        def close(self):
            pass

    nc.Dataset = Dataset
    sys.modules["netCDF4"] = nc
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid
    return Dataset


def _c(lst):
    return np.array(lst, dtype=np.complex128)


def _ragged(arrs):
    off = np.zeros(len(arrs) + 1, dtype=np.int64)
    off[1:] = np.cumsum([len(a) for a in arrs])
    return np.concatenate(arrs) if arrs else np.zeros(0, np.complex128), off


U_LIST = [1.0, 0.5, 0.0, -0.6, -1.0]


def gen_single(ref_mie):
    Mie = ref_mie.Mie
    from pymiecoated import mie_coeffs as mc
    xs = list(np.logspace(-3, np.log10(650.0), 22)) + [2.5, 4.0, 114.2]
    ms = [1.33 + 1e-9j, 1.53 + 0.008j, 1.5 + 0.5j, 1.95 + 0.79j, 1.1 + 0.0j, 3.0 + 4.0j]
    rows_x, rows_eps, rows_mu, eff, s1, s2, ans, bns = [], [], [], [], [], [], [], []
    cases = [(x, m * m, 1.0 + 0j) for m in ms for x in xs]
    cases += [(x, 2.2 + 0.8j, 1.6 + 1.4j) for x in [0.05, 0.5, 4.0, 20.0, 80.0]]
    for x, eps, mu in cases:
        mie = Mie(eps=eps, mu=mu, x=x)
        eff.append([mie.qext(), mie.qsca(), mie.qabs(), mie.qb(), mie.asy(), mie.qratio()])
        ss = [mie.S12(u) for u in U_LIST]
        s1.append([a for a, _ in ss])
        s2.append([b for _, b in ss])
        an, bn, _ = mc.single_mie_coeff(complex(eps), complex(mu), float(x), [], [])
        ans.append(an)
        bns.append(bn)
        rows_x.append(x)
        rows_eps.append(eps)
        rows_mu.append(mu)
    an_all, off = _ragged(ans)
    bn_all, _ = _ragged(bns)
    np.savez_compressed(os.path.join(HERE, "mie_single.npz"), x=np.array(rows_x), eps=_c(rows_eps),
                        mu=_c(rows_mu), eff=np.array(eff), u=np.array(U_LIST), s1=_c(s1), s2=_c(s2),
                        an=an_all, bn=bn_all, offsets=off)
    print("mie_single: %d instances, sum nmax %d" % (len(rows_x), off[-1]))


def gen_coated(ref_mie):
    Mie = ref_mie.Mie
    from pymiecoated import mie_coeffs as mc
    cases = [(1.5, 5.0, 1.5 + 0.5j, 1.2 + 0.2j)]  # test_mie.py:68
    for y in [0.05, 0.3, 1.0, 5.0, 20.0, 62.8]:
        for f in [0.05, 0.2, 0.5]:
            cases.append((y * f ** (1.0 / 3.0), y, 1.95 + 0.79j, 1.53 + 0.01j))
    cases += [(3.0, 8.0, 1.33 + 0.0j, 1.6 + 0.1j), (0.4, 0.9, 2.0 + 1.0j, 1.4 + 1e-6j)]
    xs, ys, m1s, m2s, eff, s1, s2, ans, bns = [], [], [], [], [], [], [], [], []
    for x, y, m1, m2 in cases:
        mie = Mie(m=m1, m2=m2, x=x, y=y)
        eff.append([mie.qext(), mie.qsca(), mie.qabs(), mie.qb(), mie.asy(), mie.qratio()])
        ss = [mie.S12(u) for u in U_LIST]
        s1.append([a for a, _ in ss])
        s2.append([b for _, b in ss])
        an, bn, _ = mc.coated_mie_coeff(m1 * m1, m2 * m2, x, y)
        ans.append(an)
        bns.append(bn)
        xs.append(x)
        ys.append(y)
        m1s.append(m1)
        m2s.append(m2)
    an_all, off = _ragged(ans)
    bn_all, _ = _ragged(bns)
    np.savez_compressed(os.path.join(HERE, "mie_coated.npz"), x=np.array(xs), y=np.array(ys),
                        m1=_c(m1s), m2=_c(m2s), eff=np.array(eff), u=np.array(U_LIST),
                        s1=_c(s1), s2=_c(s2), an=an_all, bn=bn_all, offsets=off)
    print("mie_coated: %d instances" % len(xs))


def gen_size_range(ref_mie):
    lam = 0.55e-6
    r = np.logspace(np.log10(0.01e-6), np.log10(10e-6), 80)
    x = 2 * np.pi * r / lam
    ang = np.linspace(0.0, 180.0, 37)
    cost = np.cos(np.radians(ang))
    mm = ref_mie.MultipleMie(x, None, cost)
    mm.preCalculate()
    v = mm.calculateS12SizeRange(1.53, 0.008)
    s1 = _c([[a for a, _ in row] for row in v["s12"]])
    s2 = _c([[b for _, b in row] for row in v["s12"]])
    np.savez_compressed(os.path.join(HERE, "size_range.npz"), x=x, cost=cost, mr=1.53, mi=0.008,
                        s1=s1, s2=s2, **{k: np.array(v[k]) for k in
                                         ["qext", "qsca", "qabs", "asy", "qb", "qratio"]})
    print("size_range: %d sizes x %d angles" % (len(x), len(cost)))


TABLE_CASES = {
    # lognormal, 'simple' growth, a one-mode bin and a two-mode bin
    "lognorm": {
        "rhop0": 1700.0,
        "rh": [0.0, 0.5, 0.9, 0.99],
        "rhDep": {"type": "simple", "params": {"gf": [1.0, 1.39, 1.77, 2.16]}},
        "psd": {"type": "lognorm", "params": {
            "r0": [[0.0695e-6], [0.05e-6, 0.3e-6]],
            "rmin0": [[0.005e-6], [0.005e-6, 0.005e-6]],
            "rmax0": [[0.3e-6], [0.5e-6, 0.5e-6]],
            "sigma": [[2.03], [1.8, 2.2]],
            "numperdec": [18, 12],
            "fracs": [[1.0], [0.7, 0.3]]}},
        "ri": [[0.40, 1.45, -1e-8], [0.55, 1.43, -1e-8], [1.00, 1.42, -2e-6]],
    },
    # 'trivial' growth (RH > 0 copies RH = 0), absorbing, rhop0 per bin, maxrh
    "trivial": {
        "rhop0": [1800.0],
        "rh": [0.0, 0.8, 0.95],
        "maxrh": 0.9,
        "rhDep": {"type": "trivial", "params": {"gf": [1.0, 1.0, 1.0]}},
        "psd": {"type": "lognorm", "params": {
            "r0": [[0.0118e-6]], "rmin0": [[0.001e-6]], "rmax0": [[0.3e-6]],
            "sigma": [[2.0]], "numperdec": [15], "fracs": [[1.0]]}},
        "ri": [[0.35, 1.75, -0.46], [0.55, 1.75, -0.44], [1.2, 1.77, -0.45]],
    },
    # sulfate: CARMA 'su' growth (Tabazadeh weight percent, Kelvin effect; the
    # growth of each mode radius depends on its dry size), two lognormal bins
    "su": {
        "rhop0": 1923.0,
        "rh": [0.0, 0.5, 0.9, 0.99],
        "rhDep": {"type": "su", "params": {"temp": 220.0}},
        "psd": {"type": "lognorm", "params": {
            "r0": [[0.0695e-6], [0.03e-6, 0.2e-6]],
            "rmin0": [[0.005e-6], [0.004e-6, 0.004e-6]],
            "rmax0": [[0.3e-6], [0.4e-6, 0.4e-6]],
            "sigma": [[2.03], [1.6, 2.0]],
            "numperdec": [15, 12],
            "fracs": [[1.0], [0.6, 0.4]]}},
        "ri": [[0.40, 1.44, -1e-8], [0.55, 1.43, -1e-8], [1.00, 1.42, -2e-6]],
    },
    # sea-salt: Gerber growth, Gong PSD, maxrh capping
    "seasalt": {
        "rhop0": 2200.0,
        "rh": [0.0, 0.5, 0.95, 0.98],
        "maxrh": 0.95,
        "rhDep": {"type": "ss", "params": {"c1": 0.7674, "c2": 3.079, "c3": 2.573e-11, "c4": -1.424}},
        "psd": {"type": "ss", "params": {
            "rMinMaj": [0.1e-6], "rMaxMaj": [0.5e-6], "fracs": [[1.0]], "numperdec": [12]}},
        "ri": [[0.44, 1.50, -1e-8], [0.87, 1.48, -1e-6]],
    },
}


def gen_tables(ref_src, Dataset):
    geosmie_dir = os.path.join(ref_src, "geosmie")
    import dointegration
    import particleparams as pp
    cwd = os.getcwd()
    os.chdir(geosmie_dir)
    try:
        waterm = pp.getWaterM()
    finally:
        os.chdir(cwd)
    only = os.environ.get("GOLDEN_TABLES")
    for name, case in TABLE_CASES.items():
        if only and name not in only.split(","):
            continue
        with tempfile.TemporaryDirectory() as td:
            ri = np.array(case["ri"], dtype=np.float64)
            rifile = os.path.join(td, "ri-%s.wsv" % name)
            np.savetxt(rifile, ri, header="lambda[um] m_real m_imaginary")
            params = {k: v for k, v in case.items() if k != "ri"}
            params["ri"] = {"format": "wsv", "path": [rifile]}
            jfile = os.path.join(td, "%s.json" % name)
            with open(jfile, "w") as fp:
                json.dump(params, fp)
            Dataset.opened.clear()
            os.chdir(geosmie_dir)
            try:
                with contextlib.redirect_stdout(io.StringIO()):
                    dointegration.fun(jfile, "json", td, False)
            finally:
                os.chdir(cwd)
            ds = Dataset.opened[-1]
            out = {("out_" + k): v.data for k, v in ds.variables.items()}
            params_rec = dict(params)
            params_rec["ri"] = {"format": "wsv", "path": ["<inline>"]}
            mlist = pp.getMSep(rifile, None)
            np.savez_compressed(os.path.join(HERE, "table_%s.npz" % name),
                                params_json=json.dumps(params_rec), mlist=np.array([mlist]),
                                waterm=np.array(waterm), **out)
            print("table_%s: p11 %s" % (name, out["out_p11"].shape))


BAND_MODES = [("GEOS5", False), ("GEOS5", True), ("RRTMG", False), ("RRTMGP", False), ("PURDUE", False)]


def bands_input():
    """A seeded synthetic table: 2 bins x 60 wavelengths (0.2-40 um) x 3 RH,
    smooth positive quantities with some structure in wavelength."""
    rng = np.random.default_rng(20261203)
    nbin, nlam, nrh = 2, 60, 3
    lam = np.logspace(np.log10(0.2e-6), np.log10(40e-6), nlam)
    rh = np.array([0.0, 0.5, 0.95])
    ll = np.log(lam)[None, :, None]
    data = {"wavelength": lam, "rh": rh, "bin": np.arange(1, nbin + 1, dtype=np.float64)}
    for k, name in enumerate(["qsca", "qext", "bsca", "bext", "g", "bbck", "refreal", "refimag"]):
        a = rng.uniform(0.5, 2.0, (nbin, 1, nrh))
        b = rng.uniform(-1.0, 1.0, (nbin, 1, nrh))
        c = rng.uniform(0.5, 3.0)
        data[name] = a * (1.5 + np.sin(c * ll + b)) * np.exp(-0.1 * (ll - ll.mean()) ** 2)
    data["rEff"] = rng.uniform(0.1e-6, 2e-6, (nbin, nrh))
    data["rMass"] = rng.uniform(0.1e-6, 2e-6, (nbin, nrh))
    data["rLow"] = np.tile(np.array([[0.01e-6], [0.1e-6]]), (1, nrh))
    data["rUp"] = np.tile(np.array([[0.1e-6], [1.0e-6]]), (1, nrh))
    return data


def gen_bands(ref_src, Dataset):
    sys.path.insert(0, os.path.join(ref_src, "geosmie"))
    import bandaverage
    data = bands_input()

    class In:
        variables = data
    out = {("in_" + k): v for k, v in data.items()}
    for mode, noir in BAND_MODES:
        Dataset.opened.clear()
        tag = "%s%s" % (mode, "_noIR" if noir else "")
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                bandaverage.fun(In, "su", "unused.nc", mode, False, noir)
        except TypeError as e:
            # RRTMGP: the band edges stay Python lists and `lBandLow * 1e6`
            # (bandaverage.py:260) raises after the averages were written
            out["error_%s" % tag] = np.array(str(e))
        ds = Dataset.opened[-1]
        for k, v in ds.variables.items():
            out["out_%s_%s" % (tag, k)] = v.data
    # doAverage edge cases: a band partly and wholly outside the table, a
    # band with reversed edges, wavelength edges
    lam = data["wavelength"]
    var = data["qext"][0, :, 1]
    cases = [(100.0, 300.0, True), (10.0, 40.0, True), (30000.0, 60000.0, True), (60000.0, 52000.0, True),
             (0.175e-6, 0.225e-6, False), (29.412e-6, 40e-6, False), (3.333e-6, 5.263e-6, False)]
    out["edge_cases"] = np.array(cases, dtype=np.float64)
    out["edge_out"] = np.array([bandaverage.doAverage(lam, var, l, r, w, None) for (l, r, w) in cases])
    np.savez_compressed(os.path.join(HERE, "bands.npz"), **out)
    print("bands: %d arrays" % len(out))


def gen_hydrophobic(ref_src):
    """hydrophobic.doConversion on the one-bin reference tables (table_trivial,
    table_seasalt), non-legacy and legacy layout, through an in-memory
    netCDF4 with the parts doConversion uses."""
    sys.path.insert(0, os.path.join(ref_src, "geosmie"))

    class Dim:
        def __init__(self, n):
            self.n = n

        def __len__(self):
            return self.n

    class Var:
        def __init__(self, data, dims, dtype):
            object.__setattr__(self, "_a", {})
            self.data = np.array(data, dtype=dtype)
            self.dimensions = tuple(dims)
            self.dtype = np.dtype(dtype)

        @property
        def shape(self):
            return self.data.shape

        def ncattrs(self):
            return list(self._a)

        def __setattr__(self, k, v):
            if k in ("data", "dimensions", "dtype"):
                object.__setattr__(self, k, v)
            else:
                self._a[k] = v

        def __getattr__(self, k):
            a = object.__getattribute__(self, "_a")
            if k in a:
                return a[k]
            raise AttributeError(k)

        def __getitem__(self, k):
            return self.data[k]

        def __setitem__(self, k, v):
            self.data[k] = v

    files = {}

    class Dataset:
        def __init__(self, path, mode="r"):
            self.path = path
            if mode == "w":
                self.dimensions = {}
                self.variables = {}
                files[path] = self
            else:
                src = files[path]
                self.dimensions = src.dimensions
                self.variables = src.variables

        def ncattrs(self):
            return []

        def createDimension(self, name, size):
            self.dimensions[name] = Dim(size)

        def createVariable(self, name, dtype, dims, **kw):
            v = Var(np.zeros(tuple(len(self.dimensions[d]) for d in dims)), dims, dtype)
            self.variables[name] = v
            return v

        def close(self):
            pass

    nc = types.ModuleType("netCDF4")
    nc.Dataset = Dataset
    saved = sys.modules.get("netCDF4")
    sys.modules["netCDF4"] = nc
    sys.modules.pop("hydrophobic", None)
    import hydrophobic
    from geosmie_gb300 import lutfile
    out = {}
    for name in ("trivial", "seasalt"):
        d = np.load(os.path.join(HERE, "table_%s.npz" % name))
        table = {k[4:]: d[k] for k in d.files if k.startswith("out_")}
        for legacy in (False, True):
            dims, variables = lutfile.optics_file(table, table["rh"], table["wavelength"], table["ang"], legacy)
            src = Dataset("in.nc", "w")
            for dn, size in dims:
                src.createDimension(dn, size)
            for vn, code, vdims, data, attrs in variables:
                v = src.createVariable(vn, "f8" if code == "f8" else "i8", vdims)
                v.data[...] = data
                for ak, av in attrs.items():
                    setattr(v, ak, av)
            hydrophobic.doConversion("in.nc", "out.nc", "", legacy)
            res = files["out.nc"]
            tag = "%s_%s" % (name, "legacy" if legacy else "new")
            for vn, v in res.variables.items():
                out["%s__%s" % (tag, vn)] = v.data
    if saved is not None:
        sys.modules["netCDF4"] = saved
    np.savez_compressed(os.path.join(HERE, "hydrophobic.npz"), **out)
    print("hydrophobic: %d arrays" % len(out))


def gen_growth(ref_src):
    """growth_su.npz: the reference's CARMA sulfate growth (carma_utils.py:
    wtpct :136-188, dens :190-243, grow_v75 :245-314) over 7 RH x 6 dry radii
    x 3 temperatures (126 cases)."""
    sys.path.insert(0, os.path.join(ref_src, "geosmie"))
    import carma_utils as cu
    rh = np.array([0.01, 0.2, 0.5, 0.8, 0.9, 0.95, 0.99])
    rd = np.array([5e-9, 2e-8, 6.95e-8, 2e-7, 1e-6, 5e-6])
    temp = np.array([200.0, 220.0, 273.0])
    ratio = np.empty((rh.size, rd.size, temp.size))
    wt = np.empty((rh.size, temp.size))
    de = np.empty((rh.size, temp.size))
    for i, h in enumerate(rh):
        for k, t in enumerate(temp):
            wt[i, k] = cu.wtpct(float(h), temp=float(t))
            de[i, k] = cu.dens(float(h), temp=float(t))
            for j, r in enumerate(rd):
                ratio[i, j, k] = cu.grow_v75(float(h), float(r), temp=float(t))
    np.savez(os.path.join(HERE, "growth_su.npz"), rh=rh, rd=rd, temp=temp, ratio=ratio, wtpct=wt, dens=de)
    print("growth_su: %d cases" % ratio.size)


# --------------------------------------------------------------------------
# GSF pins: the reference's own reconstruction (utils/eval_gsfun.py) and its
# own rungsf glue (gsf/convertncdf.py processFileRaw, pygeos mode)
# --------------------------------------------------------------------------
class _DA(object):
    """The few xarray.DataArray features eval_gsfun's reconstructions use
    (named dimensions, isel, dict indexing, name-aligned arithmetic,
    ufuncs); eval_gsfun imports xarray, which this image lacks."""

    def __init__(self, data=None, dims=(), coords=None):
        self.dims = tuple(dims)
        if data is None:
            shape = tuple(np.asarray(getattr(coords[d], "data", coords[d])).size for d in self.dims)
            data = np.full(shape, np.nan)
        self.data = np.array(data, dtype=np.float64)

    @property
    def values(self):
        return self.data

    @property
    def sizes(self):
        return dict(zip(self.dims, self.data.shape))

    def isel(self, **kw):
        x, dims = self.data, []
        ax = 0
        for d in self.dims:
            if d in kw and np.ndim(kw[d]) == 0:
                x = np.take(x, int(kw[d]), axis=ax)
            else:
                if d in kw:
                    x = np.take(x, np.asarray(kw[d]), axis=ax)
                dims.append(d)
                ax += 1
        return _DA(x, dims)

    def _on(self, dims):
        x = np.transpose(self.data, [self.dims.index(d) for d in dims if d in self.dims])
        return x.reshape([self.data.shape[self.dims.index(d)] if d in self.dims else 1 for d in dims])

    def _op(self, other, f, swap=False):
        if isinstance(other, _DA):
            dims = list(self.dims) + [d for d in other.dims if d not in self.dims]
            a, b = self._on(dims), other._on(dims)
            return _DA(f(b, a) if swap else f(a, b), dims)
        return _DA(f(other, self.data) if swap else f(self.data, other), self.dims)

    def __add__(self, o):
        return self._op(o, np.add)

    def __radd__(self, o):
        return self._op(o, np.add, True)

    def __sub__(self, o):
        return self._op(o, np.subtract)

    def __rsub__(self, o):
        return self._op(o, np.subtract, True)

    def __mul__(self, o):
        return self._op(o, np.multiply)

    def __rmul__(self, o):
        return self._op(o, np.multiply, True)

    def __iadd__(self, o):
        r = self._op(o, np.add)
        assert set(r.dims) == set(self.dims)
        self.data = np.broadcast_to(r._on(self.dims), self.data.shape).copy()
        return self

    def __getitem__(self, key):
        return self.isel(**key)

    def __setitem__(self, key, val):
        if isinstance(key, slice):
            self.data[key] = val
            return
        idx = tuple(key.get(d, slice(None)) for d in self.dims)
        rest = [d for d in self.dims if d not in key]
        self.data[idx] = val._on(rest) if isinstance(val, _DA) else val

    def __iter__(self):
        for v in self.data:
            yield float(v)

    def __array_ufunc__(self, ufunc, method, *inputs, **kw):
        dims = next(x.dims for x in inputs if isinstance(x, _DA))
        args = [x.data if isinstance(x, _DA) else x for x in inputs]
        return _DA(getattr(ufunc, method)(*args, **kw), dims)


def gen_gsf_reconstruct(src):
    """The reference's own reconstruction of the six phase-matrix elements
    from pmom (eval_gsfun.OPTICS.calcP11/calcP12/calcP22_P33/calcP34, with
    its d_mn Wigner recurrences and scipy eval_legendre), applied to the
    oracle's pmom of a smooth workload whose expansion is exact."""
    xr = types.ModuleType("xarray")
    xr.DataArray = _DA
    sys.modules["xarray"] = xr
    sys.path.insert(0, os.path.join(src, "utils"))
    import eval_gsfun
    root = os.path.dirname(os.path.dirname(HERE))
    sys.path.insert(0, root)
    from geosmie_gb300 import workloads
    from oracle import integration
    spec, _ = workloads.gsf_smooth()
    n = spec["ang"].size
    tab = integration.run_spec(spec, n_gsf=n)
    pm = tab["pmom"]                                  # [bin, wl, rh, 6, m]
    nb, nl, nr = pm.shape[:3]

    class _Optics(object):
        p = _DA([11, 12, 33, 34, 22, 44], ("p",))

        def __getitem__(self, k):
            return {"pmom": _DA(pm, ("bin", "wavelength", "rh", "p", "m"))}[k]
    o = eval_gsfun.OPTICS.__new__(eval_gsfun.OPTICS)
    o.optics = _Optics()
    o.nMom = n
    o.theta = _DA(np.radians(spec["ang"]), ("ang",))
    o.irh, o.ibin, o.iwav = np.arange(nr), np.arange(nb), np.arange(nl)
    o.dims = ("bin", "wavelength", "rh", "ang")
    o.coords = {"rh": np.arange(nr), "wavelength": np.arange(nl), "bin": np.arange(nb), "ang": spec["ang"]}
    o.getPmatrix()
    out = {"recon_" + k: getattr(o, k).data for k in ["p11", "p12", "p22", "p33", "p34", "p44"]}
    np.savez(os.path.join(HERE, "gsf_reconstruct.npz"), ang=spec["ang"], pmom=pm,
             **{"phase_" + k: tab[k] for k in ["p11", "p12", "p22", "p33", "p34", "p44"]}, **out)
    print("gsf_reconstruct: %d entries x %d nodes" % (nb * nl * nr, n))


def gen_rungsf(src):
    """convertncdf.processFileRaw in pygeos mode (the rungsf pass) on the
    reference's own lognormal table (table_lognorm.npz), with a stand-in
    ./spher_expan.x that runs the oracle's C restatement on each text file and
    writes its .expan_coeff in the Fortran program's layout (a header, then
    L and AL1 AL2 AL3 AL4 BET1 BET2 at F17.10, spher_expan.f:93-107).  What
    is recorded is the pmom the reference's glue writes: element remap,
    zero padding to 129 moments, F17.10 quantisation."""
    root = os.path.dirname(os.path.dirname(HERE))
    g = np.load(os.path.join(HERE, "table_lognorm.npz"))
    nc = types.ModuleType("netCDF4")
    prepared = {}

    class Var(object):
        def __init__(self, data, dims):
            self.data = np.array(data, dtype=np.float64)
            self.dims = dims

        def __getitem__(self, k):
            return self.data[k]

        def __setitem__(self, k, v):
            self.data[k] = v

        def __len__(self):
            return self.data.shape[0]

        def __setattr__(self, k, v):
            object.__setattr__(self, k, v)

    class Dataset(object):
        def __init__(self, path, mode="r"):
            d = prepared[os.path.basename(path).replace("nomom.", "")]
            self.dims, self.variables = d

        def createDimension(self, name, size):
            self.dims[name] = size

        def createVariable(self, name, dtype, dims, **kw):
            dims = (dims,) if isinstance(dims, str) else tuple(dims)
            v = Var(np.zeros([self.dims[d] for d in dims]), dims)
            self.variables[name] = v
            return v

        def close(self):
            pass
    nc.Dataset = Dataset
    sys.modules["netCDF4"] = nc
    sys.path.insert(0, os.path.join(src, "gsf"))
    import convertncdf
    ang = g["out_ang"]
    dims = {"rh": g["out_rh"].size, "wavelength": g["out_wavelength"].size, "bin": g["out_bin"].size, "p": 6,
            "ang": ang.size}
    vars_ = {"wavelength": Var(g["out_wavelength"], ("wavelength",)), "rh": Var(g["out_rh"], ("rh",)),
             "bin": Var(g["out_bin"], ("bin",)), "p": Var([11, 12, 33, 34, 22, 44], ("p",)),
             "ang": Var(ang, ("ang",))}
    for k in ["p11", "p12", "p22", "p33", "p34", "p44"]:
        vars_[k] = Var(g["out_" + k], ("bin", "wavelength", "rh", "ang"))
    name = "integ-lognorm-raw.nomom.nc4"
    prepared[name.replace("nomom.", "")] = (dims, vars_)
    old = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            open(name, "w").close()
            exe = os.path.join(tmp, "spher_expan.x")
            with open(exe, "w") as fp:
                fp.write(_SPHER_STANDIN.replace("@PYTHON@", sys.executable).replace("@ROOT@", repr(root)))
            os.chmod(exe, 0o755)
            with contextlib.redirect_stdout(io.StringIO()):
                convertncdf.processFileRaw(name, ".", 0, None, "pygeos", False)
        finally:
            os.chdir(old)
    pmom = vars_["pmom"].data
    np.savez(os.path.join(HERE, "rungsf_pygeos.npz"), pmom=pmom, ang=ang)
    print("rungsf_pygeos: pmom %s" % (pmom.shape,))


_SPHER_STANDIN = r"""#!@PYTHON@
# stand-in for spher_expan.x: the oracle's C restatement on one text file,
# coefficients written in the Fortran program's layout (spher_expan.f:93-107)
import sys
sys.path.insert(0, @ROOT@)
import numpy as np
from oracle import gsf
t = np.loadtxt(sys.argv[1])
coef, cnorm = gsf.expand(t[:, 0], t[:, 1:7].T[None], 129)
with open(sys.argv[1] + ".expan_coeff", "w") as fp:
    fp.write(" %5d%17.10f\n" % (128, cnorm[0]))
    for l in range(129):
        fp.write(" %5d" % l + "".join("%17.10f" % v for v in coef[0, :, l]) + "\n")
"""


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GEOSMIE_REF"),
                    help="root of the GEOSmie reference tree (default: $GEOSMIE_REF)")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref (or set GEOSMIE_REF) to the root of the GEOSmie reference tree")
    src = os.path.join(a.ref, "src")
    Dataset = _install_shims()
    sys.path.insert(0, os.path.join(src, "pymiecoated"))
    sys.path.insert(0, os.path.join(src, "geosmie"))
    from pymiecoated import mie_coated
    sel = a.only.split(",") if a.only else ["single", "coated", "size_range", "tables", "bands", "hydrophobic",
                                             "growth", "gsf_reconstruct", "rungsf"]
    if "single" in sel:
        gen_single(mie_coated)
    if "coated" in sel:
        gen_coated(mie_coated)
    if "size_range" in sel:
        gen_size_range(mie_coated)
    if "tables" in sel:
        gen_tables(src, Dataset)
    if "bands" in sel:
        gen_bands(src, Dataset)
    if "growth" in sel:
        gen_growth(src)
    if "gsf_reconstruct" in sel:
        gen_gsf_reconstruct(src)
    if "rungsf" in sel:
        gen_rungsf(src)
    if "hydrophobic" in sel:
        sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
        gen_hydrophobic(src)


if __name__ == "__main__":
    main()
