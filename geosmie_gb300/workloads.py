"""Synthetic table workloads (seeded, numpy default_rng(20261203)).

These stand in for GEOS species tables at the sizes the benchmark names; no
dataset is involved.  Each builder returns a TablePlan spec (see
geosmie_gb300.table.TablePlan) plus a short description.

  homogeneous_single   one wavelength, m = 1.53 + 0.008i, 1000 radii
                       0.01-10 um, lognormal r_g = 0.3 um, sigma_g = 2.0,
                       181 angles
  dust_bins            40 wavelengths 0.2-40 um, random m per wavelength,
                       5 bins (edges logspace(-1, 1, 6) um) x 1000 radii,
                       r^-4 PSD inside each bin, no humidity growth; one
                       spec per bin
  sulfate_table        36 RH x 60 wavelengths x 5 bins x 2000 radii x 181
                       angles + 64 GSF moments, kappa growth (0.6), volume
                       mixed index of 1.43 + 1e-8i with water 1.333 + 1e-9i
  coated_bc            core 1.95 + 0.79i in a humidified 1.53 + 0.01i shell,
                       20 RH x 10 core fractions x 30 wavelengths x 2000
                       outer radii x 181 angles
  seasalt_large        m = 1.50 + 1e-8i, 20 wavelengths 0.2-4 um, 4000 radii
                       0.03-20 um (x up to ~630), lognormal r_g = 1 um,
                       sigma_g = 2.0; angles at the 4000 Gauss-Legendre
                       nodes, expanded to 1000 GSF moments on those nodes
"""
import numpy as np

SEED = 20261203
# su.json:5-8 relative humidities
SU_RH = [0.00, 0.05, 0.10, 0.15, 0.20, 0.25, 0.30, 0.35, 0.40, 0.45, 0.50, 0.55, 0.60, 0.65, 0.70, 0.75, 0.80,
         0.81, 0.82, 0.83, 0.84, 0.85, 0.86, 0.87, 0.88, 0.89, 0.90, 0.91, 0.92, 0.93, 0.94, 0.95, 0.96, 0.97,
         0.98, 0.99]


def get_dr(arr):
    """Centred widths of a grid (the reference's getDR, dointegration.py:93-101)."""
    arr = np.asarray(arr, np.float64)
    d = np.empty_like(arr)
    d[0] = arr[1] - arr[0]
    d[1:-1] = ((arr[1:-1] - arr[:-2]) + (arr[2:] - arr[1:-1])) / 2.0
    d[-1] = arr[-1] - arr[-2]
    return d


def _lognormal_spec(lam, r, m, gf, rg_dry, sigma, rhop0, ang):
    nbin = len(rg_dry)
    nrh = len(gf)
    gf = np.asarray(gf, np.float64)
    rrat3 = gf ** -3.0
    return {
        "lambda": np.asarray(lam, np.float64), "grid": r, "dgrid": get_dr(r), "grid_kind": 1, "m": m,
        "psd_kind": 0,
        # no truncation: rmin0 = 0, rmax0 = 1e30 (lognormal over the whole grid)
        "psd_param": np.array([[[g, 0.0, 1e30, sigma]] for g in rg_dry]),
        "gf_psd": gf, "rh0_index": 0, "frac": np.ones((nbin, 1)),
        "rhop": np.tile(rrat3 * rhop0 + (1.0 - rrat3) * 1000.0, (nbin, 1)),
        "rhop0": np.full(nbin, float(rhop0)), "gf": gf, "rlow": np.full(nbin, r[0]), "rup": np.full(nbin, r[-1]),
        "ang": np.asarray(ang, np.float64),
    }


def homogeneous_single(nang=181):
    lam = np.array([0.55e-6])
    r = np.logspace(np.log10(0.01e-6), np.log10(10e-6), 1000)
    m = np.full((1, 1, 1), 1.53 + 0.008j)
    spec = _lognormal_spec(lam, r, m, [1.0], [0.3e-6], 2.0, 1700.0, np.linspace(0.0, 180.0, nang))
    return spec, "homogeneous sphere: 1 wavelength x 1000 radii x %d angles" % nang


def sulfate_table(n_rh=36, n_lambda=60, n_radii=2000, nang=181):
    rh = np.array(SU_RH[:n_rh]) if n_rh <= len(SU_RH) else np.linspace(0.0, 0.99, n_rh)
    gf = (1.0 + 0.6 * rh / (1.0 - rh)) ** (1.0 / 3.0)
    lam = np.logspace(np.log10(0.2e-6), np.log10(40e-6), n_lambda)
    r = np.logspace(np.log10(0.005e-6), np.log10(5e-6), n_radii)
    ndry, nw = 1.43 + 1e-8j, 1.333 + 1e-9j
    m = (nw + (ndry - nw) * gf ** -3.0)[None, :, None] * np.ones((n_lambda, 1, 1))
    rg = 0.0695e-6 * np.array([0.25, 0.5, 1.0, 2.0, 4.0])
    spec = _lognormal_spec(lam, r, m, gf, rg, 2.03, 1700.0, np.linspace(0.0, 180.0, nang))
    desc = ("sulfate-like hygroscopic table: %d RH x %d wavelengths x 5 bins x %d radii x %d angles"
            % (n_rh, n_lambda, n_radii, nang))
    return spec, desc


def dust_bins(n_lambda=40, n_sub=1000, nang=181):
    rng = np.random.default_rng(SEED)
    lam = np.logspace(np.log10(0.2e-6), np.log10(40e-6), n_lambda)
    mr = rng.uniform(1.45, 1.60, n_lambda)
    mi = 10.0 ** rng.uniform(-4.0, -2.0, n_lambda)
    edges = np.logspace(-1, 1, 6) * 1e-6
    specs = []
    for b in range(5):
        r = np.logspace(np.log10(edges[b]), np.log10(edges[b + 1]), n_sub)
        m = (mr + 1j * mi)[:, None, None] * np.ones((1, 1, 1))
        specs.append({
            "lambda": lam, "grid": r, "dgrid": get_dr(r), "grid_kind": 1, "m": m, "psd_kind": 1,
            "psd_param": np.array([[[edges[b], edges[b + 1], 0.0, 0.0]]]), "gf_psd": np.ones(1), "rh0_index": 0,
            "frac": np.ones((1, 1)), "rhop": np.full((1, 1), 2650.0), "rhop0": np.array([2650.0]),
            "gf": np.ones(1), "rlow": np.array([edges[b]]), "rup": np.array([edges[b + 1]]),
            "ang": np.linspace(0.0, 180.0, nang),
        })
    return specs, "dust-like: 40 wavelengths x 5 bins x 1000 radii x %d angles" % nang


def gauss_angles(n):
    """Scattering angles (degrees, ascending) at the n Gauss-Legendre nodes
    of [-1, 1]."""
    z, _ = np.polynomial.legendre.leggauss(n)
    return np.degrees(np.arccos(z))[::-1].copy()


def seasalt_large(n_lambda=20, n_radii=4000, n_nodes=4000, n_moments=1000):
    """Returns (spec, description, n_moments, n_nodes): the angle grid is the
    GSF quadrature itself, so the expansion needs no interpolation."""
    lam = np.logspace(np.log10(0.2e-6), np.log10(4e-6), n_lambda)
    r = np.logspace(np.log10(0.03e-6), np.log10(20e-6), n_radii)
    m = np.full((n_lambda, 1, 1), 1.50 + 1e-8j)
    spec = _lognormal_spec(lam, r, m, [1.0], [1e-6], 2.0, 2200.0, gauss_angles(n_nodes))
    desc = ("sea-salt-like: %d wavelengths x %d radii x %d Gauss-node angles, %d GSF moments"
            % (n_lambda, n_radii, n_nodes, n_moments))
    return spec, desc, n_moments, n_nodes


def gsf_smooth(n_nodes=64):
    """Small particles (x <= 1.8, nmax <= 10) on n_nodes Gauss-node angles:
    2 wavelengths x 2 RH x 1 lognormal bin x 120 radii 0.01-0.15 um,
    m = 1.45 + 0.01i.  S1/S2 are polynomials of degree <= nmax in cos(theta),
    so the phase matrix is a polynomial of degree <= 20 and an expansion in
    n_nodes >= 21 generalized spherical functions on n_nodes Gauss nodes
    reproduces it to rounding: the workload on which the expansion can be
    checked against a reconstruction."""
    lam = np.array([0.55e-6, 1.02e-6])
    r = np.logspace(np.log10(0.01e-6), np.log10(0.15e-6), 120)
    m = np.full((2, 2, 1), 1.45 + 0.01j)
    spec = _lognormal_spec(lam, r, m, [1.0, 1.15], [0.05e-6], 1.8, 1700.0, gauss_angles(n_nodes))
    return spec, "smooth small-particle table on %d Gauss nodes" % n_nodes


def coated_bc(n_lambda=30, n_radii=2000, n_rh=20, n_frac=10, nang=181):
    """Black-carbon core in an organic shell swollen by humidity.

    Core m = 1.95 + 0.79i; shell 1.53 + 0.01i volume-mixed with water
    (1.333 + 1e-9i) by the kappa-growth factor (kappa = 0.6) at 20 RH (every
    other value of the sulfate-table RH list, 18, plus 0.97 and 0.99); core
    volume fractions f = 0.05 .. 0.5 (linear) of the
    whole particle, x_core = y f^(1/3); 30 wavelengths 0.2-3 um; 2000 outer
    radii 0.01-2 um; one lognormal bin (r_g = 0.1 um, sigma_g = 2.0) over the
    grid.  The table's "RH" axis holds the n_rh x n_frac (RH, f) conditions,
    RH-major.
    """
    rh = np.array(sorted(SU_RH[::2] + [0.97, 0.99])[:n_rh])
    gf = (1.0 + 0.6 * rh / (1.0 - rh)) ** (1.0 / 3.0)
    f = np.linspace(0.05, 0.5, n_frac)
    lam = np.logspace(np.log10(0.2e-6), np.log10(3e-6), n_lambda)
    r = np.logspace(np.log10(0.01e-6), np.log10(2e-6), n_radii)
    shell0, nw, core = 1.53 + 0.01j, 1.333 + 1e-9j, 1.95 + 0.79j
    shell = nw + (shell0 - nw) * gf ** -3.0                         # per RH
    gfc = np.repeat(gf, n_frac)                                      # per condition
    m = np.repeat(shell, n_frac)[None, :, None] * np.ones((n_lambda, 1, 1))
    spec = _lognormal_spec(lam, r, m, gfc, [0.1e-6], 2.0, 1500.0, np.linspace(0.0, 180.0, nang))
    spec["gf_psd"] = np.ones(gfc.size)          # the lognormal is over the outer (wet) grid as given
    spec["m_core"] = np.full(m.shape, core)
    spec["core_ratio"] = np.tile(np.cbrt(f), n_rh)
    desc = ("coated black carbon: %d RH x %d core fractions x %d wavelengths x %d outer radii x %d angles"
            % (n_rh, n_frac, n_lambda, n_radii, nang))
    return spec, desc


def nmax_of(x):
    return np.rint(2.0 + x + 4.0 * np.cbrt(x)).astype(np.int64)


def work_counts(spec):
    """Per-workload counts used by the roofline figures: instances, sum of
    nmax and of the D_n start nmx over instances, distinct x rows."""
    lam = np.asarray(spec["lambda"])
    grid = np.asarray(spec["grid"])
    m = np.asarray(spec["m"])
    mcore = spec.get("m_core")
    mabs = np.abs(m) if mcore is None else np.maximum(np.abs(m), np.abs(np.asarray(mcore)).reshape(m.shape))
    nl, nrh, ncomp = m.shape
    x = 2 * np.pi * grid[None, :] / lam[:, None] if int(spec["grid_kind"]) == 1 else np.tile(grid, (1, 1))
    nm = nmax_of(x)                                   # [nle, ns]
    le = np.arange(nl) if int(spec["grid_kind"]) == 1 else np.zeros(nl, np.int64)
    sum_nmax = 0
    sum_nmx = 0
    sum_warm = 0   # D_n steps above nmax of the mixed kernel (warm-up shortened where it converges)
    for li in range(nl):
        xs = x[le[li]]
        nmi = nm[le[li]]
        for ri in range(nrh):
            for c in range(ncomp):
                z = mabs[li, ri, c] * xs   # coated: max(|m_core|, |m_shell|) y (mie_coated.py:131,166)
                nmx = np.rint(np.maximum(nmi, z) + 16.0)
                sum_nmax += int(nmi.sum())
                sum_nmx += int(nmx.sum())
                warm = nmx - 1 - nmi
                short = z < nmi + 1
                q = 2.0 * np.log((2.0 * (nmi + 1) + 1.0) / np.where(short, z, 1.0))
                need = np.ceil(23.0 / np.where(short, q, 1.0)) + 2
                sum_warm += int(np.where(short, np.minimum(warm, need), warm).sum())
    # tensor-core tiles: 64 sizes, orders in chunks of 16 up to the tile's
    # largest nmax, per unit
    sum_kc16 = 0
    sum_kc16_half = 0   # the same per half tile of 32 sizes (MMA N = 64; a whole tile runs both halves)
    tsize = np.minimum(64, grid.size - np.arange(0, grid.size, 64))
    halves = np.where(tsize > 32, 2, 1)
    for li in range(nl):
        nmi = nm[le[li]]
        last = nmi[np.minimum(np.arange(63, grid.size + 63, 64), grid.size - 1)]
        sum_kc16 += int(np.sum((last + 15) // 16)) * nrh * ncomp
        sum_kc16_half += int(np.sum((last + 15) // 16 * halves)) * nrh * ncomp
    return {"instances": int(nl * nrh * ncomp * grid.size), "units": int(nl * nrh * ncomp),
            "sum_nmax": sum_nmax, "sum_nmx": sum_nmx, "sum_warm": sum_warm,
            "sum_kc16": sum_kc16, "sum_kc16_half": sum_kc16_half,
            "rows": int(x.shape[0] * grid.size), "nbin": int(np.asarray(spec["frac"]).shape[0]),
            "nang": int(np.asarray(spec["ang"]).size), "coated": mcore is not None}
