"""The benchmark workloads (homogeneous single wavelength, dust-like bins,
sea-salt-like large sizes on Gauss nodes, coated black carbon) through the
table pipeline.

Parity: the GPU FP64 table against the oracle's restatement on the same
seeded inputs (reduced sizes where the oracle would take minutes), and the
mixed-precision table against the FP64 table at full size.  Tolerances: FP64
phase elements 1e-9 of P11 at the same angle, qext/qsca/g 1e-10 relative,
the other scalars 1e-9, GSF moments 1e-9 absolute (alpha1(0) = 1); mixed
path 1e-6 (phase elements of P11, scalars relative, moments of max alpha1).
"""
import numpy as np
import pytest

from geosmie_gb300 import workloads
from test_table import LOOSE, SCAT, TIGHT, _check_table


def test_workload_specs_cpu():
    """Shapes and seeded inputs of the workloads (no GPU)."""
    spec, _ = workloads.homogeneous_single()
    assert spec["m"].shape == (1, 1, 1) and spec["grid"].size == 1000 and spec["ang"].size == 181
    specs, _ = workloads.dust_bins()
    assert len(specs) == 5 and all(s["m"].shape == (40, 1, 1) for s in specs)
    again, _ = workloads.dust_bins()
    assert np.array_equal(specs[0]["m"], again[0]["m"])   # seeded
    mr, mi = specs[0]["m"][:, 0, 0].real, specs[0]["m"][:, 0, 0].imag
    assert np.all((mr >= 1.45) & (mr <= 1.60)) and np.all((mi >= 1e-4) & (mi <= 1e-2))
    spec, _, nm, nn = workloads.seasalt_large()
    ang = spec["ang"]
    assert ang.size == nn == 4000 and nm == 1000 and np.all(np.diff(ang) > 0)
    z, _ = np.polynomial.legendre.leggauss(8)
    assert np.allclose(np.cos(np.radians(workloads.gauss_angles(8)))[::-1], z, atol=1e-15)
    counts = workloads.work_counts(spec)
    assert counts["instances"] == 20 * 4000 and counts["units"] == 20


def _mixed_plain(spec, n_gsf=0, n_gsf_nodes=0):
    from geosmie_gb300.table import TablePlan
    out = []
    for prec in (0, 1):
        plan = TablePlan(spec, precision=prec, n_gsf=n_gsf, n_gsf_nodes=n_gsf_nodes)
        plan.run()
        out.append(plan.results())
        plan.close()
    return out


def _check_mixed(a, b, n_gsf, phase_tol=1e-6):
    p11 = np.abs(a["p11"])
    for k in SCAT:
        assert np.max(np.abs(b[k] - a[k]) / p11) < phase_tol, k
    for k in TIGHT + LOOSE:
        assert np.max(np.abs(b[k] - a[k]) / np.abs(a[k])) < 1e-6, k
    # qabs relative to itself (the mixed path sums each order's absorption
    # directly), with 1e-12 of qext for the FP64 table's qext - qsca rounding
    assert np.max(np.abs(b["qabs"] - a["qabs"]) / (np.abs(a["qabs"]) + 1e-12 * np.abs(a["qext"]))) < 1e-6
    if n_gsf:
        scale = np.max(np.abs(a["pmom"][..., 0, :]), axis=-1)[..., None, None]
        assert np.max(np.abs(b["pmom"] - a["pmom"]) / scale) < 1e-6


@pytest.mark.gpu
def test_homogeneous_single_full_gpu():
    """One wavelength, m = 1.53 + 0.008i, 1000 radii 0.01-10 um, 181 angles:
    the whole workload against the oracle, and mixed against FP64."""
    from oracle import integration
    spec, _ = workloads.homogeneous_single()
    a, b = _mixed_plain(spec, n_gsf=64)
    ref = integration.run_spec(spec, n_gsf=64)
    _check_table(a, ref)
    assert np.max(np.abs(a["pmom"] - ref["pmom"])) < 1e-9
    _check_mixed(a, b, 64)


@pytest.mark.gpu
def test_dust_bins_gpu():
    """Random index per wavelength, r^-4 law inside each of 5 bins: reduced
    (3 wavelengths x 5 bins x 150 radii) against the oracle, the full
    40 x 5 x 1000 workload mixed against FP64."""
    from oracle import integration
    small, _ = workloads.dust_bins(n_lambda=3, n_sub=150)
    for spec in small:
        a, _ = _mixed_plain(spec)
        _check_table(a, integration.run_spec(spec))
    full, _ = workloads.dust_bins()
    for spec in full:
        a, b = _mixed_plain(spec, n_gsf=32)
        _check_mixed(a, b, 32)


@pytest.mark.gpu
def test_seasalt_large_gauss_nodes_gpu():
    """x up to ~630 (nmax up to 665) on Gauss-node angles with more nodes
    than moments: reduced (2 wavelengths x 300 radii x 600 nodes, 150
    moments) against the oracle; the full 20 x 4000 x 4000-node, 1000-moment
    workload mixed against FP64, including the forward peak (theta < 1 deg)."""
    from oracle import integration
    spec, _, nm, nn = workloads.seasalt_large(n_lambda=2, n_radii=300, n_nodes=600, n_moments=150)
    a, b = _mixed_plain(spec, n_gsf=nm, n_gsf_nodes=nn)
    ref = integration.run_spec(spec, n_gsf=nm, n_gsf_nodes=nn)
    _check_table(a, ref)
    assert np.max(np.abs(a["pmom"] - ref["pmom"])) < 1e-9
    _check_mixed(a, b, nm)
    spec, _, nm, nn = workloads.seasalt_large()
    a, b = _mixed_plain(spec, n_gsf=nm, n_gsf_nodes=nn)
    _check_mixed(a, b, nm)
    fwd = spec["ang"] < 1.0
    assert fwd.sum() >= 10
    err = np.max(np.abs(b["p11"][..., fwd] - a["p11"][..., fwd]) / a["p11"][..., fwd])
    assert err < 1e-6, err
    assert np.allclose(a["pmom"][..., 0, 0], 1.0, atol=1e-12)


def _check_units(a, ref, units, n_gsf):
    """The FP64 GPU table against the oracle at the given (wavelength, RH)
    units, all bins: the tolerances of _check_table (phase 1e-9 of P11,
    qext/qsca/g 1e-10, other scalars 1e-9, qabs 1e-10 of qext), GSF moments
    1e-9 absolute."""
    li = np.array([u[0] for u in units])
    ri = np.array([u[1] for u in units])
    sub = lambda d: {k: v[:, li, ri] for k, v in d.items() if isinstance(v, np.ndarray) and v.ndim >= 3}
    _check_table(sub(a), sub(ref))
    if n_gsf:
        assert np.max(np.abs(a["pmom"][:, li, ri] - ref["pmom"][:, li, ri])) < 1e-9


@pytest.mark.gpu
def test_sulfate_table_full_gpu():
    """The benchmark's headline table in full -- 36 RH x 60 wavelengths x 5
    bins x 2000 radii x 181 angles + 64 GSF moments: the mixed-precision
    table against the FP64 table on every output (phase elements 1e-6 of
    P11, every scalar 1e-6 relative, qabs 1e-6 of itself, GSF moments 1e-6
    of the entry's largest alpha1), and the FP64 table against the oracle on
    stratified (wavelength, RH) units spanning the wavelength and RH range
    (dointegration.py:786-1031)."""
    from oracle import integration
    spec, _ = workloads.sulfate_table()
    a, b = _mixed_plain(spec, n_gsf=64)
    _check_mixed(a, b, 64)
    pb = np.max(np.abs(b["pback"] - a["pback"]) / np.abs(a["pback"][..., :1]))
    assert pb < 1e-6, pb
    for k in ["nl_" + k for k in ["mass", "volume", "area", "rEff", "rMass", "rhop", "growth_factor"]]:
        assert np.max(np.abs(b[k] - a[k]) / np.abs(a[k])) < 1e-6, k
    units = [(0, 0), (0, 35), (29, 18), (59, 0), (59, 35)]
    ref = integration.run_spec(spec, n_gsf=64, units=units)
    _check_units(a, ref, units, 64)


@pytest.mark.gpu
def test_dn_fp64_variant_gpu():
    """The mixed path with its D_n recurrence in FP64 from the reference's
    start (gbmie_table_plan_set_dn_fp64) against the FP64 table, on reduced
    dust-like bins (Im m 1e-4..1e-2, x up to 314) and a reduced sulfate-like
    table: every output within the mixed path's 1e-6; the default
    double-float form stays within 1e-6 of it too."""
    from geosmie_gb300.table import TablePlan
    small, _ = workloads.dust_bins(n_lambda=4, n_sub=200)
    sul, _ = workloads.sulfate_table(n_rh=4, n_lambda=5, n_radii=300)
    for spec in small[3:] + [sul]:
        a, b = _mixed_plain(spec, n_gsf=16)
        plan = TablePlan(spec, precision=1, n_gsf=16)
        plan.set_dn_fp64(True)
        plan.run()
        c = plan.results()
        plan.set_dn_fp64(False)
        plan.run()
        d = plan.results()
        plan.close()
        _check_mixed(a, c, 16)
        for k in SCAT:
            assert np.max(np.abs(d[k] - b[k]) / np.abs(a["p11"])) < 1e-10, k   # the default form is unchanged
        assert np.max(np.abs(c["p11"] - b["p11"]) / np.abs(a["p11"])) < 1e-6


def test_coated_workload_spec_cpu():
    spec, _ = workloads.coated_bc()
    assert spec["m"].shape == (30, 200, 1) and spec["m_core"].shape == (30, 200, 1)
    assert spec["core_ratio"].shape == (200,) and np.all((spec["core_ratio"] > 0) & (spec["core_ratio"] < 1))
    f = spec["core_ratio"][:10] ** 3
    assert np.allclose(f, np.linspace(0.05, 0.5, 10))


@pytest.mark.gpu
def test_coated_table_gpu():
    """Coated black-carbon table: reduced (3 wavelengths x 3 RH x 2 core
    fractions x 200 outer radii) FP64 against the oracle's per-size coated
    coefficients (the reference's own ratio chain); the full 30 x 200 x 2000
    workload mixed (FP64 coated recurrences, FP32 coefficients into the tensor
    cores) against FP64."""
    from oracle import integration
    spec, _ = workloads.coated_bc(n_lambda=3, n_radii=200, n_rh=3, n_frac=2)
    a, b = _mixed_plain(spec, n_gsf=16)
    ref = integration.run_spec(spec, n_gsf=16)
    _check_table(a, ref)
    assert np.max(np.abs(a["pmom"] - ref["pmom"])) < 1e-9
    _check_mixed(a, b, 16)
    spec, _ = workloads.coated_bc()
    a, b = _mixed_plain(spec)
    _check_mixed(a, b, 0)


@pytest.mark.gpu
def test_large_nmax_table_gpu():
    """Real sea-salt/nitrate tables reach nmax ~7600: one wavelength, 8 radii
    up to x ~ 7540, FP64 against the oracle and mixed against FP64.  The
    mixed path's phase elements are held to 2e-6 of P11 here (measured
    1.2e-6 for p34 at side angles: the FP32 sum over ~160 accumulation
    windows of terms that cancel to a small S); bulk quantities to 1e-6."""
    from oracle import integration
    lam = np.array([0.2e-6])
    r = np.logspace(np.log10(20e-6), np.log10(240e-6), 8)
    m = np.full((1, 1, 1), 1.50 + 1e-6j)
    spec = workloads._lognormal_spec(lam, r, m, [1.0], [100e-6], 1.6, 2200.0, np.linspace(0.0, 180.0, 181))
    counts = workloads.work_counts(spec)
    assert counts["sum_nmax"] > 7 * 1000
    a, b = _mixed_plain(spec)
    ref = integration.run_spec(spec)
    _check_table(a, ref)
    _check_mixed(a, b, 0, phase_tol=2e-6)
