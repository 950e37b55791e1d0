"""The GSF expansion (rungsf) pinned to the reference's own code.

Two fixtures, both recorded by tests/golden/make_golden.py from the reference:

* gsf_reconstruct.npz -- the reference's reconstruction of the six
  phase-matrix elements from pmom (utils/eval_gsfun.py:154-285: Legendre
  sums for P11/P44, its d_mn Wigner recurrences :43-72 for P12, P22 +- P33
  and P34, with its sign factor Re(i^(n-m))), applied to the oracle's pmom of
  a smooth small-particle table on 64 Gauss nodes.  There the expansion is
  exact, so the reconstruction must give back the table's phase matrix
  divided by alpha1(0) = (1/2) sum_g w_g F11(mu_g).  This checks the
  conventions of alpha2/alpha3, beta1, beta2, the normalisation and the
  p order [P11, P12, P33, P34, P22, P44] independently of the oracle's
  restatement of spher_expan.f.
* rungsf_pygeos.npz -- the pmom that gsf/convertncdf.py:319-401
  (processFileRaw, pygeos mode) writes for the reference's own lognormal
  table, with the oracle standing in for spher_expan.x: element remap
  [0, 4, 2, 5, 1, 3], zero padding to 129 moments, F17.10 rounding.

Tolerances: reconstruction 1e-12 of P11 on the CPU (exact expansion, FP64
rounding) and 1e-9 on the GPU; pmom 1e-9 absolute (the fixture is rounded to
1e-10); the mixed path 1e-6 of the entry's largest alpha1.
"""
import numpy as np
import pytest

from conftest import load_golden

SCAT = ["p11", "p12", "p22", "p33", "p34", "p44"]


def _alpha1_0(ang_deg, p11):
    """(1/2) sum_g w_g F11(mu_g) on the Gauss nodes the angles sit at."""
    z, w = np.polynomial.legendre.leggauss(ang_deg.size)
    mu = np.cos(np.radians(ang_deg))
    assert np.max(np.abs(mu[::-1] - z)) < 1e-14
    return 0.5 * np.sum(p11[..., ::-1] * w, axis=-1)[..., None]


def _check_reconstruction(g, phase, tol):
    c = _alpha1_0(g["ang"], phase["p11"])
    p11 = np.abs(phase["p11"])
    for k in SCAT:
        err = np.max(np.abs(g["recon_" + k] * c - phase[k]) / p11)
        assert err < tol, (k, err)


def test_oracle_expansion_reconstructed_by_reference_cpu():
    """The oracle's pmom of the smooth workload equals the recorded one, and
    the reference's reconstruction of it gives back the oracle's phase
    matrix."""
    from geosmie_gb300 import workloads
    from oracle import integration
    g = load_golden("gsf_reconstruct.npz")
    spec, _ = workloads.gsf_smooth()
    assert np.array_equal(spec["ang"], g["ang"])
    tab = integration.run_spec(spec, n_gsf=spec["ang"].size)
    assert np.max(np.abs(tab["pmom"] - g["pmom"])) < 1e-12
    _check_reconstruction(g, tab, 1e-12)
    # the conventions the reconstruction fixes are not trivially satisfied:
    # swapping alpha2/alpha3 or the sign of beta1 breaks it
    bad = {k: g["recon_" + k] for k in SCAT}
    bad["p22"], bad["p33"] = g["recon_p33"], g["recon_p22"]
    c = _alpha1_0(g["ang"], tab["p11"])
    assert np.max(np.abs(bad["p22"] * c - tab["p22"]) / np.abs(tab["p11"])) > 1e-3


def test_rungsf_glue_cpu():
    """The product's remap and padding (gsf.pygeos_pmom) on the oracle's
    coefficients of the reference's own table equal what the reference's
    processFileRaw wrote."""
    from geosmie_gb300.gsf import ELEMENTS_IN, pygeos_pmom
    from oracle import gsf as ogsf
    r = load_golden("rungsf_pygeos.npz")
    t = load_golden("table_lognorm.npz")
    F = np.stack([t["out_" + k] for k in ELEMENTS_IN], axis=3)
    sh = F.shape
    coef, _ = ogsf.expand(t["out_ang"], F.reshape(-1, 6, sh[-1]), 129)
    pm = pygeos_pmom(coef.reshape(sh[0], sh[1], sh[2], 6, 129))
    assert pm.shape == r["pmom"].shape == (2, 3, 4, 6, 129)
    assert np.max(np.abs(pm - r["pmom"])) <= 5.1e-11   # F17.10 rounding


@pytest.mark.gpu
def test_gsf_reconstruct_gpu():
    """GPU table of the smooth workload: its pmom equals the recorded one and
    the reference's reconstruction gives back the GPU's phase matrix (FP64);
    the mixed path's pmom within 1e-6."""
    from geosmie_gb300 import workloads
    from geosmie_gb300.table import TablePlan
    g = load_golden("gsf_reconstruct.npz")
    spec, _ = workloads.gsf_smooth()
    n = spec["ang"].size
    res = []
    for prec in (0, 1):
        plan = TablePlan(spec, precision=prec, n_gsf=n)
        plan.run()
        res.append(plan.results())
        plan.close()
    a, b = res
    assert np.max(np.abs(a["pmom"] - g["pmom"])) < 1e-9
    _check_reconstruction(g, a, 1e-9)
    scale = np.max(np.abs(g["pmom"][..., 0, :]), axis=-1)[..., None, None]
    assert np.max(np.abs(b["pmom"] - g["pmom"]) / scale) < 1e-6


@pytest.mark.gpu
def test_rungsf_gpu():
    """The reference's lognormal table through the GPU table driver with 129
    GSF moments, and the GPU expansion of the reference's own phase matrix
    (gsf.pmom_from_table), against the pmom the reference's rungsf glue
    wrote."""
    import json
    from geosmie_gb300 import gsf, table
    r = load_golden("rungsf_pygeos.npz")
    t = load_golden("table_lognorm.npz")
    params = json.loads(str(t["params_json"]))
    got = table.run_table(params, list(t["mlist"]), t["waterm"], n_gsf=129)
    assert got["pmom"].shape == r["pmom"].shape
    assert np.max(np.abs(got["pmom"] - r["pmom"])) < 1e-9
    ref_tab = {k: t["out_" + k] for k in SCAT}
    pm = gsf.pmom_from_table(ref_tab, t["out_ang"])
    assert np.max(np.abs(pm - r["pmom"])) < 1e-9
