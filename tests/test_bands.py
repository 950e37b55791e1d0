"""Band averaging (bandaverage.py): the oracle against the reference's own
run (tests/golden/bands.npz), and the GPU drop-in against the oracle.

Tolerances: the oracle reproduces the reference's eight averaged variables
bit for bit (same numpy operations); the GPU kernel follows the same
arithmetic step by step, so it agrees to 1e-14 relative (bit-exact where the
host's numpy does not contract multiply-adds).
"""
import os

import numpy as np
import pytest

from oracle import bands as obands

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = [("GEOS5", False), ("GEOS5", True), ("RRTMG", False), ("RRTMGP", False), ("PURDUE", False)]


def _golden():
    d = np.load(os.path.join(HERE, "golden", "bands.npz"))
    data = {k[3:]: d[k] for k in d.files if k.startswith("in_")}
    return d, data


def test_oracle_matches_reference_bands_cpu():
    d, data = _golden()
    for mode, noir in CASES:
        tag = mode + ("_noIR" if noir else "")
        o = obands.fun(data, "su", mode, noir)
        for v in obands.VARS:
            assert np.array_equal(o[v], d["out_%s_%s" % (tag, v)]), (tag, v)
        assert np.array_equal(o["rh"], d["out_%s_rh" % tag])
    # metadata where the reference's own run completes
    for tag in ("RRTMG", "PURDUE"):
        o = obands.fun(data, "su", tag)
        for v in ("wavelength", "bandLow", "rEff", "rMass", "rLow", "rUp", "bin"):
            assert np.array_equal(np.asarray(o[v]), d["out_%s_%s" % (tag, v)]), (tag, v)
        q = ["".join(r).strip() for r in d["out_%s_qname" % tag]]
        assert q == o["qname"]
    # the reference defects the drop-in does not copy, as recorded
    assert d["out_GEOS5_wavelength"].size == 11 and d["out_GEOS5_qext"].shape[1] == 18
    assert "error_RRTMGP" in d.files
    lam = data["wavelength"]
    var = data["qext"][0, :, 1]
    e = [obands.do_average(lam, var, l, r, bool(w)) for (l, r, w) in d["edge_cases"]]
    assert np.array_equal(np.array(e), d["edge_out"])


def test_band_sets_cpu():
    from geosmie_gb300 import bands
    for mode, _ in CASES:
        a = bands.get_bands(mode)
        b = obands.get_bands(mode)
        for x, y in zip(a[:3], b[:3]):
            assert np.array_equal(np.asarray(x), np.asarray(y))
        assert a[3:] == b[3:]
    with pytest.raises(ValueError):
        bands.get_bands("NOPE")


@pytest.mark.gpu
def test_band_average_gpu():
    from geosmie_gb300 import bands
    d, data = _golden()
    for mode, noir in CASES:
        g = bands.fun(data, "su", mode, noIR=noir)
        o = obands.fun(data, "su", mode, noir)
        for v in obands.VARS:
            np.testing.assert_allclose(g[v], o[v], rtol=1e-14, atol=0, err_msg="%s %s" % (mode, v))
        for v in ("wavelength", "bandLow", "bandUp", "rEff", "rLow", "rUp"):
            np.testing.assert_array_equal(np.asarray(g[v]), np.asarray(o[v]))
        assert g["qname"] == o["qname"]


@pytest.mark.gpu
def test_band_average_edges_and_a_gpu_table_gpu():
    """Bands partly or wholly outside the table, reversed edges, unsorted
    wavelengths with a repeated one; then a table made by the GPU pipeline."""
    from geosmie_gb300 import bands
    rng = np.random.default_rng(5)
    lam = np.concatenate([np.logspace(-6.5, -4.6, 30), [1e-6]])[rng.permutation(31)]
    vals = rng.uniform(0.1, 3.0, (3, 2, 31, 4))
    low = np.array([100.0, 10.0, 30000.0, 60000.0, 5000.0, 9999.0])
    up = np.array([300.0, 40.0, 60000.0, 52000.0, 5000.0, 10001.0])
    g = bands.band_average(lam, vals, low, up, True)
    for iv in range(3):
        for b in range(2):
            for k in range(low.size):
                for r in range(4):
                    ref = obands.do_average(lam, vals[iv, b, :, r], low[k], up[k], True)
                    assert abs(g[iv, b, k, r] - ref) <= 1e-14 * abs(ref), (iv, b, k, r)
    from geosmie_gb300 import workloads
    from geosmie_gb300.table import TablePlan
    spec, _ = workloads.sulfate_table(n_rh=3, n_lambda=24, n_radii=300)
    plan = TablePlan(spec, precision=0)
    plan.run()
    t = plan.results()
    plan.close()
    vals = np.stack([t[k] for k in ("qsca", "qext", "g")])   # [3][bin][wl][rh]
    lo, up_, _, uw, _ = bands.get_bands("RRTMGP")
    g = bands.band_average(spec["lambda"], vals, lo, up_, uw)
    for iv in range(3):
        for k in range(lo.size):
            ref = obands.do_average(spec["lambda"], vals[iv, 2, :, 1], lo[k], up_[k], uw)
            assert abs(g[iv, 2, k, 1] - ref) <= 1e-14 * abs(ref)
