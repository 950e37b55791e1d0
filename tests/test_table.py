"""Table generation (dointegration.fun drop-in) and GSF expansion on the GPU.

Parity: the reference's own tables (tests/golden/table_*.npz, produced by
dointegration.fun) and, for layouts the reference does not produce (radius
grids shared by several bins, the GSF moments), the oracle's restatement.
Tolerances: phase elements 1e-9 relative to P11 at the same angle; qext,
qsca, g 1e-10 relative; the other scalars 1e-9 relative; GSF moments 1e-9
absolute (they are normalised to alpha1(0) = 1; the reference writes them
rounded to 1e-10).
"""
import json

import numpy as np
import pytest

from conftest import load_golden

SCAT = ["p11", "p12", "p22", "p33", "p34", "p44"]
TIGHT = ["qext", "qsca", "g"]
LOOSE = ["qb", "csca", "cext", "ssa", "bsca", "bext", "bbck", "refreal", "refimag", "lidar_ratio"]
NL = ["mass", "volume", "area", "rEff", "rMass", "rhop", "growth_factor", "rLow", "rUp"]


def _check_table(got, ref, prefix=""):
    p11 = np.abs(ref[prefix + "p11"])
    for k in SCAT:
        err = np.max(np.abs(got[k] - ref[prefix + k]) / p11)
        assert err < 1e-9, (k, err)
    pb = ref[prefix + "pback"]
    assert np.max(np.abs(got["pback"] - pb) / np.abs(pb[..., :1])) < 1e-9
    for k, tol in [(k, 1e-10) for k in TIGHT] + [(k, 1e-9) for k in LOOSE]:
        r = ref[prefix + k]
        err = np.max(np.abs(got[k] - r) / np.maximum(np.abs(r), 1e-300))
        assert err < tol, (k, err)
    # qabs = qext - qsca cancels for weakly absorbing particles: 1e-10 of qext
    err = np.max(np.abs(got["qabs"] - ref[prefix + "qabs"]) / np.abs(ref[prefix + "qext"]))
    assert err < 1e-10, ("qabs", err)


@pytest.mark.parametrize("name", ["lognorm", "seasalt", "su", "trivial"])
def test_bin_spec_host_fields_match_reference_cpu(name):
    """The host side of the table driver is bit-exact against the reference's
    written variables: RH growth and the mixed refractive index
    (getHumidRefractiveIndex, dointegration.py:493-537), the wet density
    (dointegration.py:874) and the bin edges.  The particle's imaginary index
    is negated for the Mie convention, as the reference does before its Mie
    calls (dointegration.py:814)."""
    from geosmie_gb300 import table
    g = load_golden("table_%s.npz" % name)
    params = json.loads(str(g["params_json"]))
    nrh = g["out_rh"].size
    for b in range(g["out_bin"].size):
        s = table.bin_spec(params, b, list(g["mlist"]), g["waterm"], table.angmie())
        rep = nrh if s["trivial_nrh"] else 1
        assert s["trivial_nrh"] in (0, nrh)
        np.testing.assert_array_equal(np.repeat(s["gf"], rep), g["out_growth_factor"][b])
        np.testing.assert_array_equal(np.repeat(s["rhop"][0], rep), g["out_rhop"][b])
        mix = np.repeat(s["m"][:, :, 0], rep, axis=1)
        np.testing.assert_array_equal(mix.real, g["out_refreal"][b])
        np.testing.assert_array_equal(-mix.imag, g["out_refimag"][b])
        assert np.all(s["rlow"][0] == g["out_rLow"][b]) and np.all(s["rup"][0] == g["out_rUp"][b])
        assert s["grid"].size > 0 and np.all(np.diff(s["grid"]) > 0)


@pytest.mark.parametrize("name", ["lognorm", "seasalt", "su", "trivial"])
def test_host_grid_and_weights_match_oracle_cpu(name):
    """The size-parameter grid and its widths (initializeXarr,
    dointegration.py:425-463) equal the oracle's bit for bit (the oracle's
    grid equals the reference's own on these definitions).  The weights the
    table driver passes to the GPU explicitly agree with the oracle's: the
    lognormal modes grown by the CARMA 'su' law (dointegration.py:549-583) bit
    for bit, the Gong sea-salt weights (dointegration.py:585-624) to the last
    bits."""
    from geosmie_gb300 import table
    from oracle import integration as oi
    g = load_golden("table_%s.npz" % name)
    params = json.loads(str(g["params_json"]))
    lam = np.asarray(list(g["mlist"])[0][0])
    rh = list(params["rh"])
    for b in range(g["out_bin"].size):
        x, dx = table._x_grid(params, b, lam[0], lam[-1])
        xo, dxo = oi.initialize_xarr(params, b, lam[0], lam[-1])
        np.testing.assert_array_equal(x, xo)
        np.testing.assert_array_equal(dx, dxo)
        if params["psd"]["type"] == "lognorm" and params["rhDep"]["type"] == "su":
            # CARMA growth of every mode radius at its own dry size: host weights
            w = table._lognorm_weights(params, b, rh, x, dx, lam)
            for li, l_ in enumerate(lam):
                for ri, r in enumerate(rh):
                    ref = oi.calculate_psd(params, b, r, rh, xo, dxo, None, l_)[0]
                    for k in range(len(ref)):
                        np.testing.assert_array_equal(w[li, ri, k], ref[k])
        if params["psd"]["type"] != "ss":
            continue
        w = table._ss_weights(params, b, rh, x, lam)
        for li, l_ in enumerate(lam):
            for ri, r in enumerate(rh):
                ref = oi.calculate_psd(params, b, r, rh, xo, dxo, None, l_)[0][0]
                assert np.max(np.abs(w[li, ri] - ref)) <= 4 * np.finfo(float).eps * np.max(ref)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lognorm", "trivial", "seasalt", "su"])
def test_reference_tables_gpu(name):
    from geosmie_gb300 import table
    g = load_golden("table_%s.npz" % name)
    params = json.loads(str(g["params_json"]))
    got = table.run_table(params, list(g["mlist"]), g["waterm"])
    _check_table(got, g, "out_")
    for k in NL:
        r = g["out_" + k]
        assert np.max(np.abs(got[k] - r) / np.maximum(np.abs(r), 1e-300)) < 1e-9, k


def synthetic_spec(nl=3, nrh=4, ns=300, nbin=3, nang=181, seed=20261203):
    """Small radius-grid table: several lognormal bins sharing one grid,
    kappa growth (the layout of the sulfate-like benchmark table)."""
    rng = np.random.default_rng(seed)
    lam = np.logspace(np.log10(0.2e-6), np.log10(4e-6), nl)
    rh = np.linspace(0.0, 0.95, nrh)
    gf = (1 + 0.6 * rh / (1 - rh)) ** (1.0 / 3.0)
    r = np.logspace(np.log10(0.005e-6), np.log10(5e-6), ns)
    ndry, nw = 1.43 + 1e-8j, 1.333 + 1e-9j
    m = np.empty((nl, nrh, 1), np.complex128)
    for i in range(nl):
        m[i, :, 0] = nw + (ndry - nw) / gf ** 3 * (1 + 0.01 * rng.random())
    rg = 0.0695e-6 * np.array([0.5, 1.0, 2.0, 4.0, 0.25, 0.125, 8.0, 1.5])[:nbin]
    return {
        "lambda": lam, "grid": r, "dgrid": np.gradient(r), "grid_kind": 1, "m": m,
        "psd_kind": 0, "psd_param": np.array([[[g_, 0.0, 1e30, 2.03]] for g_ in rg]), "gf_psd": gf,
        "rh0_index": 0, "frac": np.ones((nbin, 1)), "rhop": (gf[None, :] ** -3 * 1700 + (1 - gf ** -3) * 1000) *
        np.ones((nbin, 1)), "rhop0": np.full(nbin, 1700.0), "gf": gf, "rlow": np.full(nbin, 0.005e-6),
        "rup": np.full(nbin, 5e-6), "ang": np.linspace(0.0, 180.0, nang),
    }


def test_check_spec_cpu():
    """TablePlan's input check: every workload and test spec passes; arrays
    whose sizes do not match the dimensions (a one-component psd_param in a
    two-component table, a short rhop) are refused before any device work,
    since the C plan reads them through plain pointers."""
    import json
    from geosmie_gb300 import workloads
    from geosmie_gb300.table import bin_spec, check_spec
    specs = [workloads.homogeneous_single()[0], workloads.sulfate_table(n_lambda=2, n_rh=3, n_radii=50)[0],
             workloads.coated_bc(n_lambda=2, n_radii=40, n_rh=2, n_frac=2)[0],
             workloads.seasalt_large(n_lambda=2, n_radii=40, n_nodes=16, n_moments=8)[0],
             workloads.gsf_smooth()[0], synthetic_spec()] + workloads.dust_bins(n_lambda=2, n_sub=20)[0]
    t = load_golden("table_lognorm.npz")
    params = json.loads(str(t["params_json"]))
    specs.append(bin_spec(params, 0, list(t["mlist"]), t["waterm"], t["out_ang"]))
    for sp in specs:
        check_spec(sp)
    mix = synthetic_spec(nl=2, nrh=2, ns=30, nbin=3)
    mix["m"] = np.concatenate([mix["m"], mix["m"] * 1.02], axis=2)
    mix["frac"] = np.tile([[0.3, 0.7]], (3, 1))
    with pytest.raises(ValueError, match="psd_param"):
        check_spec(mix)
    mix["psd_param"] = np.repeat(mix["psd_param"], 2, axis=1)
    check_spec(mix)
    bad = synthetic_spec()
    bad["rhop"] = bad["rhop"][:, :-1]
    with pytest.raises(ValueError, match="rhop"):
        check_spec(bad)


@pytest.mark.gpu
def test_radius_grid_multibin_with_gsf_gpu():
    from geosmie_gb300.table import TablePlan
    from oracle import integration
    spec = synthetic_spec()
    plan = TablePlan(spec, n_gsf=32)
    plan.run()
    got = plan.results()
    ref = integration.run_spec(spec, n_gsf=32)
    _check_table(got, ref)
    for k in NL:
        assert np.max(np.abs(got["nl_" + k] - ref["nl_" + k]) / np.abs(ref["nl_" + k])) < 1e-9, k
    assert np.max(np.abs(got["pmom"] - ref["pmom"])) < 1e-9
    # idempotence: a second run of the same plan gives the same table
    plan.run()
    again = plan.results()
    assert np.max(np.abs(again["p11"] - got["p11"]) / got["p11"]) < 1e-13


@pytest.mark.gpu
def test_gsf_api_gpu():
    from geosmie_gb300 import gsf
    from oracle import gsf as ogsf
    ang = np.linspace(0.0, 180.0, 361)
    mu = np.cos(np.radians(ang))
    F = np.zeros((3, 6, ang.size))
    for t, g in enumerate([0.3, 0.6, 0.85]):
        p = (1 - g * g) / (1 + g * g - 2 * g * mu) ** 1.5
        F[t, 0] = p
        F[t, 1] = 0.9 * p
        F[t, 2] = 0.8 * p * mu
        F[t, 3] = 0.7 * p * mu
        F[t, 4] = -0.2 * p * (1 - mu * mu)
        F[t, 5] = 0.1 * p * (1 - mu * mu)
    for ng in [64, 129]:
        got, cn = gsf.expand(ang, F, ng)
        ref, rcn = ogsf.expand(ang, F, ng)
        assert np.max(np.abs(got - ref)) < 1e-10, ng
        assert np.max(np.abs(cn - rcn) / rcn) < 1e-12
        # tensor-core GEMMs on fixed-point digits: within 1e-6 of alpha1(0) = 1
        mixed, mcn = gsf.expand(ang, F, ng, precision=1)
        assert np.max(np.abs(mixed - ref)) < 1e-6, ng
        assert np.max(np.abs(mcn - rcn) / rcn) < 1e-6


def _mixed_vs_plain(spec, n_gsf):
    from geosmie_gb300.table import TablePlan
    plain = TablePlan(spec, precision=0, n_gsf=n_gsf)
    plain.run()
    a = plain.results()
    mixed = TablePlan(spec, precision=1, n_gsf=n_gsf)
    mixed.run()
    b = mixed.results()
    return a, b


@pytest.mark.gpu
@pytest.mark.parametrize("n_gsf", [0, 64])
def test_mixed_precision_within_1e6_gpu(n_gsf):
    """Tensor-core (split FP16, FP32 accumulation) table vs the FP64 table:
    phase elements within 1e-6 of P11 at the same angle, bulk scalars within
    1e-6 relative (qabs too: the mixed path sums each order's absorption
    directly; 1e-12 of qext absolute allows for the FP64 table's own
    qext - qsca rounding), GSF moments within 1e-6 of the entry's largest
    alpha1."""
    spec = synthetic_spec(nl=3, nrh=3, ns=400, nbin=5, nang=181)
    a, b = _mixed_vs_plain(spec, n_gsf)
    p11 = np.abs(a["p11"])
    for k in SCAT:
        assert np.max(np.abs(b[k] - a[k]) / p11) < 1e-6, k
    assert np.max(np.abs(b["pback"] - a["pback"]) / np.abs(a["pback"][..., :1])) < 1e-6
    # efficiencies of the mixed path: qb in FP64, qext/qsca/g sums in FP32
    for k in TIGHT + LOOSE:
        assert np.max(np.abs(b[k] - a[k]) / np.abs(a[k])) < 1e-6, k
    assert np.max(np.abs(b["qabs"] - a["qabs"]) / (np.abs(a["qabs"]) + 1e-12 * np.abs(a["qext"]))) < 1e-6
    if n_gsf:
        scale = np.max(np.abs(a["pmom"][..., 0, :]), axis=-1)[..., None, None]
        assert np.max(np.abs(b["pmom"] - a["pmom"]) / scale) < 1e-6


@pytest.mark.gpu
def test_device_wait_timeout_reported_and_context_usable_gpu():
    """Every pipeline wait of the tensor-core contraction is bounded.  With
    0 tries every wait gives up at once: the kernel flags a timeout, lets its
    copies and MMAs finish, frees its tensor memory and returns, and the next
    synchronisation raises DeviceTimeout.  With a few tries a wait may or may
    not run out in mid-pipeline; the run ends either way, with OK or a
    timeout.  The same context and plan then build the table normally, eager
    and as a captured graph, within the mixed path's 1e-6 of the FP64
    table."""
    from geosmie_gb300._native import DeviceTimeout
    spec = synthetic_spec(nl=3, nrh=3, ns=400, nbin=5, nang=181)
    from geosmie_gb300.table import TablePlan
    ref = TablePlan(spec, precision=0, n_gsf=16)
    ref.run()
    a = ref.results()
    ref.close()
    plan = TablePlan(spec, precision=1, n_gsf=16)
    plan.set_wait_limit(0)
    plan.run()
    with pytest.raises(DeviceTimeout):
        plan.sync()
    for tries in (4, 64, 1024):
        plan.set_wait_limit(tries)
        plan.run()
        try:
            plan.sync()
        except DeviceTimeout:
            pass
    plan.set_wait_limit(0)
    plan.run(graph=True)
    with pytest.raises(DeviceTimeout):
        plan.sync()
    plan.set_wait_limit(None)
    for graph in (False, True):
        plan.run(graph=graph)
        b = plan.results()
        p11 = np.abs(a["p11"])
        for k in SCAT:
            assert np.max(np.abs(b[k] - a[k]) / p11) < 1e-6, (graph, k)
        for k in TIGHT:
            assert np.max(np.abs(b[k] - a[k]) / np.abs(a[k])) < 1e-6, (graph, k)
        scale = np.max(np.abs(a["pmom"][..., 0, :]), axis=-1)[..., None, None]
        assert np.max(np.abs(b["pmom"] - a["pmom"]) / scale) < 1e-6
    plan.close()


@pytest.mark.gpu
def test_mixed_reference_layout_and_many_angles_gpu():
    """The reference's own layout (one x grid per bin, 371 angles in two
    column blocks, two-mode bin) through the mixed path, against the
    reference's table."""
    from geosmie_gb300 import table
    g = load_golden("table_lognorm.npz")
    params = json.loads(str(g["params_json"]))
    got = table.run_table(params, list(g["mlist"]), g["waterm"], precision=1)
    p11 = np.abs(g["out_p11"])
    for k in SCAT:
        assert np.max(np.abs(got[k] - g["out_" + k]) / p11) < 1e-6, k
    for k in TIGHT:
        assert np.max(np.abs(got[k] - g["out_" + k]) / np.abs(g["out_" + k])) < 1e-6, k


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_table_as_cuda_graph_gpu(precision):
    """gbmie_table_run_graph: the whole table captured once and replayed.
    Replays equal the eager run bit for bit (the angular kernels' partial sums
    are added in a fixed order); new output buffers force a fresh capture that
    writes to them."""
    import torch
    from geosmie_gb300.table import TablePlan
    spec = synthetic_spec(nl=2, nrh=3, ns=300, nbin=3, nang=181)
    plan = TablePlan(spec, precision=precision, n_gsf=16)
    plan.run()
    a = plan.results()
    for _ in range(2):
        plan.run(graph=True)
    b = plan.results()
    assert plan.h.value and plan.ctx.launches() > 0
    p11 = np.abs(a["p11"])
    for k in a:
        assert np.array_equal(b[k], a[k]), k
    # fresh output buffers: the next replay is re-captured against them
    old = {k: v for k, v in plan.out_t.items()}
    for k, v in old.items():
        plan.out_t[k] = torch.full_like(v, float("nan"))
        setattr(plan.out, k, plan.out_t[k].data_ptr())
    plan.run(graph=True)
    c = plan.results()
    assert np.all(np.isfinite(c["p11"]))
    assert np.array_equal(c["p11"], a["p11"])
    assert not np.isnan(old["phase"].cpu().numpy()).any()   # the old buffers kept their values
    plan.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_table_bits_reproducible_gpu(precision):
    """The angular kernels store their partial Mueller sums in per-block
    slots (plain: a size chunk of a unit; mixed: a tile range and size half)
    that one kernel adds in a fixed order, with no atomic additions, so a
    table's bits do not depend on the order in which blocks finish: eager
    runs, graph replays and a second plan give identical outputs.  Tables: a
    two-component mixture (sums over components) and one wavelength at one
    RH (the contraction splits each unit's tiles over many CTAs)."""
    from geosmie_gb300.table import TablePlan
    mix = synthetic_spec(nl=2, nrh=2, ns=300, nbin=3)
    mix["m"] = np.concatenate([mix["m"], mix["m"] * 1.02], axis=2)
    mix["frac"] = np.tile([[0.3, 0.7]], (3, 1))
    mix["psd_param"] = np.repeat(mix["psd_param"], 2, axis=1)
    one = synthetic_spec(nl=1, nrh=1, ns=900, nbin=2)
    for spec in (mix, one):
        outs = []
        for _ in range(2):
            plan = TablePlan(spec, precision=precision, n_gsf=16)
            plan.run()
            outs.append(plan.results())
            plan.run()
            outs.append(plan.results())
            plan.run(graph=True)
            outs.append(plan.results())
            plan.close()
        a = outs[0]
        assert np.all(np.isfinite(a["p11"]))
        for b in outs[1:]:
            for k in a:
                assert np.array_equal(b[k], a[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("nbin,nang", [(8, 181), (7, 300), (6, 512)])
def test_many_bins_and_angle_blocks_gpu(nbin, nang):
    """Tables of 6-8 bins (the contraction's largest sets of sums, its shared
    memory closest to the limit) and of 300 or 512 angles (three or four
    128-angle blocks: the resident angle chunk is reloaded per (unit,
    block)): the FP64 table against the oracle, the mixed table against the
    FP64 one at 1e-6 (phase elements of P11, scalars relative)."""
    from geosmie_gb300.table import TablePlan
    from oracle import integration
    spec = synthetic_spec(nl=2, nrh=2, ns=300, nbin=nbin, nang=nang)
    res = []
    for prec in (0, 1):
        plan = TablePlan(spec, precision=prec)
        plan.run()
        res.append(plan.results())
        plan.close()
    a, b = res
    _check_table(a, integration.run_spec(spec))
    p11 = np.abs(a["p11"])
    for k in SCAT:
        assert np.max(np.abs(b[k] - a[k]) / p11) < 1e-6, k
    for k in TIGHT:
        assert np.max(np.abs(b[k] - a[k]) / np.abs(a[k])) < 1e-6, k


@pytest.mark.gpu
@pytest.mark.parametrize("nbin,nang", [(5, 129), (2, 256), (3, 160)])
def test_second_angle_block_edges_gpu(nbin, nang):
    """The contraction's second 128-angle block with one angle (129), full
    (256) and half full (160: its active epilogue warps end inside a lane
    quadrant), whole-tile and half-tile items alike: the mixed table against
    the FP64 one at 1e-6 (phase elements of P11, scalars relative), the FP64
    table against the oracle."""
    from geosmie_gb300.table import TablePlan
    from oracle import integration
    spec = synthetic_spec(nl=2, nrh=2, ns=300, nbin=nbin, nang=nang)
    res = []
    for prec in (0, 1):
        plan = TablePlan(spec, precision=prec)
        plan.run()
        res.append(plan.results())
        plan.close()
    a, b = res
    _check_table(a, integration.run_spec(spec))
    p11 = np.abs(a["p11"])
    for k in SCAT:
        assert np.max(np.abs(b[k] - a[k]) / p11) < 1e-6, k
    assert np.max(np.abs(b["pback"] - a["pback"]) / np.abs(a["pback"][..., :1])) < 1e-6
    for k in TIGHT:
        assert np.max(np.abs(b[k] - a[k]) / np.abs(a[k])) < 1e-6, k


@pytest.mark.gpu
def test_ragged_and_refused_tables_gpu():
    """Size counts that leave partial tiles: 2 and 20 sizes (one partial half
    tile), 33 (a full half tile and one size), 65 (one tile and one size), in
    both precisions against the oracle and each other; and tables the plan
    refuses (one size, one angle, nine bins) raise ValueError before any
    device work.  With this few sizes the phase function keeps the deep
    interference minima of single large spheres (x up to 157), where the
    mixed path's error relative to P11 at the same angle is ill-conditioned
    (6e-6 at two sizes): here it is bounded by 1e-6 of the entry's largest
    P11."""
    from geosmie_gb300.table import TablePlan
    from oracle import integration
    for ns in (2, 20, 33, 65):
        spec = synthetic_spec(nl=2, nrh=2, ns=ns, nbin=2)
        res = []
        for prec in (0, 1):
            plan = TablePlan(spec, precision=prec)
            plan.run()
            res.append(plan.results())
            plan.close()
        a, b = res
        _check_table(a, integration.run_spec(spec))
        p11max = np.max(np.abs(a["p11"]), axis=-1, keepdims=True)
        for k in SCAT:
            assert np.max(np.abs(b[k] - a[k]) / p11max) < 1e-6, (ns, k)
        for k in TIGHT:
            assert np.max(np.abs(b[k] - a[k]) / np.abs(a[k])) < 1e-6, (ns, k)
    one_size = synthetic_spec(nl=1, nrh=1, ns=2, nbin=2)
    one_size["grid"], one_size["dgrid"] = one_size["grid"][:1], one_size["dgrid"][:1]
    for spec in (one_size, synthetic_spec(nl=1, nrh=1, nbin=2, nang=1)):
        with pytest.raises(ValueError, match="bad sizes"):
            TablePlan(spec, precision=1)
    spec = synthetic_spec(nl=1, nrh=1, nbin=8)
    for k in ("frac", "rhop"):
        spec[k] = np.concatenate([spec[k], spec[k][:1]], axis=0)
    for k in ("rhop0", "rlow", "rup"):
        spec[k] = np.concatenate([spec[k], spec[k][:1]])
    spec["psd_param"] = np.concatenate([spec["psd_param"], spec["psd_param"][:1]], axis=0)
    with pytest.raises(ValueError, match="n_bin"):
        TablePlan(spec, precision=1)


@pytest.mark.gpu
def test_set_tuning_gpu():
    """gbmie_table_plan_set_tuning: launch parameters given by the caller.
    The plain path's per-bucket layout (each nmax bucket its own launch, its
    chunks in consecutive partial-sum slots) equals the whole-grid layout to
    1e-12 of P11 (other partial sums); two plans with the same parameters
    give identical bits; the mixed path with window 2 or 4 stays within 1e-6
    of the FP64 table; out-of-range parameters are refused."""
    from geosmie_gb300.table import TablePlan
    spec = synthetic_spec(nl=2, nrh=2, ns=700, nbin=3)
    split = {"plain_per_bucket": True, "plain_chunk": [64, 128, 64, 256, 128],
             "plain_threads": [64, 128, 192, 256, 192], "coef_block": 128, "tc_window": 3}
    whole = dict(split, plain_per_bucket=False)
    res = {}
    for name, tun in (("split", split), ("split2", split), ("whole", whole)):
        plan = TablePlan(spec, precision=0)
        plan.set_tuning(tun)
        got = plan.tuning()
        assert got["tuned"] and all(got[k] == tun[k] for k in tun), got
        plan.run()
        res[name] = plan.results()
        plan.close()
    p11 = np.abs(res["whole"]["p11"])
    for k in SCAT:
        assert np.max(np.abs(res["split"][k] - res["whole"][k]) / p11) < 1e-12, k
    for k in res["split"]:
        assert np.array_equal(res["split"][k], res["split2"][k]), k
    for win in (2, 4):
        plan = TablePlan(spec, precision=1)
        plan.set_tuning(dict(whole, tc_window=win))
        plan.run()
        m = plan.results()
        for k in SCAT:
            assert np.max(np.abs(m[k] - res["whole"][k]) / p11) < 1e-6, (win, k)
        with pytest.raises(ValueError, match="out of range"):
            plan.set_tuning(dict(whole, plain_chunk=[100, 128, 64, 256, 128]))
        with pytest.raises(ValueError, match="out of range"):
            plan.set_tuning(dict(whole, tc_window=9))
        plan.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_gpu(precision):
    """gbmie_table_plan_autotune: the tuned table equals the default one
    (FP64: 1e-12 of P11, the order of the atomic sums aside; mixed: both
    within 1e-6 of the FP64 table), the parameters are in range, and a new
    plan of the same shape takes them from the context cache."""
    from geosmie_gb300.table import TablePlan
    spec = synthetic_spec(nl=2, nrh=3, ns=700, nbin=3, nang=181)
    ref = TablePlan(spec, precision=0)
    ref.run()
    a = ref.results()
    plan = TablePlan(spec, precision=precision)
    before = plan.tuning()
    tun = plan.autotune()
    b = plan.results()
    assert tun["tuned"]
    assert all(c in (64, 128, 256, 512) for c in tun["plain_chunk"])
    assert all(t in (64, 128, 192, 256) for t in tun["plain_threads"])   # 192: one pass over 181 angles
    assert tun["coef_block"] in (64, 128, 256) and tun["tc_window"] in (2, 3, 4)
    tol = 1e-12 if precision == 0 else 1e-6
    p11 = np.abs(a["p11"])
    for k in SCAT:
        assert np.max(np.abs(b[k] - a[k]) / p11) < tol, k
    for k in TIGHT:
        assert np.max(np.abs(b[k] - a[k]) / np.abs(a[k])) < (1e-12 if precision == 0 else 1e-6), k
    plan.run(graph=True)   # a graph captured after tuning uses the tuned launches
    c = plan.results()
    assert np.array_equal(c["p11"], b["p11"])
    again = TablePlan(spec, precision=precision)
    assert again.tuning() == tun   # taken from the context cache at creation
    again.run()
    d = again.results()
    assert np.array_equal(d["p11"], b["p11"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_run_tables_pipelined_equals_sequential_gpu(precision):
    """run_tables overlaps plan creation, runs and result copies of a sequence
    of tables (setup and copy streams, stream-ordered frees): every table
    equals the same table planned, run and read back on its own, bit for bit;
    shapes differ between neighbours so that no buffer of one table can stand
    in for the next one's."""
    from geosmie_gb300.table import TablePlan, run_tables
    specs = [synthetic_spec(nl=2, nrh=3, ns=300, seed=1), synthetic_spec(nl=3, nrh=2, ns=257, nbin=2, seed=2),
             synthetic_spec(nl=2, nrh=3, ns=300, seed=3), synthetic_spec(nl=1, nrh=4, ns=400, nbin=4, seed=4)]
    ref = []
    for sp in specs:
        plan = TablePlan(sp, precision=precision, n_gsf=16)
        plan.run()
        ref.append(plan.results())
        plan.close()
    got = list(run_tables(specs, precision=precision, n_gsf=16))
    assert len(got) == len(specs)
    for a, b in zip(ref, got):
        for k in a:
            assert a[k].shape == b[k].shape, k
            assert np.array_equal(b[k], a[k]), k


@pytest.mark.gpu
def test_angle_operand_cache_reuse_and_eviction_gpu():
    """Mixed plans share the context's cached angle-function operand (and GSF
    tables) when the angles, the largest nmax (the entry count) agree, and
    evict unused entries when more grids than the caches hold come along: a table planned again after five
    other angle grids (an eviction) equals its first planning, and plans
    alive at the same time with equal keys give equal tables."""
    from geosmie_gb300.table import TablePlan
    base = synthetic_spec(nl=2, nrh=2, ns=200, nbin=2, nang=181)

    def spec_with(nang):
        sp = dict(base)
        sp["ang"] = np.linspace(0.0, 180.0, nang)
        return sp

    def table(sp):
        plan = TablePlan(sp, precision=1, n_gsf=16)
        plan.run()
        res = plan.results()
        plan.close()
        return res

    first = table(base)
    p1 = TablePlan(base, precision=1, n_gsf=16)
    p2 = TablePlan(base, precision=1, n_gsf=16)   # the same key while p1 is alive: the shared entries
    p1.run()
    r1 = p1.results()
    p2.run()
    r2 = p2.results()
    p1.close()
    p2.close()
    for nang in (91, 121, 150, 211, 371):   # more grids than the cache's entries
        table(spec_with(nang))
    again = table(base)
    for k in SCAT + TIGHT + ["pback", "pmom"]:
        scale = np.maximum(np.abs(first[k]), 1e-300)
        for other in (r1, r2, again):
            assert np.max(np.abs(other[k] - first[k]) / scale) < 1e-12 or \
                np.max(np.abs(other[k] - first[k])) < 1e-14 * np.max(np.abs(first[k])), k


class _FakePlan(object):
    """Stands in for TablePlan in the host-side pipelining test: records the
    order of plan creation, runs, result copies and closes."""
    log = []
    fail_on = None

    def __init__(self, spec, **kw):
        if spec == _FakePlan.fail_on:
            raise RuntimeError("plan %r" % spec)
        self.spec = spec
        self.open = True
        _FakePlan.log.append(("create", spec))

    def run(self):
        _FakePlan.log.append(("run", self.spec))

    def results_async(self, stream):
        plan = self

        class _Pending(object):
            def get(self):
                _FakePlan.log.append(("copy", plan.spec))
                return {"spec": plan.spec}
        return _Pending()

    def close(self):
        if self.open:
            _FakePlan.log.append(("close", self.spec))
        self.open = False


@pytest.fixture
def fake_pipeline(monkeypatch):
    from geosmie_gb300 import table

    class _Ctx(object):
        device = "cpu"
    monkeypatch.setattr(table._native, "context", lambda device=0: _Ctx())
    monkeypatch.setattr(table.torch.cuda, "Stream", lambda device=None: object())
    monkeypatch.setattr(table, "TablePlan", _FakePlan)
    _FakePlan.log = []
    _FakePlan.fail_on = None
    return table


def test_run_tables_order_and_cleanup_cpu(fake_pipeline):
    """run_tables (host logic, CPU): table i + 1 is planned and launched
    before table i's results are copied back; every plan is closed once, also
    when the consumer stops early or a later plan fails."""
    table = fake_pipeline
    got = [r["spec"] for r in table.run_tables(["a", "b", "c"])]
    assert got == ["a", "b", "c"]
    assert _FakePlan.log == [("create", "a"), ("run", "a"), ("create", "b"), ("run", "b"), ("copy", "a"),
                             ("close", "a"), ("create", "c"), ("run", "c"), ("copy", "b"), ("close", "b"),
                             ("copy", "c"), ("close", "c")]
    assert list(table.run_tables([])) == []
    # consumer stops after the first table: the plan in flight is closed
    _FakePlan.log = []
    gen = table.run_tables(["a", "b", "c"])
    assert next(gen)["spec"] == "a"
    gen.close()
    assert [e for e in _FakePlan.log if e[0] == "close"] == [("close", "a"), ("close", "b")]
    assert ("create", "c") not in _FakePlan.log
    # a later plan fails: the error reaches the consumer and the open plan is closed
    _FakePlan.log = []
    _FakePlan.fail_on = "b"
    with pytest.raises(RuntimeError):
        list(table.run_tables(["a", "b", "c"]))
    assert [e for e in _FakePlan.log if e[0] == "close"] == [("close", "a")]
